"""Launch-shape autotuner of the draw pipeline.

The search itself is native (dg_autotune in libdrawgpu.so: coordinate descent
over the dg_tuning knobs, each candidate timed with CUDA events on the
context stream). This module runs it on a workload and keeps the result in a
JSON file keyed by the GPU and the workload's shape, so a later process can
apply a tuning without searching again.

    from draw_gb300 import autotune
    best = autotune.tune(ctx, scenes, canvases, cache="tuning.json", key="batch256")
"""
from __future__ import annotations

import json
import os

from . import renderer


def _device_name(device: int = 0) -> str:
    try:
        import torch

        return torch.cuda.get_device_name(device)
    except Exception:
        return "cuda"


def workload_key(scenes: list, canvases: list, label: str = "") -> str:
    px = sum(c.width * c.height for c in canvases)
    return f"{label}|frames={len(scenes)}|pixels={px}"


def load(cache: str) -> dict:
    try:
        with open(cache) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def apply(ctx: renderer.Context, cache: str, key: str) -> dict | None:
    """Sets a cached tuning on ctx; returns it, or None when the cache has no entry."""
    entry = load(cache).get(f"{_device_name()}|{key}")
    if not entry:
        return None
    ctx.set_tuning(**entry["tuning"])
    return entry["tuning"]


def tune(ctx: renderer.Context, scenes: list, canvases: list, reps: int = 3, cache: str | None = None,
         key: str | None = None) -> dict:
    """Runs the native search on these frames, sets the result on ctx and (with
    `cache`) stores it under the GPU name and `key`."""
    best, ms = ctx.autotune(scenes, canvases, reps=reps)
    if cache:
        k = f"{_device_name()}|{key or workload_key(scenes, canvases)}"
        data = load(cache)
        data[k] = {"tuning": best, "ms_per_render": ms}
        tmp = f"{cache}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, cache)
    return {"tuning": best, "ms_per_render": ms}
