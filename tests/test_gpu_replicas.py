"""The replica path of bench.py (one render context per rank, gloo only for the
barriers and the maximum over ranks, no collective on the data path), run as
two torchrun ranks. On a box with fewer GPUs than ranks the replicas share a
device, which is allowed because they never wait on one another. Rank 0 prints
one JSON line for the whole job (two replicas, frames/s summed over the ranks,
the end-to-end leg); the other rank prints nothing."""
import json
import os
import random
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_two_replica_ranks():
    port = str(29400 + random.randrange(500))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", port, "bench.py", "--gpus", "2", "--steps", "3", "--warmup", "3", "--no-cpu",
           "--no-batch", "--no-serve", "--no-stress", "--no-torus", "--kernel-steps", "3"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["n_gpus"] == 2 and d["scaling"] == "weak" and d["value"] > 0
    assert d["gpu_launches"] > 0 and d["e2e"]["value"] > 0
