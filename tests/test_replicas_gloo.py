"""Multi-GPU runs are replicas only (frames are independent): each rank renders
its own frames, and bench.py joins the ranks only for barriers and the
max-over-ranks time. These tests run that host logic as two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    # each rank timed its own K frames; the job's time is the slowest rank's
    t = bench.allmax(w, 0.5 + 0.25 * r)
    value = w * 10 / t
    # the reference arm runs on rank 0 only; other ranks exit 0 without work
    ref_rc = bench.run_reference(None, w, r) if r != 0 else None
    q.put((r, w, t, value, ref_rc))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_over_ranks():
    torch = pytest.importorskip("torch")
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1]
    for r, w, t, value, ref_rc in res:
        assert w == 2 and t == pytest.approx(0.75) and value == pytest.approx(2 * 10 / 0.75)
    assert res[1][4] == 0
