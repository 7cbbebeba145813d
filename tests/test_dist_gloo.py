"""Multi-rank benchmark protocol on CPU (gloo, world size 2): each rank owns its
own replica / ensemble members (no data-path collective); the ranks meet only in
the timing protocol -- a barrier around the timed region and the maximum elapsed
time over ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from nemo_gpu import dist as ndist  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    r, w = ndist.init("gloo")
    ndist.barrier()
    elapsed = 10.0 * (rank + 1)                  # rank-dependent "timed region"
    mx = ndist.max_over_ranks(elapsed)
    total = ndist.sum_over_ranks(1.0)
    lo, hi = ndist.member_range(64, r, w)
    q.put((r, w, mx, total, lo, hi))
    dist.destroy_process_group()


def test_two_ranks_timing_protocol():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == 20.0 for o in out)          # max over ranks seen by every rank
    assert all(o[3] == 2.0 for o in out)
    assert out[0][4:] == (0, 32) and out[1][4:] == (32, 64)


def test_member_partition_covers_everything():
    for n in (1, 5, 64, 65):
        for w in (1, 2, 3, 4, 8):
            got = [ndist.member_range(n, r, w) for r in range(w)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
