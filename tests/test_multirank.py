"""Multi-GPU runs are replicas: each rank integrates its own independent
solve, and the only cross-rank communication is the host-side timing
reduction of bench.py (barrier, max of the per-rank times) and the seed
offset per rank.  That logic is checked here with world_size 2 over gloo on
CPU (no GPU involved)."""
import os
import socket

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_env()
    bench.barrier(w)
    t = bench.max_over_ranks(1.5 + r, w)
    total = bench.sum_over_ranks(10.0 * (r + 1), w)
    from nlsemagic_gb300 import workloads as W
    # replicas use distinct seeds (rank offset) -> different inputs, same shapes
    wl = W.vortex_rings_3d(seed=1002 + r, n=12, method=2, steps=5)
    q.put((r, w, local, t, total, wl.U.shape, float(abs(wl.U).sum())))
    dist.destroy_process_group()


def test_replica_timing_reduction_gloo_world2():
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
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 2.5 for o in out)      # max over ranks
    assert all(o[4] == 30.0 for o in out)     # whole-job aggregate
    assert out[0][5] == out[1][5]
    assert out[0][6] != out[1][6]             # independent replicas
