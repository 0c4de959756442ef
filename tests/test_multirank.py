"""The multi-rank path of bench.py on CPU: world size 2 over gloo, one independent problem per
rank (different tissue seeds), barrier around the timed region, max-over-ranks timing and the
weak-scaling aggregate. The per-rank step is a small evaluation on the FP64 oracle."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    import time

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import bench
    from oracle import oracle
    from tests.gpu_common import configure, small_problem

    w, r, _ = bench.dist_init(backend="gloo")
    assert (w, r) == (ws, rank)
    wl, tissue, centers = small_problem(32, 2, n_gauss=8, seed=r)  # independent problem per rank
    ctx = oracle.context(32)
    configure(ctx, wl, tissue, centers)
    x = np.concatenate([np.linspace(0.2, 1.0, 8), [wl.kappa, wl.rho]])
    bench.barrier(w)
    t0 = time.perf_counter()
    J = ctx.eval_objective(x, np.zeros(32 ** 3))
    dt = time.perf_counter() - t0 + 0.05 * r  # rank 1 is slower on purpose
    bench.barrier(w)
    tmax = bench.max_over_ranks(w, dt)
    out[rank] = (J, dt, tmax, float(tissue.wm.sum()))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling():
    ws, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    (J0, t0, m0, w0), (J1, t1, m1, w1) = res[0], res[1]
    assert m0 == m1 == max(t0, t1)          # every rank sees the slowest rank's time
    assert w0 != w1 and J0 != J1            # the ranks solved different problems
    value = ws / m0                          # whole-job evaluations per second
    assert value > 0
