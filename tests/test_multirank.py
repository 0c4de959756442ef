"""The multi-rank paths on CPU, world size 2 over gloo: bench.py's weak scaling (one independent
problem per rank, barrier around the timed region, max-over-ranks timing) and the batch split
over ranks (LPT partition by n^3 nt, one gather of (J, dJ) at the end). The per-rank work is
small evaluations on the FP64 oracle."""
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
    with mp.get_context("spawn").Manager() as m:  # no fork of this threaded process
        out = m.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    (J0, t0, m0, w0), (J1, t1, m1, w1) = res[0], res[1]
    assert m0 == m1 == max(t0, t1)          # every rank sees the slowest rank's time
    assert w0 != w1 and J0 != J1            # the ranks solved different problems
    value = ws / m0                          # whole-job evaluations per second
    assert value > 0


def _small_problems():
    from glia_gb300.batch import Problem
    from tests.gpu_common import small_problem

    probs, n = [], 32
    for b, nt in enumerate((1, 2, 1, 1)):  # uneven costs n^3 nt
        wl, tissue, centers = small_problem(n, nt, n_gauss=8, seed=b)
        x = np.concatenate([np.linspace(0.2, 1.0, 8), [wl.kappa, wl.rho]])
        probs.append(Problem(n, nt, wl, tissue, centers, x, b))
    return probs


def _evaluate_on_oracle(pr):
    from oracle import oracle
    from tests.gpu_common import configure

    ctx = oracle.context(pr.n)
    configure(ctx, pr.wl, pr.tissue, pr.centers)
    J, dJ = ctx.eval_objective_and_gradient(pr.x, np.full(pr.n ** 3, 0.1))
    return float(J), [float(v) for v in dJ]


def _batch_rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import torch.distributed as dist

    from glia_gb300.batch import evaluate_sharded

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    probs = _small_problems()
    done = []

    def one(i):
        done.append(i)
        return _evaluate_on_oracle(probs[i])

    res, parts = evaluate_sharded(probs, one, rank, ws)
    out[rank] = (res, parts, done)
    dist.destroy_process_group()


def test_lpt_partition():
    from glia_gb300.batch import lpt_partition

    costs = [64 ** 3] * 16 + [128 ** 3] * 12 + [256 ** 3] * 4  # the default batch, n^3 nt / nt
    for world in (1, 2, 3, 4, 8):
        parts = lpt_partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        bound = max(max(costs), sum(costs) / world)  # no schedule does better
        assert max(loads) <= 4.0 / 3.0 * bound
        assert parts == lpt_partition(costs, world)
    assert lpt_partition(costs, 4)[0][0] == 28  # the largest problems go out first
    assert lpt_partition([], 2) == [[], []]


def test_two_gloo_ranks_sharded_batch():
    ws, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of this threaded process
        out = m.dict()
        mp.spawn(_batch_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    (r0, parts0, done0), (r1, parts1, done1) = res[0], res[1]
    assert parts0 == parts1
    assert sorted(done0 + done1) == list(range(4)) and not set(done0) & set(done1)
    assert r0 == r1  # every rank holds every problem's result after the gather
    # against one process evaluating all problems (OpenMP sums: equal to rounding)
    ref = [_evaluate_on_oracle(p) for p in _small_problems()]
    for (J, dJ), (Jr, dJr) in zip(r0, ref):
        assert abs(J - Jr) <= 1e-12 * abs(Jr)
        assert np.allclose(dJ, dJr, rtol=1e-10, atol=0)
