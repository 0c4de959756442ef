"""Batched uneven gradient evaluations: many independent problems of different grid sizes
sharing one GPU.

Each problem owns a context (its own CUDA stream, cuFFT plans, PCG graph). A pool of host
threads feeds the contexts (the C-ABI calls release the GIL), so up to `concurrency` problems are
in flight at once and the GPU overlaps their kernels; inside each problem the PCG loops run as
device-side graphs, so the threads issue work and wait on one small read per sweep. The schedule
(concurrency, launch geometry per grid size, longest-first order) is chosen by `autotune`, which
measures candidate schedules on a shortened copy of the batch and caches the winner in a JSON
file keyed by the batch's shape.

The default batch: 32 problems, 16 at 64^3, 12 at 128^3 and 4 at 256^3; problem b has tissue seed
1000 + b, rho ~ U[4, 15], kappa ~ U[0.005, 0.1], 64 / 216 / 512 Gaussians (by grid) with 5 % active,
FP32 fields with FP64 reductions.

    python -m glia_gb300.batch            # autotuned batch vs the same problems one at a time
    torchrun --nproc-per-node N -m glia_gb300.batch   # the batch split over N GPUs (LPT by n^3 nt)
"""
from __future__ import annotations

import argparse
import json
import os
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


@dataclass
class Problem:
    n: int
    nt: int
    wl: object
    tissue: object
    centers: np.ndarray
    x: np.ndarray
    seed: int


def default_batch(nt: int = 100, sizes=(64,) * 16 + (128,) * 12 + (256,) * 4):
    from . import synthetic as syn

    probs = []
    gauss = {32: 8, 64: 64, 128: 216, 256: 512}
    for b, n in enumerate(sizes):
        rng = np.random.default_rng(1000 + b)
        rho = float(rng.uniform(4.0, 15.0))
        kappa = float(rng.uniform(0.005, 0.1))
        ng = gauss.get(n, 64)
        wl = syn.GradientWorkload(n=n, nt=nt, n_gauss=ng, rho=rho, kappa=kappa,
                                  tissue_seed=1000 + b)
        tissue = wl.tissue()
        centers = syn.lattice_centers_in_mask(tissue.wm > 0.5, ng)
        p = syn.sparse_coefficients(ng, 0.05, 1000 + b)
        probs.append(Problem(n, nt, wl, tissue, centers, np.concatenate([p, [kappa, rho]]),
                             1000 + b))
    return probs


class Batch:
    """Contexts and data for a list of problems (mixed precision, checkpoint every 10 steps)."""

    def __init__(self, problems, every: int = 10):
        import torch

        from . import _abi
        from . import synthetic as syn
        from .context import Context
        from .native import load

        api = load()
        self.problems = problems
        self.ctxs, self.data, self.streams = [], [], []
        for pr in problems:
            ctx = Context(api, pr.n, _abi.GLIA_MIXED)
            s = torch.cuda.Stream()
            ctx.set_stream(s.cuda_stream)
            hist = _abi.GLIA_HISTORY_CHECKPOINT if every else _abi.GLIA_HISTORY_FULL
            syn.setup_context(ctx, pr.wl, pr.tissue, pr.centers, hist, every or 0)
            ctx.set_obs_filter(np.ones(pr.n ** 3))
            # data: forward with perturbed parameters, thresholded at half its maximum
            ctx.set_coefficients(k=pr.wl.kappa * 0.8, rho=pr.wl.rho * 1.2, k_gm_wm=pr.wl.k_gm_wm)
            p_obs = np.roll(pr.x[:-2], 1)
            c1 = ctx.solve_state(ctx.phi_apply(p_obs))
            self.data.append((c1 > 0.5 * c1.max()).astype(np.float64))
            ctx.set_coefficients(k=pr.wl.kappa, rho=pr.wl.rho, k_gm_wm=pr.wl.k_gm_wm)
            self.ctxs.append(ctx)
            self.streams.append(s)

    def set_geometry(self, geometry: dict):
        for pr, ctx in zip(self.problems, self.ctxs):
            pw, red = geometry.get(str(pr.n), (8, 4))
            ctx.set_launch_geometry(pw, red)

    def evaluate(self, concurrency: int, order=None):
        """All problems once; returns (wall seconds, [(J, dJ)])."""
        order = order if order is not None else range(len(self.ctxs))
        results = [None] * len(self.ctxs)

        def one(i):
            results[i] = self.ctxs[i].eval_objective_and_gradient(self.problems[i].x,
                                                                  self.data[i])

        t0 = time.perf_counter()
        if concurrency <= 1:
            for i in order:
                one(i)
        else:
            with ThreadPoolExecutor(max_workers=concurrency) as ex:
                list(ex.map(one, order))
        return time.perf_counter() - t0, results

    def close(self):
        for c in self.ctxs:
            c.close()


def signature(problems) -> str:
    sizes = {}
    for p in problems:
        sizes[p.n] = sizes.get(p.n, 0) + 1
    return ",".join(f"{n}x{c}" for n, c in sorted(sizes.items())) + f",nt{problems[0].nt}"


def longest_first(problems):
    return sorted(range(len(problems)), key=lambda i: -problems[i].n ** 3)


def cost(problem) -> float:
    """Estimated work of one gradient evaluation, n^3 nt (the PCG iterations per solve of this
    problem family vary little with the parameters)."""
    return float(problem.n) ** 3 * problem.nt


def lpt_partition(costs, world: int):
    """Greedy longest-processing-time assignment of problems to ranks: problems by decreasing
    cost, each to the least-loaded rank (ties to the lower rank, then the lower index), so the
    largest rank load is at most 4/3 of the optimum. One index list per rank, each by decreasing
    cost."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(i)
        loads[r] += costs[i]
    return parts


def evaluate_sharded(problems, evaluate_one, rank: int, world: int):
    """Multi-GPU batch: this rank evaluates its LPT share (evaluate_one(i) -> (J, dJ), on the
    rank's own GPU), then one all_gather_object gives every rank every problem's (J, dJ). The
    evaluations need no collective; the gather is the only exchange. Returns (results in problem
    order, the partition)."""
    parts = lpt_partition([cost(p) for p in problems], world)
    mine = {i: evaluate_one(i) for i in parts[rank]}
    gathered = [mine]
    if world > 1:
        import torch.distributed as dist

        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
    out = [None] * len(problems)
    for part in gathered:
        for i, r in part.items():
            out[i] = r
    return out, parts


def autotune(problems, nt_probe: int = 10, cache: str = CACHE, force: bool = False) -> dict:
    """Chooses concurrency and per-size launch geometry by timing a shortened copy of the batch
    (nt_probe steps); caches the choice per batch signature."""
    sig = signature(problems)
    table = json.load(open(cache)) if os.path.exists(cache) else {}
    if sig in table and not force:
        return table[sig]
    import dataclasses

    probe = [dataclasses.replace(p, nt=nt_probe,
                                 wl=dataclasses.replace(p.wl, nt=nt_probe)) for p in problems]
    batch = Batch(probe)
    order = longest_first(probe)
    candidates = []
    for conc in (1, 4, 8, 16):
        for small in ((8, 4), (2, 1), (1, 1)):
            geometry = {"64": list(small), "128": list(small), "256": [8, 4]}
            batch.set_geometry(geometry)
            batch.evaluate(conc, order)  # warm-up (plans, graphs)
            t, _ = batch.evaluate(conc, order)
            candidates.append((t, conc, geometry))
    batch.close()
    t, conc, geometry = min(candidates, key=lambda c: c[0])
    choice = {"concurrency": conc, "geometry": geometry, "probe_seconds": t,
              "candidates": [[c[0], c[1], c[2]["64"]] for c in candidates]}
    table[sig] = choice
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    json.dump(table, open(cache, "w"), indent=1)
    return choice


def run(nt: int = 100, repeats: int = 2):
    problems = default_batch(nt)
    choice = autotune(problems)
    batch = Batch(problems)
    order = longest_first(problems)
    # sequential: one problem at a time, default launch geometry
    batch.evaluate(1, order)
    t_seq = min(batch.evaluate(1, order)[0] for _ in range(repeats))
    batch.set_geometry(choice["geometry"])
    batch.evaluate(choice["concurrency"], order)
    t_bat, res = min((batch.evaluate(choice["concurrency"], order) for _ in range(repeats)),
                     key=lambda r: r[0])
    batch.close()
    n = len(problems)
    return {"problems": signature(problems), "sequential_s": t_seq, "batched_s": t_bat,
            "sequential_evals_per_s": n / t_seq, "batched_evals_per_s": n / t_bat,
            "speedup": t_seq / t_bat, "schedule": choice}


def run_distributed(nt: int = 100):
    """The default batch over WORLD_SIZE ranks (torchrun, one GPU per rank): each rank builds
    contexts for its LPT share on its GPU and evaluates them with the autotuned schedule; rank 0
    reports the slowest rank's wall time and the gathered results' count."""
    import torch
    import torch.distributed as dist

    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
    dist.init_process_group("nccl")
    problems = default_batch(nt)
    parts = lpt_partition([cost(p) for p in problems], world)
    share = [problems[i] for i in parts[rank]]
    choice = autotune(share) if share else {"concurrency": 1, "geometry": {}}
    batch = Batch(share)
    batch.set_geometry(choice["geometry"])
    local = {i: k for k, i in enumerate(parts[rank])}
    dist.barrier()
    t0 = time.perf_counter()
    _, res = batch.evaluate(choice["concurrency"])
    results, _ = evaluate_sharded(problems, lambda i: res[local[i]], rank, world)
    dist.barrier()
    dt = torch.tensor([time.perf_counter() - t0], dtype=torch.float64, device="cuda")
    dist.all_reduce(dt, op=dist.ReduceOp.MAX)
    batch.close()
    out = {"problems": signature(problems), "ranks": world, "wall_s": float(dt.item()),
           "evals_per_s": len(problems) / float(dt.item()), "gathered": sum(
               r is not None for r in results), "partition": parts}
    dist.destroy_process_group()
    return out if rank == 0 else None


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--nt", type=int, default=100)
    a = ap.parse_args()
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        r = run_distributed(a.nt)
        if r is not None:
            print(json.dumps(r))
    else:
        print(json.dumps(run(a.nt)))
