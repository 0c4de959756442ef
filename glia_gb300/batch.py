"""Batched uneven gradient evaluations: many independent problems of different grid sizes
sharing one GPU.

Each problem owns a context (its own CUDA stream, cuFFT plans, PCG graph). Two ways to run them:
- one CUDA graph (`GraphBatch`, glia_batch_* of the C-ABI): every problem's forward, adjoint and
  gradient sweeps, with their PCG loops as conditional WHILE nodes, captured as parallel branches
  of one graph that is launched once; branches are ordered in groups (contexts of one group run
  concurrently, groups one after another);
- host threads (`Batch.evaluate`): a pool feeds up to `concurrency` contexts at once (the C-ABI
  calls release the GIL); inside each problem the PCG loops run as device-side graphs.
The schedule (launch geometry per grid size; branch grouping for the graph, concurrency for the
threads) is chosen by `autotune_graph` / `autotune`, which measure candidate schedules on a
shortened copy of the batch and cache the winner in a JSON file keyed by the batch's shape.

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


class GraphBatch:
    """A Batch's evaluations as one CUDA graph (glia_batch_capture / launch / results). Each
    context first runs one ordinary evaluation (plans and per-context PCG graphs are created
    there; `reference` keeps those results), then the graph is captured at the problems' x and
    data. The launch geometry must be set before construction: it is part of the graph."""

    def __init__(self, batch: "Batch", group=None):
        import ctypes

        from .native import load

        self.batch = batch
        self.api = load()
        n = len(batch.ctxs)
        self.reference = [c.eval_objective_and_gradient(p.x, d)
                          for c, p, d in zip(batch.ctxs, batch.problems, batch.data)]
        hs = (ctypes.c_void_p * n)(*[c._h.value for c in batch.ctxs])
        self.h = ctypes.c_void_p()
        self._check(self.api.batch_create(hs, n, ctypes.byref(self.h)), "batch_create")
        self.capture(group)

    def _check(self, rc, where):
        if rc != 0:
            from .context import GliaError

            msg = self.api.batch_last_error(self.h) if self.h else b""
            raise GliaError(rc, where, msg.decode() if msg else "")

    def capture(self, group=None):
        import ctypes

        b = self.batch
        n = len(b.ctxs)
        self._xs = [np.ascontiguousarray(p.x, dtype=np.float64) for p in b.problems]
        self._ds = [np.ascontiguousarray(d, dtype=np.float64) for d in b.data]
        D = ctypes.POINTER(ctypes.c_double)
        xs = (D * n)(*[x.ctypes.data_as(D) for x in self._xs])
        nx = (ctypes.c_int * n)(*[x.size for x in self._xs])
        ds = (ctypes.c_void_p * n)(*[d.ctypes.data for d in self._ds])
        grp = None if group is None else (ctypes.c_int * n)(*[int(g) for g in group])
        self._check(self.api.batch_capture(self.h, xs, nx, ds, grp), "batch_capture")
        for c in b.ctxs:  # the capture rewrote the contexts' histories
            c._touch()

    def launch(self):
        self._check(self.api.batch_launch(self.h, None), "batch_launch")

    def results(self):
        import ctypes

        n = len(self.batch.ctxs)
        J = np.zeros(n)
        dJ = [np.zeros(x.size) for x in self._xs]
        D = ctypes.POINTER(ctypes.c_double)
        arr = (D * n)(*[g.ctypes.data_as(D) for g in dJ])
        self._check(self.api.batch_results(self.h, None, J.ctypes.data_as(D), arr),
                    "batch_results")
        return [(float(J[i]), dJ[i]) for i in range(n)]

    def evaluate(self):
        """All problems once through the graph; returns (wall seconds, [(J, dJ)])."""
        t0 = time.perf_counter()
        self.launch()
        res = self.results()
        return time.perf_counter() - t0, res

    def close(self):
        if self.h:
            self.api.batch_destroy(self.h)
            self.h = None


def groupings(problems) -> dict:
    """Candidate branch groupings of the graph: all problems as parallel branches; the largest
    grids first (on their own), then the rest in parallel; one group per grid size, largest
    first; two interleaved halves by decreasing size."""
    n = len(problems)
    sizes = sorted({p.n for p in problems}, reverse=True)
    order = longest_first(problems)
    halves = [0] * n
    for k, i in enumerate(order):
        halves[i] = k % 2
    return {"parallel": [0] * n,
            "largest_first": [0 if p.n == sizes[0] else 1 for p in problems],
            "by_size": [sizes.index(p.n) for p in problems],
            "two_waves": halves}


def autotune_graph(problems, nt_probe: int = 10, cache: str = CACHE, force: bool = False) -> dict:
    """Chooses the launch geometry of the small grids and the branch grouping of the one-graph
    batch by timing each candidate graph on a shortened copy of the batch (nt_probe steps);
    caches the choice per batch signature."""
    sig = "graph:" + signature(problems)
    table = json.load(open(cache)) if os.path.exists(cache) else {}
    if sig in table and not force:
        return table[sig]
    import dataclasses

    probe = [dataclasses.replace(p, nt=nt_probe,
                                 wl=dataclasses.replace(p.wl, nt=nt_probe)) for p in problems]
    candidates = []
    for small in ((8, 4), (2, 1)):
        geometry = {"32": list(small), "64": list(small), "128": list(small), "256": [8, 4]}
        batch = Batch(probe)
        batch.set_geometry(geometry)
        gb = None
        for name, grp in groupings(probe).items():
            if gb is None:
                gb = GraphBatch(batch, grp)
            else:
                gb.capture(grp)
            gb.evaluate()  # warm-up launch
            t, _ = gb.evaluate()
            candidates.append((t, name, geometry, grp))
        gb.close()
        batch.close()
    t, name, geometry, grp = min(candidates, key=lambda c: c[0])
    choice = {"grouping": name, "group": grp, "geometry": geometry, "probe_seconds": t,
              "candidates": [[c[0], c[1], c[2]["64"]] for c in candidates]}
    table[sig] = choice
    os.makedirs(os.path.dirname(cache), exist_ok=True)
    json.dump(table, open(cache, "w"), indent=1)
    return choice


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
    """The batch three ways: one problem at a time (default geometry), host threads (autotuned
    concurrency) and one CUDA graph (autotuned grouping), each the best of `repeats`; the
    graph's results are checked against the ordinary evaluations of the same contexts."""
    problems = default_batch(nt)
    gchoice = autotune_graph(problems)
    choice = autotune(problems)
    n = len(problems)
    batch = Batch(problems)
    order = longest_first(problems)
    batch.evaluate(1, order)
    t_seq = min(batch.evaluate(1, order)[0] for _ in range(repeats))
    batch.set_geometry(choice["geometry"])
    batch.evaluate(choice["concurrency"], order)
    t_thr = min(batch.evaluate(choice["concurrency"], order)[0] for _ in range(repeats))
    batch.set_geometry(gchoice["geometry"])
    gb = GraphBatch(batch, gchoice["group"])
    gb.evaluate()
    t_gr, res = min((gb.evaluate() for _ in range(repeats)), key=lambda r: r[0])
    same = all(J == Jr and np.array_equal(g, gr)
               for (J, g), (Jr, gr) in zip(res, gb.reference))
    gb.close()
    batch.close()
    return {"problems": signature(problems), "sequential_s": t_seq,
            "sequential_evals_per_s": n / t_seq,
            "graph_s": t_gr, "graph_evals_per_s": n / t_gr, "graph_speedup": t_seq / t_gr,
            "graph_equals_single_problem_runs": same,
            "threads_s": t_thr, "threads_evals_per_s": n / t_thr, "threads_speedup": t_seq / t_thr,
            "graph_schedule": {k: gchoice[k] for k in ("grouping", "geometry", "probe_seconds",
                                                       "candidates")},
            "threads_schedule": choice}


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
