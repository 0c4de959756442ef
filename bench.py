"""Throughput of the GB300 reaction–diffusion gradient path (one JSON line on rank 0).

Workload (default): 256^3 forward + adjoint gradient evaluation of J = h^3/2 ||c(1) - d||^2 with
respect to (p[512], kappa, rho); tissue = the seeded synthetic brain, 512 Gaussians
(sigma = 2pi/64) at the first in-WM lattice points, p ~ U[0,1] on 5 % of entries, rho = 8,
kappa = 0.02, dt = 0.01, nt = 100, data = perturbed forward thresholded at 0.5, O = I, beta = 0.
Mixed precision (FP32 fields / transforms, FP64 reductions), checkpoints every 10 steps.

A step is one call of glia_eval_objective_and_gradient. `value` uses device-resident inputs;
`e2e` calls the same entry point with host float64 buffers (the data field crosses PCIe/C2C
every step). Multi-GPU: one independent problem per rank, no data-path collective ("weak").

  python bench.py [--steps K] [--warmup W] [--n 256] [--nt 100] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "256³ fwd+adj gradient evals/s, mixed vs FP64 on GB300 at ≤1e-4 rel grad err"
UNIT = "gradient evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nt", type=int, default=100)
    ap.add_argument("--n-gauss", type=int, default=512)
    ap.add_argument("--every", type=int, default=10, help="checkpoint interval (0 = full history)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison legs")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    ap.add_argument("--no-clocks", action="store_true")
    ap.add_argument("--timing-off", action="store_true", help="no per-kernel event timing")
    return ap.parse_args()


# ------------------------------------------------------------------------------------------
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, enabled, gpu_index):
        self.proc = None
        self.path = None
        if not enabled:
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": reasons, "samples": len(rows)}


def dist_init(args=None, backend=None):
    """One process per GPU (torchrun env). Ranks run independent problems; the process group
    carries only the barrier and the max-over-ranks timing (nccl on GPUs, gloo on CPUs)."""
    import torch

    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------------------------------
def build_workload(args, seed_offset=0):
    from glia_gb300 import synthetic as syn

    wl = syn.GradientWorkload(n=args.n, nt=args.nt, n_gauss=args.n_gauss,
                              tissue_seed=seed_offset)
    tissue = wl.tissue()
    centers = wl.centers(tissue)
    return wl, tissue, centers


def fixture_data(wl):
    """The thresholded observation of the FP64 oracle's stored evaluation of this workload
    (tests/golden/workload256*), or None when the workload is not the stored one."""
    try:
        from tests.golden.make_config1 import load, load_data
        want = load(wl.n)
    except (OSError, ImportError):
        return None, None
    if (want["nt"], want["n_gauss"], want["rho"], want["kappa"]) != (wl.nt, wl.n_gauss, wl.rho,
                                                                     wl.kappa):
        return None, None
    return load_data(wl.n), want


class OracleSample:
    """The FP64 CPU oracle (the port of the reference's CPU path: CN-PCG with the spectral
    preconditioner, Strang splitting, full time history with recomputed half steps, Phi, adjoint,
    trapezoid kappa/rho gradients) set up for the workload with nt_sample time steps. One sample
    is one complete glia_eval_objective_and_gradient call (forward, adjoint, gradient, Phi and
    Phi^T) at the workload's grid; a gradient evaluation at nt steps costs about nt / nt_sample
    samples (the per-evaluation Phi work is counted nt / nt_sample times, so the extrapolation
    slightly overstates the CPU time per evaluation)."""

    def __init__(self, wl, tissue, centers, d, threads, nt_sample=1):
        from glia_gb300 import _abi
        from glia_gb300 import synthetic as syn
        from oracle import oracle

        oracle.set_num_threads(threads)
        self.wl, self.nt_sample, self.threads = wl, nt_sample, threads
        self.o = oracle.context(wl.n)
        syn.setup_context(self.o, wl, tissue, centers, _abi.GLIA_HISTORY_FULL, 0)
        self.o.set_time(wl.dt, nt_sample, 2)
        self.o.set_obs_filter(np.ones(wl.n ** 3))
        self.d = d
        self.x = wl.x_eval()

    def step(self):
        """Seconds of one sample."""
        t0 = time.perf_counter()
        self.o.eval_objective_and_gradient(self.x, self.d)
        return time.perf_counter() - t0

    def evals_per_s(self, t_step):
        return self.nt_sample / (t_step * self.wl.nt)

    def describe(self, t_step, fixture):
        st = self.o.stats()
        its = st["total_pcg_iterations"] / max(1, st["total_diffusion_solves"])
        return (f"one full FP64 oracle gradient evaluation (forward, adjoint with recomputed half "
                f"steps, kappa/rho/p gradients) of the {self.wl.n}^3 workload with nt = "
                f"{self.nt_sample} on {self.threads} threads, {t_step:.2f} s ({its:.1f} PCG its "
                f"per solve, data {'of the oracle fixture' if fixture else 'stand-in'}); "
                f"extrapolated to nt = {self.wl.nt} as {self.wl.nt // self.nt_sample} such "
                f"evaluations")


def reference_data(wl, tissue, centers):
    d, want = fixture_data(wl)
    if d is not None:
        return d, True
    # stand-in data for other sizes: the thresholded initial condition of the perturbed p
    from oracle import oracle
    from glia_gb300 import _abi
    from glia_gb300 import synthetic as syn

    o = oracle.context(wl.n)
    syn.setup_context(o, wl, tissue, centers, _abi.GLIA_HISTORY_FULL, 0)
    c = o.phi_apply(wl.p_obs())
    return (c > 0.5 * c.max()).astype(np.float64), False


# ------------------------------------------------------------------------------------------
def run_reference(args):
    """The reference's CPU implementation of the path (the FP64 oracle port of it) on all host
    cores. Each step is one complete gradient evaluation of the workload at nt = 1 (every stage
    of the path at full grid size); `value` extrapolates it to nt = args.nt."""
    rank = int(os.environ.get("RANK", "0"))
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    wl, tissue, centers = build_workload(args)
    d, fixture = reference_data(wl, tissue, centers)
    smp = OracleSample(wl, tissue, centers, d, cores)
    times = []
    for k in range(args.warmup + args.steps):
        t = smp.step()
        if k >= args.warmup:
            times.append(t)
    t_step = statistics.mean(times)
    v = smp.evals_per_s(t_step)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": workload_config(args),
            "arm": "reference CPU path (FP64 oracle port), all host cores",
            "extrapolated": {"nt_per_step": smp.nt_sample, "nt_per_evaluation": wl.nt,
                             "seconds_per_evaluation": t_step * wl.nt / smp.nt_sample},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": smp.describe(t_step, fixture)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": (f"{args.n}^3 forward+adjoint gradient of J w.r.t. (p[{args.n_gauss}], "
                         f"kappa, rho), nt={args.nt}, dt=0.01, Strang + CN-PCG (rtol 1e-6)"),
            "n": args.n, "nt": args.nt, "n_gauss": args.n_gauss,
            "l2": ("per-step working set > 1 GB (larger than L2 / last-level cache); the GPU arm "
                   "also flushes L2 (256 MiB write) between timed steps")}


# ------------------------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    from glia_gb300 import native

    ws, rank, local = dist_init(args)
    api = native.load()
    # weak scaling: every rank solves its own problem (tissue seed = rank)
    wl, tissue, centers = build_workload(args, seed_offset=rank)
    stream = torch.cuda.Stream()  # the library and the timing events share this stream
    with torch.cuda.stream(stream):
        run_ours(args, torch, api, wl, tissue, centers, stream, ws, rank)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_ours(args, torch, api, wl, tissue, centers, stream, ws, rank):
    from glia_gb300 import _abi
    from glia_gb300 import synthetic as syn
    from glia_gb300.context import Context

    def make_ctx(prec, engine=_abi.GLIA_ENGINE_FUSED, every=args.every):
        ctx = Context(api, wl.n, prec, engine)
        ctx.set_stream(stream.cuda_stream)
        hist = _abi.GLIA_HISTORY_CHECKPOINT if every else _abi.GLIA_HISTORY_FULL
        syn.setup_context(ctx, wl, tissue, centers, hist, every or 0)
        ctx.set_obs_filter(np.ones(wl.n ** 3))
        return ctx

    ctx = make_ctx(_abi.GLIA_MIXED)
    # observation: forward with perturbed parameters, thresholded at 0.5 — the FP64 oracle's
    # (stored with its full evaluation of this workload) when this is the stored workload, else
    # this path's own forward
    d_host, oracle_eval = fixture_data(wl) if rank == 0 else (None, None)
    if d_host is None:
        ctx.set_coefficients(k=wl.kappa * 0.8, rho=wl.rho * 1.2, k_gm_wm=wl.k_gm_wm)
        c_obs1 = ctx.solve_state(ctx.phi_apply(wl.p_obs()))
        d_host = (c_obs1 > 0.5).astype(np.float64)
        ctx.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    x = wl.x_eval()

    # ---- device-resident timed region ------------------------------------------------------
    ctx.set_pointer_mode(_abi.GLIA_PTR_DEVICE_F32)
    d_dev = torch.tensor(d_host, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        ctx.eval_objective_and_gradient(x, d_dev)
    ctx.reset_stats()
    clocks = Clocks(not args.no_clocks and rank == 0, torch.cuda.current_device())
    barrier(ws)
    torch.cuda.synchronize()
    step_ms = []
    J = grad = None
    for _ in range(args.steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("timed_step")
        e0.record(stream)
        J, grad = ctx.eval_objective_and_gradient(x, d_dev)
        e1.record(stream)
        e1.synchronize()
        torch.cuda.nvtx.range_pop()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    st = ctx.stats()
    ms = max_over_ranks(ws, statistics.mean(step_ms))
    value = ws * 1000.0 / ms
    # per-kernel live timing: one more evaluation with every launch bracketed by CUDA events on
    # the library's stream (the PCG loop then runs host-driven instead of as a graph)
    kt = {}
    if not args.timing_off:
        ctx.set_timing(True)
        flush.fill_(1.0)
        torch.cuda.nvtx.range_push("instrumented_eval")
        ctx.eval_objective_and_gradient(x, d_dev)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        kt = ctx.timing()
        ctx.set_timing(False)

    # ---- roofline of the dominant kernel ---------------------------------------------------
    peak, peak_kind = peaks()
    ours = {k: v for k, v in kt.items() if not k.startswith("cufft") and k != "copy_d2d" and v[0]}
    roofline = None
    breakdown = {}
    total_kt = sum(v[1] for v in kt.values()) or 1.0
    for k, (launches, kms, kbytes) in kt.items():
        if launches:
            breakdown[k] = {"launches": launches, "ms": round(kms, 3),
                            "share": round(kms / total_kt, 4),
                            "gbs": round(kbytes / (kms * 1e-3) / 1e9, 1) if kms else None}
    if ours:
        dom = max(ours, key=lambda k: ours[k][1])
        launches, kms, kbytes = ours[dom]
        achieved = kbytes / (kms * 1e-3) / 1e9
        roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1),
                    "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                    "traffic": traffic_for(dom, kbytes / launches, wl.n),
                    "algorithmic_bytes_per_launch": kbytes / launches,
                    "avg_launch_us": kms * 1e3 / launches,
                    "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)"
                    if peak_kind == "measured" else "fallback 6.8 TB/s"}
    our_launches = args.steps * sum(v[0] for k, v in kt.items()
                                    if not k.startswith("cufft") and k != "copy_d2d")
    path_bytes = sum(v[2] for v in kt.values())
    path_gbs = path_bytes / (ms * 1e-3) / 1e9 if kt else None

    # ---- end to end through the host-buffer API --------------------------------------------
    ctx.set_pointer_mode(_abi.GLIA_PTR_HOST_F64)
    d_pin = torch.from_numpy(d_host).pin_memory().numpy()
    ctx.eval_objective_and_gradient(x, d_pin)
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        Je, ge = ctx.eval_objective_and_gradient(x, d_pin)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_s = max_over_ranks(ws, e2e_s)
    e2e = {"value": ws / e2e_s, "unit": UNIT, "h2d_bytes_per_step": d_host.nbytes + x.nbytes,
           "d2h_bytes_per_step": 8 + grad.nbytes}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 (f64 reductions)", "data": "synthetic",
           "config": workload_config(args),
           "arm": (f"mixed fused GPU path, checkpoint every {args.every}" if args.every
                   else "mixed fused GPU path, full history"),
           "data_source": ("the FP64 oracle's observation (tests/golden/workload256_data.npz)"
                           if oracle_eval else "this path's own perturbed forward"),
           "e2e": e2e, "gpu_launches": our_launches, "roofline": roofline,
           "path_gbs_algorithmic": round(path_gbs, 1) if path_gbs else None,
           "kernels": breakdown, "clocks": clk,
           "pcg": {"solves_per_eval": st["total_diffusion_solves"] / args.steps,
                   "its_per_solve": st["total_pcg_iterations"] / max(1, st["total_diffusion_solves"]),
                   "pcg_loop": "CUDA graph, device-side WHILE node",
                   "ffts_per_eval": st["total_fft_execs"] / args.steps},
           "J": J}

    if oracle_eval is not None:
        out.update(grad_errors(grad, np.array(oracle_eval["dJ"]), wl.n_gauss, "oracle"))
        out["J_rel_err_vs_oracle"] = abs(J - oracle_eval["J"]) / abs(oracle_eval["J"])

    # ---- FP64 GPU legs: our fused FP64 and the reference-structured plain FP64 path ---------
    # (one-GPU runs only: under torchrun they would hold every rank's GPU for minutes)
    if not args.no_fp64 and rank == 0 and ws == 1:
        legs = {}
        ref_grad = None
        for name, prec, engine, every in (("fp64_fused", _abi.GLIA_FP64, _abi.GLIA_ENGINE_FUSED, args.every),
                                          ("fp64_plain_reference_structured", _abi.GLIA_FP64,
                                           _abi.GLIA_ENGINE_REFERENCE, 0)):
            del_ctx = None
            try:
                c2 = make_ctx(prec, engine, every)
                c2.set_pointer_mode(_abi.GLIA_PTR_DEVICE_F64)
                d64 = torch.tensor(d_host, dtype=torch.float64, device="cuda")
                c2.eval_objective_and_gradient(x, d64)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                J2, g2 = c2.eval_objective_and_gradient(x, d64)
                e1.record(stream)
                e1.synchronize()
                t = e0.elapsed_time(e1)
                legs[name] = {"ms_per_step": t, "value": 1000.0 / t, "J": J2}
                if ref_grad is None:
                    ref_grad = g2
                del_ctx = c2
            except Exception as exc:  # noqa: BLE001
                legs[name] = {"error": str(exc)[:200]}
            finally:
                if del_ctx is not None:
                    del_ctx.close()
                torch.cuda.empty_cache()
        if ref_grad is not None:
            npp = wl.n_gauss
            out.update(grad_errors(grad, ref_grad, npp, "fp64"))
            if oracle_eval is not None:
                e = grad_errors(ref_grad, np.array(oracle_eval["dJ"]), npp, "oracle")
                legs["fp64_fused"]["grad_rel_err_vs_oracle"] = e["grad_rel_err_vs_oracle"]
            out["grad_fp64"] = {"kappa": float(ref_grad[npp]), "rho": float(ref_grad[npp + 1]),
                                "p_norm": float(np.linalg.norm(ref_grad[:npp]))}
        out["fp64_gpu"] = legs
        plain = legs.get("fp64_plain_reference_structured", {}).get("value")
        if plain:
            out["speedup_vs_fp64_plain_gpu"] = value / plain

    # ---- CPU baseline (rank 0, one GPU) ----------------------------------------------------
    if not args.no_cpu and rank == 0 and ws == 1:
        try:
            cores = os.cpu_count() or 1
            smp = OracleSample(wl, tissue, centers, d_host, cores)
            smp.step()  # first touch of the oracle's buffers
            t_step = smp.step()
            out["cpu_baseline"] = {"value": smp.evals_per_s(t_step), "unit": UNIT, "cores": cores,
                                   "kind": "port",
                                   "sample": smp.describe(t_step, oracle_eval is not None)}
        except Exception as exc:  # noqa: BLE001
            out["cpu_baseline"] = {"error": str(exc)[:200]}
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()


def grad_errors(grad, ref, npp, name):
    """Relative L2 error of a gradient (p[npp], kappa, rho) against `ref`, whole and per block."""
    return {f"grad_rel_err_vs_{name}": float(np.linalg.norm(grad - ref) / np.linalg.norm(ref)),
            f"grad_rel_err_blocks_vs_{name}": {
                "p": float(np.linalg.norm(grad[:npp] - ref[:npp]) / np.linalg.norm(ref[:npp])),
                "kappa": float(abs(grad[npp] - ref[npp]) / abs(ref[npp])),
                "rho": float(abs(grad[npp + 1] - ref[npp + 1]) / abs(ref[npp + 1]))}}


def traffic_for(kernel: str, algorithmic_per_launch: float, n: int):
    """DRAM bytes per launch of `kernel` from the committed ncu summary (profiles/traffic.json),
    scaled to n^3 by voxel count when it was captured on a smaller grid."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    d = json.load(open(p)).get(kernel)
    if not d:
        return None
    return d["dram_bytes_per_launch"] * (n / d["n"]) ** 3


if __name__ == "__main__":
    main()
