"""Writes the FP64 oracle's full gradient evaluation of the 256^3 headline workload:
tests/golden/workload256.json (J, the 514-entry gradient, PCG totals, state checksums) and
tests/golden/workload256_data.npz (the thresholded observation d as packed bits).

Workload: 256^3, nt = 100, dt = 0.01, 512 Gaussians (sigma = 2pi/64) at the first in-WM lattice
points, p ~ U[0,1] on 5 % (seed 1), rho = 8, kappa = 0.02, k = kappa (wm + 0.2 gm); data = the
oracle's forward with rho * 1.2, kappa * 0.8 and p re-seeded (seed 2), thresholded at 0.5;
O = I, beta = 0. The evaluation follows DerivativeOperatorsRD::evaluateObjectiveAndGradient
(src/grad/DerivativeOperatorsRD.cpp:130-226) with all gradient blocks from one sweep.

The oracle (FP64 C++/OpenMP restatement of the reference's CPU path, pinned to the reference's
known answers by tests/test_oracle_pins.py) needs about an hour on 8 host cores and ~30 GB of
host memory for the full time history at this size.

    python tests/golden/make_config1.py [--threads 8] [--n 256] [--nt 100] [--n-gauss 512]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))


def paths(n):
    stem = os.path.join(HERE, f"workload{n}")
    return stem + ".json", stem + "_data.npz"


def weights(n):
    """Fixed +-/ramp weights for state checksums (x-major voxel index)."""
    i = np.arange(n ** 3, dtype=np.float64)
    return i % 7 - 3.0, np.cos(i * (2 * np.pi / 1009.0))


def load_data(n=256):
    """The thresholded observation d of the fixture as float64 (n^3)."""
    _, npz = paths(n)
    z = np.load(npz)
    bits = np.unpackbits(z["d_bits"])[: n ** 3]
    return bits.astype(np.float64)


def load(n=256):
    js, _ = paths(n)
    with open(js) as f:
        return json.load(f)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nt", type=int, default=100)
    ap.add_argument("--n-gauss", type=int, default=512)
    args = ap.parse_args()

    from glia_gb300 import _abi
    from glia_gb300 import synthetic as syn
    from oracle import oracle

    oracle.set_num_threads(args.threads)
    wl = syn.GradientWorkload(n=args.n, nt=args.nt, n_gauss=args.n_gauss)
    tissue = wl.tissue()
    centers = wl.centers(tissue)
    o = oracle.context(wl.n)
    syn.setup_context(o, wl, tissue, centers, _abi.GLIA_HISTORY_FULL, 0)
    o.set_obs_filter(np.ones(wl.n ** 3))

    t0 = time.time()
    o.set_coefficients(k=wl.kappa * 0.8, rho=wl.rho * 1.2, k_gm_wm=wl.k_gm_wm)
    c_obs1 = o.solve_state(o.phi_apply(wl.p_obs()))
    d = (c_obs1 > 0.5).astype(np.float64)
    margin = float(np.min(np.abs(c_obs1 - 0.5)))
    near = int(np.count_nonzero(np.abs(c_obs1 - 0.5) < 1e-6))
    st_obs = o.stats()
    t_obs = time.time() - t0
    print(f"observation: {t_obs:.0f} s, {int(d.sum())} voxels above 0.5, margin {margin:.3e}",
          flush=True)

    o.set_coefficients(k=wl.kappa, rho=wl.rho, k_gm_wm=wl.k_gm_wm)
    o.reset_stats()
    x = wl.x_eval()
    t0 = time.time()
    J, dJ = o.eval_objective_and_gradient(x, d)
    t_eval = time.time() - t0
    st = o.stats()
    c1 = o.get_state(wl.nt)
    w1, w2 = weights(wl.n)
    print(f"evaluation: {t_eval:.0f} s, J = {J:.12e}", flush=True)

    js, npz = paths(wl.n)
    np.savez_compressed(npz, d_bits=np.packbits(d.astype(np.uint8)))
    out = {"n": wl.n, "nt": wl.nt, "dt": wl.dt, "n_gauss": wl.n_gauss, "rho": wl.rho,
           "kappa": wl.kappa, "k_gm_wm": wl.k_gm_wm, "x": [float(v) for v in x],
           "data_voxels_above": int(d.sum()), "data_margin_to_threshold": margin,
           "data_voxels_within_1e-6": near,
           "observation_pcg_its": int(st_obs["diff_ksp_itr_state"]),
           "J": float(J), "dJ": [float(v) for v in dJ],
           "c1_norm": float(np.linalg.norm(c1)), "c1_sum": float(c1.sum()),
           "c1_weighted_mod7": float(c1 @ w1), "c1_weighted_cos": float(c1 @ w2),
           "stats": {k: (int(v) if float(v).is_integer() else float(v)) for k, v in st.items()},
           "oracle_seconds": {"observation": round(t_obs, 1), "evaluation": round(t_eval, 1),
                              "threads": args.threads}}
    with open(js, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("J", "c1_norm", "stats")}))


if __name__ == "__main__":
    main()
