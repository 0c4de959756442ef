"""Writes tests/golden/small_workload.json: regression values of the FP64 oracle (pinned to the
reference's known answers in tests/test_oracle_pins.py) on a seeded 32^3 workload — the state
norm and checksums, J and the gradient (p, kappa, rho), the PCG iteration counts, a D apply
checksum. The reference itself cannot run here (PETSc, MPI, accFFT absent), so these pin the
oracle and the library against drift, not against the reference.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_workload.json")


def compute(ctx):
    """The fixture's quantities from a configured context (oracle or CUDA library)."""
    from tests.gpu_common import configure, observation, small_problem
    from tests.helpers import reference_test_field

    n, nt = 32, 4
    wl, tissue, centers = small_problem(n, nt, n_gauss=8, seed=0)
    configure(ctx, wl, tissue, centers)
    ctx.set_obs_filter(np.ones(n ** 3))
    x = np.concatenate([np.linspace(0.2, 0.9, len(centers)), [wl.kappa, wl.rho]])
    d1 = observation(wl, tissue, centers)
    weight = np.arange(n ** 3, dtype=np.float64) % 7 - 3.0
    c1 = ctx.solve_state(ctx.phi_apply(x[:-2]))
    st = ctx.stats()
    J, dJ = ctx.eval_objective_and_gradient(x, d1)
    df = ctx.apply_d(reference_test_field(n))
    return {"n": n, "nt": nt, "c1_norm": float(np.linalg.norm(c1)), "c1_sum": float(c1.sum()),
            "c1_weighted": float(c1 @ weight), "state_pcg_its": int(st["diff_ksp_itr_state"]),
            "J": float(J), "dJ": [float(v) for v in dJ],
            "applyd_weighted": float(df @ weight), "applyd_norm": float(np.linalg.norm(df))}


if __name__ == "__main__":
    from oracle import oracle

    vals = compute(oracle.context(32))
    with open(OUT, "w") as f:
        json.dump(vals, f, indent=1)
    print(json.dumps(vals))
