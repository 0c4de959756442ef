"""Regression fixture tests/golden/small_workload.json (made by tests/golden/make_golden.py from
the FP64 oracle, which tests/test_oracle_pins.py pins to the reference's known answers): the
oracle reproduces it (CPU), the CUDA library matches it within the parity bars (GPU)."""
import json
import os

import numpy as np
import pytest

from glia_gb300 import _abi
from tests.golden.make_golden import compute

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "small_workload.json")


def _golden():
    with open(GOLDEN) as f:
        return json.load(f)


def _check(got, want, rel, its=True):
    wnorm = np.linalg.norm(np.arange(want["n"] ** 3) % 7 - 3.0)
    for k in ("c1_norm", "c1_sum", "J", "applyd_norm"):
        assert abs(got[k] - want[k]) <= rel * abs(want[k]), k
    for k, scale in (("c1_weighted", want["c1_norm"]), ("applyd_weighted", want["applyd_norm"])):
        assert abs(got[k] - want[k]) <= rel * scale * wnorm, k
    g, w = np.array(got["dJ"]), np.array(want["dJ"])
    assert np.linalg.norm(g - w) <= max(rel, 1e-4 if rel > 1e-9 else rel) * np.linalg.norm(w)
    if its:
        assert got["state_pcg_its"] == want["state_pcg_its"]


def test_oracle_reproduces_the_golden_values():
    from oracle import oracle

    _check(compute(oracle.context(32)), _golden(), 1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [_abi.GLIA_FP64, _abi.GLIA_MIXED])
def test_gpu_matches_the_golden_values(prec):
    from tests.gpu_common import gpu

    got = compute(gpu(32, prec))
    if prec == _abi.GLIA_FP64:
        _check(got, _golden(), 1e-6)
    else:
        _check(got, _golden(), 1e-4, its=False)
