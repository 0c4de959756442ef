"""Batched uneven problems on one GPU (glia_gb300/batch.py): concurrent contexts give the same
results as running the problems one at a time; the autotuner picks and caches a schedule."""
import json

import numpy as np
import pytest

from glia_gb300 import batch as gb

pytestmark = pytest.mark.gpu


def test_concurrent_batch_equals_sequential():
    probs = gb.default_batch(nt=3, sizes=(32, 32, 32, 64, 64))
    b = gb.Batch(probs)
    b.set_geometry({"32": (2, 1), "64": (2, 1)})
    _, seq = b.evaluate(1)
    _, con = b.evaluate(4, gb.longest_first(probs))
    b.close()
    for (J0, g0), (J1, g1) in zip(seq, con):
        assert J0 == J1 and np.array_equal(g0, g1)


def test_autotune_writes_a_schedule(tmp_path):
    probs = gb.default_batch(nt=2, sizes=(32, 32, 64))
    cache = tmp_path / "autotune.json"
    choice = gb.autotune(probs, nt_probe=2, cache=str(cache))
    assert choice["concurrency"] in (1, 4, 8, 16)
    table = json.load(open(cache))
    assert gb.signature(probs) in table
    assert gb.autotune(probs, nt_probe=2, cache=str(cache)) == table[gb.signature(probs)]
