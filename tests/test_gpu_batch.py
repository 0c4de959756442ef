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


def test_graph_batch_equals_single_problem_runs():
    """One CUDA graph over uneven problems (glia_batch_*): every grouping of the branches gives
    each problem's (J, dJ) bit for bit as its own ordinary evaluation, launch after launch."""
    probs = gb.default_batch(nt=3, sizes=(32, 64, 32, 128, 64, 256))
    b = gb.Batch(probs)
    b.set_geometry({"32": (2, 1), "64": (2, 1), "128": (8, 4), "256": (8, 4)})
    g = gb.GraphBatch(b)
    try:
        for name, grp in gb.groupings(probs).items():
            g.capture(grp)
            for _ in range(2):
                _, res = g.evaluate()
                for (J, dJ), (Jr, gr) in zip(res, g.reference):
                    assert J == Jr, name
                    assert np.array_equal(dJ, gr), name
    finally:
        g.close()
        b.close()


def test_graph_batch_members_match_the_oracle():
    """The 64^3 members of a graph batch against the FP64 oracle on the same inputs."""
    from glia_gb300 import _abi
    from glia_gb300 import synthetic as syn
    from tests.gpu_common import GRAD_TOL, orc
    from tests.helpers import rel_l2

    probs = gb.default_batch(nt=4, sizes=(64, 64, 32))
    b = gb.Batch(probs)
    g = gb.GraphBatch(b, [0, 0, 1])
    try:
        _, res = g.evaluate()
    finally:
        g.close()
        b.close()
    for pr, d, (J, dJ) in zip(probs, b.data, res):
        if pr.n != 64:
            continue
        o = orc(64)
        syn.setup_context(o, pr.wl, pr.tissue, pr.centers, _abi.GLIA_HISTORY_FULL, 0)
        o.set_obs_filter(np.ones(64 ** 3))
        Jo, go = o.eval_objective_and_gradient(pr.x, d)
        assert abs(J - Jo) <= 1e-4 * abs(Jo)
        assert rel_l2(dJ, go) <= GRAD_TOL


def test_graph_autotune_writes_a_schedule(tmp_path):
    probs = gb.default_batch(nt=2, sizes=(32, 32, 64))
    cache = tmp_path / "autotune.json"
    choice = gb.autotune_graph(probs, nt_probe=2, cache=str(cache))
    assert choice["grouping"] in gb.groupings(probs)
    assert len(choice["group"]) == len(probs)
    table = json.load(open(cache))
    assert "graph:" + gb.signature(probs) in table


def test_captured_contexts_report_no_history_until_a_launch_is_read():
    """After glia_batch_capture nothing has run: the contexts refuse the adjoint (no valid state
    history) until glia_batch_results has read a launch of the graph."""
    from glia_gb300.context import GliaError

    probs = gb.default_batch(nt=2, sizes=(32, 32))
    b = gb.Batch(probs)
    g = gb.GraphBatch(b)
    try:
        pt = np.zeros(32 ** 3)
        with pytest.raises(GliaError, match="GLIA_ERR_STATE"):
            b.ctxs[0].solve_adjoint(pt)
        g.evaluate()
        b.ctxs[0].solve_adjoint(pt)  # the launch's history is valid now
    finally:
        g.close()
        b.close()
