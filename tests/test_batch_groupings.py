"""The branch groupings the batch-graph autotuner tries (glia_gb300/batch.py, `groupings`), on the
CPU: every grouping covers every problem, and the size-based ones order the largest grids
first."""
from dataclasses import dataclass

from glia_gb300 import batch as gb


@dataclass
class _P:
    n: int


def test_groupings_cover_every_problem_and_order_by_size():
    probs = [_P(64), _P(256), _P(128), _P(64), _P(256), _P(128), _P(64)]
    g = gb.groupings(probs)
    assert set(g) == {"parallel", "largest_first", "by_size", "two_waves"}
    for grp in g.values():
        assert len(grp) == len(probs)
    assert g["parallel"] == [0] * len(probs)
    assert [x for x, p in zip(g["largest_first"], probs) if p.n == 256] == [0, 0]
    assert all(x == 1 for x, p in zip(g["largest_first"], probs) if p.n != 256)
    assert g["by_size"] == [{256: 0, 128: 1, 64: 2}[p.n] for p in probs]
    # two interleaved waves by decreasing size: each wave gets one of the two 256^3 problems
    assert sorted(x for x, p in zip(g["two_waves"], probs) if p.n == 256) == [0, 1]
