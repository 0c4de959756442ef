"""The mbarrier phase bookkeeping of the bulk-copy staged kernels (ownfft.cuh) on the CPU.

Each slot's barrier completes one phase per copy staged into it. A wait for phase j uses parity
j & 1 and is only correct while the barrier's current phase is j or j + 1. When a bounded wait
runs out, the kernel must wait (bounded) for exactly the copies still in flight before the CTA
returns, or a copy could land in shared memory that the next CTA on the SM already owns.

The models below restate the kernels' order of stage/issue and wait calls per CTA and check, at
every wait site: the normal wait names the oldest pending phase, and the timeout handler's waits
name every pending phase of both barriers (same parity) and nothing else.
"""
import pytest


class Barrier:
    def __init__(self):
        self.staged = 0      # phases armed (arrive.expect_tx issued)
        self.completed = 0   # phases completed

    def pending(self):
        return list(range(self.completed, self.staged))


def check_wait(bar, parity):
    """A normal wait: the barrier's oldest pending phase j has parity `parity`; complete it."""
    pend = bar.pending()
    assert pend, "wait on a barrier with no copy armed"
    assert pend[0] & 1 == parity
    bar.completed += 1


def check_handler(bars, late, handler_waits):
    """Timeout at barrier `late`: the handler's (barrier, parity) waits cover every pending phase."""
    want = sorted((b, p & 1) for b in range(len(bars)) for p in bars[b].pending())
    assert all(len(bar.pending()) <= 1 for bar in bars)  # one parity names one phase
    assert sorted(handler_waits) == want, (late, handler_waits, want)


def yinv_bulk_schedule(block, grid, ntiles):
    """k_yinv_bulk: slot 0 holds G_x, slot 1 G_0 of the same tile; slot 0 is re-staged during the
    G_x transform, slot 1 after its rows are read into registers."""
    bars = [Barrier(), Barrier()]

    def stage(slot, t):
        if t < ntiles:
            bars[slot].staged += 1

    stage(0, block)
    stage(1, block)
    it = 0
    tile = block
    while tile < ntiles:
        nxt = tile + grid < ntiles
        # ready(0, it, next)
        check_handler(bars, 0, [(0, it & 1), (1, it & 1)])
        check_wait(bars[0], it & 1)
        stage(0, tile + grid)
        # ready(1, it, next)
        check_handler(bars, 1, [(1, it & 1)] + ([(0, (it + 1) & 1)] if nxt else []))
        check_wait(bars[1], it & 1)
        stage(1, tile + grid)
        tile += grid
        it += 1
    assert all(b.pending() == [] for b in bars)


def yfwd_schedule(block, grid, ntiles):
    """k_yfwd (TMA option): items i = 3 per tile through slots i % 2, item i + 2 issued during
    item i's transform; phase of item i on its slot = i >> 1."""
    bars = [Barrier(), Barrier()]
    mytiles = (ntiles - block + grid - 1) // grid if block < ntiles else 0
    nitems = 3 * mytiles

    def issue(i):
        if i < nitems:
            bars[i & 1].staged += 1

    issue(0)
    issue(1)
    for i in range(nitems):
        handler = [(q & 1, (q >> 1) & 1) for q in range(i, min(i + 2, nitems))]
        check_handler(bars, i & 1, handler)
        check_wait(bars[i & 1], (i >> 1) & 1)
        issue(i + 2)
    assert all(b.pending() == [] for b in bars)


# n -> tiles of the y passes (n * (n/2) / T with YDecomp's T) and the persistent grids used
TILES = {64: 64 * 1, 128: 128 * 2, 256: 256 * 8}
GRIDS = [1, 2, 3, 7, 152, 304, 456, 608, 5000]


@pytest.mark.parametrize("n", sorted(TILES))
@pytest.mark.parametrize("grid", GRIDS)
def test_yinv_bulk_timeout_waits_cover_the_copies_in_flight(n, grid):
    ntiles = TILES[n]
    for block in sorted({0, 1, grid // 2, grid - 1}):
        yinv_bulk_schedule(block, grid, ntiles)


@pytest.mark.parametrize("n", sorted(TILES))
@pytest.mark.parametrize("grid", GRIDS)
def test_yfwd_timeout_waits_cover_the_copies_in_flight(n, grid):
    ntiles = TILES[n]
    for block in sorted({0, 1, grid // 2, grid - 1}):
        yfwd_schedule(block, grid, ntiles)


def test_the_model_catches_the_stale_parity():
    """The earlier handler of k_yinv_bulk waited on slot 0 with parity it & 1 after slot 1 ran
    late, although slot 0 was already re-staged (phase it + 1): the model rejects it."""
    bars = [Barrier(), Barrier()]
    bars[0].staged, bars[1].staged = 1, 1
    check_wait(bars[0], 0)
    bars[0].staged += 1  # re-staged for the next tile
    with pytest.raises(AssertionError):
        check_handler(bars, 1, [(1, 0), (0, 0)])
