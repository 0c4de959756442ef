"""Bounded device waits (the mbarrier waits of the TMA staging): a wait that nothing satisfies
gives up after its time limit (about one second), records the fault for the host and leaves the
context usable. The wait is on an mbarrier that no copy signals; nothing faults or hangs."""
import numpy as np
import pytest

from glia_gb300 import _abi


@pytest.mark.gpu
def test_bounded_device_wait_times_out_and_context_survives():
    from glia_gb300.context import Context
    from glia_gb300.native import load

    api = load()
    ctx = Context(api, 64, _abi.GLIA_MIXED)
    assert api.selftest_bounded_wait(ctx._h) == _abi.GLIA_OK
    f = np.random.default_rng(0).standard_normal(64 ** 3)
    assert np.isfinite(ctx.apply_d(f)).all()
    ctx.close()
