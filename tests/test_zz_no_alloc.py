"""glia_mismatch_f32_noalloc, the entry point for callers that cannot allocate device memory
(graph-capturing callers, fixed-budget allocators, callers without a context), against the data
term that glia_eval_objective computes for the same state. Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from glia_gb300 import _abi, native
from tests.gpu_common import MIXED, configure, gpu, observation, small_problem

pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_noalloc_mismatch_matches_eval_objective_on_two_calls():
    import torch

    n, nt = 32, 4
    wl, tissue, centers = small_problem(n, nt)
    d1 = observation(wl, tissue, centers)
    g = gpu(n, MIXED)
    configure(g, wl, tissue, centers)
    g.set_obs_filter(np.ones(n ** 3))
    x = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    J = g.eval_objective(x, d1)               # beta = 0: J = h^3 / 2 ||c(1) - d||^2
    c1 = g.get_state(nt)
    h3 = (2 * np.pi / n) ** 3

    api = native.load()
    dev = torch.device("cuda")
    c = torch.tensor(c1, dtype=torch.float32, device=dev)
    obs = torch.ones(n ** 3, dtype=torch.float32, device=dev)
    d = torch.tensor(d1, dtype=torch.float32, device=dev)
    pt = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    expect_pt = -(c * obs - d) * obs
    for _ in range(2):  # the shared scratch must be reusable call after call
        out.zero_()
        pt.fill_(float("nan"))
        rc = api.mismatch_f32_noalloc(_p(c), _p(obs), _p(d), _p(pt), n ** 3, _p(out),
                                      ctypes.c_void_p(stream))
        assert rc == _abi.GLIA_OK
        torch.cuda.synchronize()
        assert abs(0.5 * h3 * out.item() - J) <= 1e-6 * abs(J)
        assert torch.allclose(pt, expect_pt, rtol=1e-6, atol=1e-7)

    # inputs beyond the scratch capacity are refused without touching the GPU
    rc = api.mismatch_f32_noalloc(_p(c), _p(obs), _p(d), None, 2 ** 29 + 1, _p(out),
                                  ctypes.c_void_p(stream))
    assert rc == _abi.GLIA_ERR_INVALID


@pytest.mark.parametrize("n", [64, 128])
def test_noalloc_mismatch_over_many_tiles_on_two_calls(n):
    """4 (64^3) and 32 (128^3) tiles of 65536 voxels: the FP64 partials in the shared array, the
    ticket counter, the last-tile combine and the counter reset between calls, against a float64
    sum on the host. The second call gets other inputs, so a stale partial would show."""
    import torch

    api = native.load()
    dev = torch.device("cuda")
    rng = np.random.default_rng(n)
    stream = torch.cuda.current_stream().cuda_stream
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    pt = torch.empty(n ** 3, dtype=torch.float32, device=dev)
    for call in range(2):
        c = rng.uniform(0.0, 1.0, n ** 3).astype(np.float32)
        obs = (rng.uniform(size=n ** 3) > 0.3 * (call + 1)).astype(np.float32)
        d = (rng.uniform(size=n ** 3) > 0.5).astype(np.float32)
        r = c * obs - d                      # float32, as the kernel forms it
        want = float(np.sum(r.astype(np.float64) ** 2))
        tc, to, td = (torch.tensor(a, device=dev) for a in (c, obs, d))
        out.fill_(-1.0)
        pt.fill_(float("nan"))
        rc = api.mismatch_f32_noalloc(_p(tc), _p(to), _p(td), _p(pt), n ** 3, _p(out),
                                      ctypes.c_void_p(stream))
        assert rc == _abi.GLIA_OK
        torch.cuda.synchronize()
        assert abs(out.item() - want) <= 1e-6 * want, (call, out.item(), want)
        assert torch.equal(pt.cpu(), torch.tensor(-(r * obs)))
