"""torch.autograd on the CUDA library: the adjoint gradient against central finite differences
(h = 1e-3, 8 random directions) and the discrete adjoint of the forward map."""
import numpy as np
import pytest
import torch

from glia_gb300 import autograd as ga
from tests.gpu_common import FP64, MIXED, configure, gpu, observation, small_problem

pytestmark = pytest.mark.gpu


def _setup(prec, n=32, nt=6):
    wl, tissue, centers = small_problem(n, nt)
    d1 = observation(wl, tissue, centers)
    g = gpu(n, prec)
    configure(g, wl, tissue, centers)
    g.set_obs_filter(np.ones(n ** 3))
    g.set_pcg(1e-11 if prec == FP64 else 1e-6, 5000, 1, wl.dt)
    x0 = np.concatenate([np.linspace(0.1, 0.9, len(centers)), [wl.kappa, wl.rho]])
    return g, d1, x0, len(centers)


def test_autograd_gradient_matches_central_differences():
    g, d1, x0, np_ = _setup(FP64)
    x = torch.tensor(x0, requires_grad=True)
    ga.rd_objective(x, g, d1).backward()
    grad = x.grad.numpy()
    rng = np.random.default_rng(3)
    h = 1e-3
    for _ in range(8):
        d = rng.standard_normal(x0.size)
        d[np_:] *= 1e-2 * x0[np_:]          # kappa, rho directions on their own scale
        d /= np.linalg.norm(d)
        fd = (g.eval_objective(x0 + h * d, d1) - g.eval_objective(x0 - h * d, d1)) / (2 * h)
        # p block exact (discrete adjoint); kappa/rho are the reference's trapezoid quadrature
        assert abs(fd - grad @ d) <= 1e-4 * abs(fd), (fd, grad @ d)


def test_mixed_autograd_gradient_matches_fp64():
    out = []
    for prec in (FP64, MIXED):
        g, d1, x0, _ = _setup(prec)
        x = torch.tensor(x0, requires_grad=True)
        ga.rd_objective(x, g, d1).backward()
        out.append(x.grad.numpy())
    assert np.linalg.norm(out[1] - out[0]) <= 1e-4 * np.linalg.norm(out[0])


def test_solve_state_backward_on_gpu_is_the_adjoint():
    g, d1, x0, np_ = _setup(FP64)
    n = 32
    rng = np.random.default_rng(0)
    c0 = torch.tensor(g.phi_apply(x0[:np_]), requires_grad=True)
    w = torch.tensor(rng.standard_normal(n ** 3))
    (ga.solve_state(c0, g) * w).sum().backward()
    v = rng.standard_normal(n ** 3) * 1e-2
    h = 1e-4
    cp = g.solve_state(c0.detach().numpy() + h * v)
    cm = g.solve_state(c0.detach().numpy() - h * v)
    assert float(w.numpy() @ ((cp - cm) / (2 * h))) == pytest.approx(float(c0.grad.numpy() @ v),
                                                                     rel=1e-6)


@pytest.mark.parametrize("prec", [FP64, MIXED])
def test_device_path_equals_host_path_bit_for_bit(prec):
    """CUDA-tensor arguments go to the library as device pointers on the caller's stream; the
    results equal those of host float64 buffers exactly (same conversions, same kernels)."""
    g, d1, x0, np_ = _setup(prec)
    n = 32
    rng = np.random.default_rng(5)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        x = torch.tensor(x0, requires_grad=True)
        Jh = ga.rd_objective(x, g, d1)
        Jh.backward()
        gh = x.grad.clone()
        x = torch.tensor(x0, requires_grad=True)
        Jd = ga.rd_objective(x, g, torch.tensor(d1, device="cuda"))
        Jd.backward()
        assert Jh.item() == Jd.item()
        assert torch.equal(gh, x.grad)

        w = torch.tensor(rng.standard_normal(n ** 3))
        c0h = torch.tensor(g.phi_apply(x0[:np_]), requires_grad=True)
        c1h = ga.solve_state(c0h, g)
        (c1h * w).sum().backward()
        c0d = c0h.detach().cuda().requires_grad_()
        c1d = ga.solve_state(c0d, g)
        (c1d * w.cuda()).sum().backward()
        assert torch.equal(c1h, c1d.cpu())
        assert torch.equal(c0h.grad, c0d.grad.cpu())
        if prec == MIXED:  # float32 tensors: no conversion on the way in, exact on the way out
            c1f = ga.solve_state(c0h.detach().to("cuda", torch.float32), g)
            assert c1f.dtype == torch.float32
            assert torch.equal(c1f.cpu(), c1h.detach().to(torch.float32))
    s.synchronize()
    assert g.ptr_mode == 0 and g.stream == 0  # the context's own modes are restored
