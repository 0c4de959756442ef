"""Data-driven Gaussian centres on the GPU (glia_phi_data_centers, Phi::setGaussians(Vec data),
src/mat/Phi.cpp:615-1004) against the FP64 oracle's restatement: the same centres in the same
order and the same tumour-fraction field, exactly (integer counts, FP64 threshold test), for
both precisions and both pointer modes."""
import math

import numpy as np
import pytest

from glia_gb300 import _abi
from tests.gpu_common import FP64, MIXED, gpu, orc
from tests.test_preprocess import _blobs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [FP64, MIXED])
@pytest.mark.parametrize("n,r_vox,frac,sf", [(64, 1.0, 0.0, 2.0), (64, 2.5, 0.15, 2.0),
                                             (128, 2.0, 0.05, 2.5)])
def test_gpu_centres_equal_the_oracle(prec, n, r_vox, frac, sf):
    data = _blobs(n, 11).reshape(-1)
    sigma = r_vox * 2 * math.pi / n
    c_o, f_o = orc(n).phi_data_centers(data, sigma, 0.05, frac, sf, with_frac=True)
    g = gpu(n, prec)
    c_g, f_g = g.phi_data_centers(data, sigma, 0.05, frac, sf, with_frac=True)
    assert len(c_o) > 0
    assert np.array_equal(c_g, c_o)
    if prec == FP64:
        assert np.array_equal(f_g, f_o)
    else:
        assert np.allclose(f_g, f_o, rtol=1e-7, atol=0)


def test_gpu_centres_from_device_float32_data():
    """A float32 CUDA tensor as the data: the threshold test runs on its exact FP64 values."""
    import torch

    n = 64
    data = _blobs(n, 13).reshape(-1).astype(np.float32).astype(np.float64)
    sigma = 1.5 * 2 * math.pi / n
    c_o, _ = orc(n).phi_data_centers(data, sigma, 0.05, 0.1)
    g = gpu(n, MIXED)
    g.set_pointer_mode(_abi.GLIA_PTR_DEVICE_F32)
    c_g, _ = g.phi_data_centers(torch.tensor(data, dtype=torch.float32, device="cuda"), sigma,
                                0.05, 0.1)
    assert np.array_equal(c_g, c_o)
