"""netCDF classic reader / writer, label parsing and splitSegmentation (glia_gb300/netcdf.py).

Files are produced by scipy's independent netCDF implementation (CDF-1 and CDF-2) and by our
writer; a seeded synthetic label volume with the reference's atlas label convention
(wm=6, gm=5, vt=7, csf=8, as in its scripts/forward.py) stands in for atlas data."""
import os

import numpy as np
import pytest

from glia_gb300 import netcdf

scipy_io = pytest.importorskip("scipy.io")


def _labels(n=32, seed=0):
    rng = np.random.default_rng(seed)
    seg = rng.choice([0, 5, 6, 7, 8, 1, 2, 4], size=(n, n, n),
                     p=[0.3, 0.25, 0.25, 0.05, 0.05, 0.04, 0.03, 0.03]).astype(np.float64)
    return seg


@pytest.mark.parametrize("version", [1, 2])
@pytest.mark.parametrize("dtype", ["f8", "f4", "i2"])
def test_reads_files_written_by_scipy(tmp_path, version, dtype):
    seg = _labels(16)
    p = os.path.join(tmp_path, "seg.nc")
    f = scipy_io.netcdf_file(p, "w", version=version)
    for d in "xyz":
        f.createDimension(d, 16)
    v = f.createVariable("data", dtype, ("x", "y", "z"))
    v[:] = seg.astype(dtype)
    f.close()
    assert np.array_equal(netcdf.read(p), seg)


def test_writer_round_trip_and_scipy_reads_it(tmp_path):
    rng = np.random.default_rng(1)
    a = rng.standard_normal((8, 12, 16))
    p = os.path.join(tmp_path, "a.nc")
    netcdf.write(p, a)
    assert np.array_equal(netcdf.read(p), a)
    f = scipy_io.netcdf_file(p, "r", mmap=False)
    assert f.version_byte == 2 and int(f._attributes["CDF-5 mode"]) == 0
    assert np.array_equal(np.array(f.variables["data"][:]), a)
    netcdf.write(p, a, single=True)
    assert np.array_equal(netcdf.read(p), a.astype(np.float32).astype(np.float64))


def test_parse_labels():
    assert netcdf.parse_labels("[wm=6,gm=5,vt=7,csf=8]") == [6, 5, 7, 8, -1, -1, -1, -1]
    assert netcdf.parse_labels("[wm=6,gm=5,vt=7,csf=8,ed=2,nec=1,en=4]") == [6, 5, 7, 8, -1, 1, 4, 2]
    assert netcdf.parse_labels("[wm=1,gm=2,vt=3,tc=5]")[:5] == [1, 2, 3, -1, 5]
    # keys are matched verbatim: " gm" is not "gm"
    assert netcdf.parse_labels("[wm=1, gm=2]") == [1, -1, -1, -1, -1, -1, -1, -1]


def test_split_segmentation():
    seg = _labels(16)
    lab = netcdf.parse_labels("[wm=6,gm=5,vt=7,csf=8,ed=2,nec=1,en=4]")
    m = netcdf.split_segmentation(seg, lab, with_tumor=True, with_edema=True)
    assert np.array_equal(m["gm"], (seg == 5).astype(float))
    assert np.array_equal(m["vt"], (seg == 7).astype(float))
    assert np.array_equal(m["csf"], (seg == 8).astype(float))
    tumor = (seg == 1) | (seg == 4)
    assert np.array_equal(m["tu"], tumor.astype(float))
    assert np.array_equal(m["ed"], (seg == 2).astype(float))
    # tumor and edema voxels count as white matter
    assert np.array_equal(m["wm"], ((seg == 6) | tumor | (seg == 2)).astype(float))
    # without the tumor vectors the tumor labels stay unassigned
    m2 = netcdf.split_segmentation(seg, lab)
    assert np.array_equal(m2["wm"], (seg == 6).astype(float)) and "tu" not in m2


@pytest.mark.gpu
def test_gpu_forward_on_an_atlas_file_matches_the_oracle(tmp_path):
    from glia_gb300 import _abi
    from tests.gpu_common import gpu, orc
    from tests.helpers import gaussian_at, rel_l2

    n = 32
    seg = _labels(n, seed=3)
    p = os.path.join(tmp_path, "atlas.nc")
    netcdf.write(p, seg)
    lab = netcdf.parse_labels("[wm=6,gm=5,vt=7,csf=8]")
    out = []
    for ctx in (gpu(n, _abi.GLIA_FP64), orc(n)):
        ctx.set_time(0.01, 4, 2)
        maps = netcdf.load_atlas(ctx, p, lab, smoothing_factor=1.0)
        ctx.set_coefficients(k=0.05, rho=10.0, k_gm_wm=0.2)
        c0 = gaussian_at(n, (np.pi, np.pi, np.pi), 2 * np.pi / 64 * 2)
        out.append((maps, ctx.solve_state(c0)))
    for k in ("wm", "gm", "vt", "csf"):
        assert rel_l2(out[0][0][k], out[1][0][k]) < 1e-12
    assert rel_l2(out[0][1], out[1][1]) < 1e-10
