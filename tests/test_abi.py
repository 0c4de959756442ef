"""The C-ABI library builds for sm_103a, loads, and exports every entry point of
include/glia_rd.h (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from glia_gb300 import _abi, build, native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    with open(os.path.join(ROOT, "include", "glia_rd.h")) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(glia_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_table_agree():
    assert header_functions() == sorted(_abi.exported_names("glia_"))


def test_library_builds_and_exports_every_symbol():
    lib = build.build()
    assert os.path.exists(lib)
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(glia_[a-z0-9_]+)\b", out))
    missing = [f for f in header_functions() if f not in exported]
    assert not missing, missing
    api = native.load()
    for name in _abi.SIGNATURES:
        assert callable(getattr(api, name))


def test_build_targets_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_create_without_gpu_reports_no_device():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    api = native.load()
    h = ctypes.c_void_p()
    assert api.create(32, _abi.GLIA_FP64, _abi.GLIA_ENGINE_FUSED, ctypes.byref(h)) == \
        _abi.GLIA_ERR_NO_DEVICE


def test_argument_validation_without_device():
    api = native.load()
    h = ctypes.c_void_p()
    assert api.create(30, 0, 0, ctypes.byref(h)) == _abi.GLIA_ERR_INVALID  # n % 8 != 0
    assert api.create(64, 7, 0, ctypes.byref(h)) == _abi.GLIA_ERR_INVALID
    assert api.set_time(None, 0.1, 1, 2) == _abi.GLIA_ERR_INVALID


def test_phi_mesh_matches_reference_lattice():
    """Phi::phiMesh (src/mat/Phi.cpp:148-234) for odd and even lattices."""
    import numpy as np

    from glia_gb300.context import phi_mesh
    from oracle import oracle

    api, orc_api = native.load(), oracle.load()
    for np_ in (1, 8, 27, 64, 125, 216):
        a = phi_mesh(api, np_, [np.pi, np.pi, np.pi], 2 * np.pi / 64, 1.5)
        b = phi_mesh(orc_api, np_, [np.pi, np.pi, np.pi], 2 * np.pi / 64, 1.5)
        assert np.array_equal(a, b)
        assert len(np.unique(a.round(12), axis=0)) == np_


def test_header_is_plain_c99():
    """The boundary header must compile as C (no C++ types cross the ABI)."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest

        pytest.skip("no C compiler")
    r = subprocess.run([cc, "-x", "c", "-std=c99", "-fsyntax-only", "-Wall", "-Wextra",
                        "-pedantic", "-Werror", os.path.join(ROOT, "include", "glia_rd.h")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_shim_header_compiles():
    """include/glia/shim.hpp (the reference's class names over the C-ABI) compiles as C++17."""
    import shutil
    import subprocess
    import tempfile

    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        import pytest

        pytest.skip("no C++ compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "use_shim.cpp")
        with open(src, "w") as f:
            f.write('#include "glia/shim.hpp"\nint main() { return 0; }\n')
        r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                            "-I", os.path.join(ROOT, "include"), src],
                           capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
