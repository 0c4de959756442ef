"""The reference's pdesolver unit test compiled as C++ against include/glia/shim.hpp (the
reference's class names over the C-ABI) and run on the GPU."""
import os
import subprocess

import pytest

from glia_gb300 import build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_shim_test():
    lib = build.build()
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_pdesolver_shim")
    src = os.path.join(ROOT, "tests", "cpp", "test_pdesolver_shim.cpp")
    libdir = os.path.dirname(lib)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src,
                    "-L", libdir, "-lglia_rd", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("precision", [0, 1])
def test_reference_pdesolver_test_through_cpp_shim(precision):
    exe = compile_shim_test()
    r = subprocess.run([exe, str(precision)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
