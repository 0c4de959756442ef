"""The reference's pdesolver and grad unit tests compiled as C++ against include/glia/shim.hpp
(the reference's class names over the C-ABI) and run on the GPU."""
import os
import subprocess

import pytest

from glia_gb300 import build

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_shim_test(name="test_pdesolver_shim"):
    lib = build.build()
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, name)
    src = os.path.join(ROOT, "tests", "cpp", name + ".cpp")
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


@pytest.mark.parametrize("precision", [0, 1])
def test_reference_grad_test_through_cpp_shim(precision):
    """src/test/grad.cpp:7-80: PdeOperatorsRD::solveState and
    DerivativeOperatorsRD::updateReactionAndDiffusion / evaluateObjective from C++."""
    exe = compile_shim_test("test_grad_shim")
    r = subprocess.run([exe, str(precision)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
