"""The Markstein sequences of the candidate kernel's exact numerics
(shade_device.cuh: correctly rounded square root, reciprocal and division
from the hardware's approximate reciprocal and reciprocal square root and one
fused-multiply-add correction, P. Markstein, IBM J. Res. Dev. 34(1), 1990)
checked against CUDA's correctly rounded intrinsics on every input they
receive: every positive normal float for the square root and the reciprocal
square root, every float in [2^-126, 2^126) for the reciprocal, every divisor
in [2, 16) for the edge integral's division (with eight numerators each in
[0.5, 2); Markstein's theorem makes the quotient correctly rounded for every
numerator once the reciprocal is), and 2^28 random quotients with operands
of magnitude 2^-60 to 2^60 for the reservoir replay's divisions.  Exact numerics uses them only where this
test shows them bit-identical; everything else keeps the intrinsics."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def compile_check(out_dir):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    so = os.path.join(out_dir, "libieee_check.so")
    subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "--fmad=false",
                    "-prec-div=true", "-prec-sqrt=true", "-Xcompiler", "-fPIC", "-shared", "-I",
                    os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cuda", "ieee_check.cu"), "-o", so],
                   check=True)
    return so


def test_check_compiles_for_sm103a(tmp_path):
    assert os.path.getsize(compile_check(str(tmp_path))) > 0


@pytest.mark.gpu
def test_markstein_sequences_equal_the_intrinsics_on_every_input(gpu, tmp_path):
    lib = ctypes.CDLL(compile_check(str(tmp_path)))
    counts = np.zeros(7, np.uint64)
    assert lib.risltc_test_markstein(ctypes.c_void_p(counts.ctypes.data)) == 0
    print("sqrt %d, rcp %d, rsqrt %d, rcp[2,16) %d, div %d of %d, wide div %d" % tuple(int(c) for c in counts))
    assert counts[5] == 8 * (0x41800000 - 0x40000000)
    assert list(counts[:5]) == [0, 0, 0, 0, 0] and counts[6] == 0
