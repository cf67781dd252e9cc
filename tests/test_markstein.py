"""The Markstein sequences of shade_device.cuh (reciprocal, reciprocal
square root and the edge integral's division from the hardware's
approximate reciprocal with one fused-multiply-add correction, P. Markstein,
IBM J. Res. Dev. 34(1), 1990) against CUDA's correctly rounded intrinsics on
every input they can receive: every float in [2^-126, 2^126) for the
reciprocal, every 32-bit pattern for the reciprocal square root, every
divisor in [2, 16) with eight numerators in [0.5, 2) and 2^28 random pairs
in the edge integral's operand box for the division; and the branch-free
square root (the hardware approximation corrected by Tuckerman's test)
against __fsqrt_rn on every float of [2^-76, 2^126], the range the candidate
kernel uses it on.  Exact numerics may use them only because they are
bit-identical there."""
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
    print("rcp %d, rsqrt %d, div %d of %d, edge div %d, sqrt %d, range %d" % tuple(int(c) for c in counts))
    assert counts[3] == 8 * (0x41800000 - 0x40000000)
    assert counts[0] == 0 and counts[1] == 0 and counts[2] == 0 and counts[4] == 0
    assert counts[5] == 0
    # tuckerman_range admits exactly the positive floats of [2^-76, 2^126].
    assert counts[6] == 0x7e800000 - 0x19800000 + 1
