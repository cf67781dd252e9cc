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


def _tuckerman_round(s, d):
    """tuckerman_round of shade_device.cuh on float32 arrays: the signs of
    d - s * s+ and d - s * s- are exact in float64 (the products have at most
    48 significant bits and the differences stay within 53)."""
    bits = s.view(np.uint32)
    up = (bits + np.uint32(1)).view(np.float32)
    dn = (bits - np.uint32(1)).view(np.float32)
    d64, s64 = d.astype(np.float64), s.astype(np.float64)
    above = d64 - s64 * up.astype(np.float64) > 0.0
    below = d64 - s64 * dn.astype(np.float64) <= 0.0
    return np.where(above, up, np.where(below, dn, s))


def test_tuckerman_rounding_recovers_the_correctly_rounded_root_from_one_ulp_away():
    # The correction step alone: from the correctly rounded square root or
    # either neighbour (an approximation within one unit in the last place),
    # Tuckerman's test returns the correctly rounded root, across the range
    # [2^-76, 2^126] the candidate kernel uses, binade edges included.
    rng = np.random.default_rng(7)
    lo, hi = 0x19800000, 0x7E800000
    u = rng.integers(lo, hi + 1, 2_000_000, dtype=np.int64).astype(np.uint32)
    edges = np.array([lo, hi] + [(e << 23) + k for e in range(52, 253, 2) for k in (0, 1, 0x7FFFFF)],
                     dtype=np.int64).astype(np.uint32)
    d = np.concatenate([u, edges[(edges >= lo) & (edges <= hi)]]).view(np.float32)
    exact = np.sqrt(d.astype(np.float64)).astype(np.float32)  # RN(sqrt) of a float32 via float64 is exact
    bits = exact.view(np.uint32)
    for off in (-1, 0, 1):
        s = (bits.astype(np.int64) + off).astype(np.uint32).view(np.float32)
        np.testing.assert_array_equal(_tuckerman_round(s, d).view(np.uint32), bits)
