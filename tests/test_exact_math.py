"""Exact FP32 helpers of the kernels, checked on the CPU.

The kernels replace IEEE division by dx, dz, dt with a correction-step
quotient and the reference's double-precision boundary mix with an FP32
error-free evaluation (geopvi_gb300/csrc/fwi2d_exact.h).  Both must return
exactly what the reference's C computes; this compiles the same header for
the host (no FMA contraction) and compares bit for bit.
"""
import ctypes
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("exact") / "libexact.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
                    "-o", out, os.path.join(HERE, "exact_harness.cpp")], check=True)
    L = ctypes.CDLL(out)
    L.harness_div_mismatches.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int]
    L.harness_div_mismatches.restype = ctypes.c_longlong
    L.harness_div_fast_binades.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int]
    L.harness_div_fast_binades.restype = ctypes.c_longlong
    L.harness_div2_any.argtypes = [ctypes.c_float]
    L.harness_div2_any.restype = ctypes.c_longlong
    L.harness_div2_fast_binades.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_int]
    L.harness_div2_fast_binades.restype = ctypes.c_longlong
    L.harness_blend_ties.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_uint,
                                     ctypes.POINTER(ctypes.c_longlong)]
    L.harness_blend_ties.restype = ctypes.c_longlong
    L.harness_blend_mismatches.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_uint,
                                           ctypes.POINTER(ctypes.c_longlong)]
    L.harness_blend_mismatches.restype = ctypes.c_longlong
    L.harness_blend_fast.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_uint,
                                     ctypes.POINTER(ctypes.c_longlong)]
    L.harness_blend_fast.restype = ctypes.c_longlong
    return L


@pytest.mark.parametrize("y", [10.0, 12.0, 9.0, 20.0, 1e-3, 2e-3, 8e-4])
def test_division_by_grid_constants_is_correctly_rounded(harness, y):
    assert harness.harness_div_mismatches(y, -105, 105) == 0


@pytest.mark.parametrize("y", [10.0, 12.0, 1e-3, 8e-4, 2.0 ** -20, 2.0 ** 20])
def test_fast_quotient_at_the_ends_of_its_range(harness, y):
    # the fast path's proved range is 2^-100 <= |x| <= 2^100 (binades -100 and 99 are its ends)
    assert harness.harness_div_fast_binades(y, -100, -99) == 0
    assert harness.harness_div_fast_binades(y, 98, 99) == 0


@pytest.mark.parametrize("y", [10.0, 12.0, 1e-3, 8e-4])
def test_two_step_quotient_without_sign_fixup(harness, y):
    """div2_fast: (x/y)/y from two negated quotients, signed zeros included,
    over the ends of its range (2^-80 .. 2^80) and a middle binade."""
    assert harness.harness_div2_fast_binades(y, -80, -80) == 0
    assert harness.harness_div2_fast_binades(y, 0, 0) == 0
    assert harness.harness_div2_fast_binades(y, 79, 79) == 0


@pytest.mark.parametrize("y", [10.0, 12.0, 9.0, 1e-3, 8e-4, 2.0 ** -20, 2.0 ** 20])
def test_two_step_quotient_of_tiny_values(harness, y):
    """div2_any: the inline scaled path for |x| < 2^-80, IEEE below it."""
    assert harness.harness_div2_any(y) == 0


@pytest.mark.parametrize("pml0", [4, 8, 20])
def test_blend_exact_ties(harness, pml0):
    """Weights whose 1 - w has few bits put the sum exactly on float midpoints;
    the FP32 evaluation rounds those half to even itself."""
    ok32 = ctypes.c_longlong(0)
    trials = 20000
    assert harness.harness_blend_ties(pml0, trials, 99 + pml0, ctypes.byref(ok32)) == 0
    assert ok32.value >= 0.999 * pml0 * trials * 0.99  # nearly every nonzero trial settled in FP32


@pytest.mark.parametrize("pml0", [1, 5, 10, 20, 30])
def test_blend_matches_double_formula(harness, pml0):
    fb = ctypes.c_longlong(0)
    assert harness.harness_blend_mismatches(pml0, 20000, 1234 + pml0, ctypes.byref(fb)) == 0


@pytest.mark.parametrize("pml0", [1, 5, 8, 10, 20, 30])
def test_blend_one_fma_path_matches_double_formula(harness, pml0):
    """blend_fast: one FMA where the exponent-spread test proves that the exact sum is a
    double (so the reference's double rounding is a single rounding), the exact FP32 /
    FP64 blend otherwise; bit for bit against the double formula."""
    fast = ctypes.c_longlong(0)
    trials = 40000
    assert harness.harness_blend_fast(pml0, trials, 77 + pml0, ctypes.byref(fast)) == 0
    assert fast.value > 0
