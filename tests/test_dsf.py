"""Double-single arithmetic and elementary functions (csrc/dsf.cuh) against
40-digit mpmath, on the host build of the same header.

Tolerances (relative): products/sums and sqrt, 1/x 2e-14; the unnormalised
accumulator (dsacc, renormalised every 4 or 16 steps) 1e-14 of the sum of
the magnitudes added (a handful of
roundings at 2^-48 in the worst case; the median is ~5e-16); exp(y) on [-36, 0] 8e-15 (1 + |y|)
and erfc(x), exp(-x^2) on [0, 6) 1.5e-14 (1 + x^2): exp amplifies the
double-single rounding of its argument by |y| (the near-image Ewald sums use
x = lambda r in (0, 4], where the images near x = 4 weigh ~1e-6 of a block,
so their ~1e-13 relative error is negligible there)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dsf_check.cpp")
INC = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "csrc")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("dsf") / "libdsf_check.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", "-I", INC, SRC,
                           "-o", so])
    L = ctypes.CDLL(so)
    d2 = ctypes.c_double * 2
    L.dsf_check_erfc_gauss.argtypes = [ctypes.c_double, d2]
    L.dsf_check_exp_neg.argtypes = [ctypes.c_double]
    L.dsf_check_exp_neg.restype = ctypes.c_double
    L.dsf_check_sqrt_rcp.argtypes = [ctypes.c_double, d2]
    L.dsf_check_ops.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, d2]
    dp = ctypes.POINTER(ctypes.c_double)
    L.dsf_check_accumulate.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_int]
    L.dsf_check_accumulate.restype = ctypes.c_double
    L.d2 = d2
    return L


def rel(got, want):
    want = mp.mpf(want)
    return float(abs(mp.mpf(got) - want) / abs(want))


def test_erfc_and_gauss(lib):
    mp.mp.dps = 40
    worst_e = worst_g = 0.0
    for x in np.concatenate([np.linspace(1e-3, 5.999, 3001), [0.137, 0.25, 0.5, 1.0, 3.75, 4.0]]):
        out = lib.d2()
        # the device rounds x to a float pair first; compare at that argument
        xs = float(np.float32(x)) + float(np.float32(x - float(np.float32(x))))
        lib.dsf_check_erfc_gauss(x, out)
        worst_e = max(worst_e, rel(out[0], mp.erfc(mp.mpf(xs))) / (1 + xs * xs))
        worst_g = max(worst_g, rel(out[1], mp.exp(-mp.mpf(xs) ** 2)) / (1 + xs * xs))
    assert worst_e <= 1.5e-14, worst_e
    assert worst_g <= 1.5e-14, worst_g


def test_exp_neg(lib):
    mp.mp.dps = 40
    worst = 0.0
    for y in np.linspace(-36.0, 0.0, 4001):
        ys = float(np.float32(y)) + float(np.float32(y - float(np.float32(y))))
        worst = max(worst, rel(lib.dsf_check_exp_neg(y), mp.exp(mp.mpf(ys))) / (1 + abs(ys)))
    assert worst <= 8e-15, worst


def test_sqrt_rcp_and_ops(lib):
    mp.mp.dps = 40
    rng = np.random.default_rng(3)
    ws = wr = wf = wd = 0.0
    for a in np.exp(rng.uniform(-12, 12, 2000)):
        out = lib.d2()
        lib.dsf_check_sqrt_rcp(a, out)
        as_ = float(np.float32(a)) + float(np.float32(a - float(np.float32(a))))
        ws = max(ws, rel(out[0], mp.sqrt(mp.mpf(as_))))
        wr = max(wr, rel(out[1], 1 / mp.mpf(as_)))
    for a, b, c in rng.normal(size=(2000, 3)):
        out = lib.d2()
        lib.dsf_check_ops(a, b, c, out)
        q = lambda v: mp.mpf(float(np.float32(v))) + mp.mpf(float(np.float32(v - float(np.float32(v)))))
        scale = abs(q(a) * q(b)) + abs(q(c))
        wf = max(wf, float(abs(mp.mpf(out[0]) - (q(a) * q(b) + q(c))) / scale))
        wd = max(wd, float(abs(mp.mpf(out[1]) - (q(a) - q(b))) / (abs(q(a)) + abs(q(b)))))
    assert ws <= 2e-14 and wr <= 2e-14, (ws, wr)
    assert wf <= 2e-14 and wd <= 2e-14, (wf, wd)


@pytest.mark.parametrize("every", [4, 16])
@pytest.mark.parametrize("n", [1, 7, 300, 5000])
def test_unnormalised_accumulator(lib, n, every):
    """sum a_i b_i + sum c_i through dsacc renormalised every 4 (the
    near-image sums) or 16 (the reciprocal sums) steps: error below 1e-14 of
    sum |terms|, also when the sum cancels to a small fraction of its
    terms."""
    mp.mp.dps = 50
    rng = np.random.default_rng(11 + n)
    for trial in range(4):
        a = rng.normal(size=n) * np.exp(rng.uniform(-6, 6, n))
        b = rng.normal(size=n)
        c = rng.normal(size=n) * np.exp(rng.uniform(-6, 6, n))
        if trial == 3:  # cancelling sum
            c = -a * b + 1e-9 * rng.normal(size=n)
        q = lambda v: mp.mpf(float(np.float32(v))) + mp.mpf(float(np.float32(v - float(np.float32(v)))))
        terms = [q(x) * q(y) for x, y in zip(a, b)] + [q(z) for z in c]
        exact = mp.fsum(terms)
        scale = mp.fsum(abs(t) for t in terms)
        ptr = lambda v: np.ascontiguousarray(v, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        got = lib.dsf_check_accumulate(n, ptr(a), ptr(b), ptr(c), every)
        assert float(abs(mp.mpf(got) - exact) / scale) <= 1e-14
