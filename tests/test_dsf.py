"""Double-single arithmetic and elementary functions (csrc/dsf.cuh) against
40-digit mpmath, on the host build of the same header.

Tolerances (relative): products/sums and sqrt, 1/x 2e-14 (a handful of
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
