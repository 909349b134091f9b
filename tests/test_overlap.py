"""Overlap corrections of the grand mobility (per_GRPY_YZD.f90:98-116):
method 1, overlap_Yamakawa_CORRECTION_IJ (GRPY_YZD.f90:789-811), and method
2, overlap_Regular_CORRECTION_IJ (813-836, Regularization.f90).  The
oracle's restatements are checked by limits of the formulas, and the device
code (csrc/overlap.cuh with the generated csrc/overlap_gen.cuh, built for
the host with g++) against the oracle.  No GPU needed.  (gen_overlap.py
itself checks the regularized potential's derivative tensors against
sympy's derivatives when it generates the header.)

Two properties of the reference's formulas, asserted here as they are:
  - stokesian_Green.f90's free-space pair (ROTNE_PRAGER_IJ_FTS) differs
    from the unscreened Ewald chain in the sign of one term of the fourth
    derivative (Init_DDD2_Jg), which changes its QQ and H blocks;
  - Yamakawa's TD and RD forms (GRPY_YZD.f90:512-640) meet the free-space
    G and H at contact with the opposite sign (YAMAKAWA_IJ passes R where
    the TR block uses -R and a transpose).
TT, RR, TR and QQ of the Yamakawa forms meet the Ewald-chain free-space
pair at contact."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as o
from tests.test_generated_forms import unpack

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "cpp", "overlap_check.cpp")
NAMES = ["TT", "RR", "TR", "QQ", "G", "H"]
RADII = [(1.0, 1.0), (1.0, 0.6), (0.5, 1.4)]


@pytest.fixture(scope="module")
def ovl(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("ovl") / "overlap_check.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, "-o", out, SRC])
    return ctypes.CDLL(out)


def free_space_lattice():
    lat = o.Lattice()
    lat.lammda, lat.NR, lat.NI, lat.phi, lat.LV = 0.0, 0, 0, 0.0, 1.0
    return lat


def d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def call60(fn, R, ai, aj, method=None):
    out = np.zeros(60)
    if method is None:
        fn(d(R), ctypes.c_double(ai), ctypes.c_double(aj), d(out))
    else:
        fn(ctypes.c_int(method), d(R), ctypes.c_double(ai), ctypes.c_double(aj), d(out))
    return unpack(out)


def unit(rng):
    u = rng.normal(size=3)
    return u / np.linalg.norm(u)


@pytest.mark.parametrize("ai,aj", RADII)
def test_yamakawa_meets_free_space_pair_at_contact(ai, aj):
    rng = np.random.default_rng(11)
    lat = free_space_lattice()
    for _ in range(3):
        R = unit(rng) * (ai + aj)
        Y = o.yamakawa_ij(R, ai, aj)
        F = o.per_rotne_prager_ij(lat, R, ai, aj, include_k=False)
        for name, y, f in zip(NAMES, Y, F):
            scale = np.abs(f).max()
            want = -f if name in ("G", "H") else f
            assert np.abs(y - want).max() <= 1e-13 * scale, name


@pytest.mark.parametrize("ai,aj", [(1.0, 0.6), (0.5, 1.4)])
def test_yamakawa_inside_the_larger_sphere(ai, aj):
    """Fully inside (r <= |a_i - a_j|): the larger sphere's single-sphere
    translation and rotation mobilities, no rotation-stresslet coupling."""
    abig = max(ai, aj)
    R = np.array([0.1, -0.2, 0.15]) * (abig - min(ai, aj))
    TT, RR, TR, QQ, G, H = o.yamakawa_ij(R, ai, aj)
    assert np.allclose(TT, np.eye(3) / (6 * abig), rtol=0, atol=1e-15)
    assert np.allclose(RR, np.eye(3) / (8 * abig ** 3), rtol=0, atol=1e-15)
    assert np.all(H == 0)
    if ai > aj:
        assert np.all(G == 0)


def test_free_space_pair_of_the_green_chain():
    """ROTNE_PRAGER_IJ_FTS differs from the Ewald-chain free-space pair only
    in QQ and H (the sign of one fourth-derivative term)."""
    lat = free_space_lattice()
    rng = np.random.default_rng(12)
    for ai, aj in RADII:
        R = unit(rng) * 1.3 * (ai + aj)
        Gr = o.rotne_prager_ij_fts(R, ai, aj)
        F = o.per_rotne_prager_ij(lat, R, ai, aj, include_k=False)
        for name, g, f in zip(NAMES, Gr, F):
            scale = np.abs(f).max()
            if name in ("QQ", "H"):
                assert np.abs(g - f).max() > 1e-3 * scale, name
            else:
                assert np.abs(g - f).max() <= 1e-14 * scale, name


@pytest.mark.parametrize("ai,aj", RADII)
def test_regular_pair_tends_to_free_space_at_contact(ai, aj):
    """kapa = sqrt(pi)/3/|a_I + a_J - r| grows without bound at contact,
    where the regularized pair becomes the unscreened (Ewald-chain) one."""
    rng = np.random.default_rng(14)
    lat = free_space_lattice()
    for f in (1 - 1e-3, 1 - 1e-6):
        R = unit(rng) * (ai + aj) * f
        Rg = o.regular_rotne_prager_ij(R, ai, aj)
        F = o.per_rotne_prager_ij(lat, R, ai, aj, include_k=False)
        for name, g, fr in zip(NAMES, Rg, F):
            assert np.abs(g - fr).max() <= 1e-13 * np.abs(fr).max(), name


@pytest.mark.parametrize("ai,aj", RADII)
def test_device_regular_pair_matches_oracle(ovl, ai, aj):
    """The generated regularized pair (overlap_gen.cuh) against the oracle's
    restatement of Regular_ROTNE_PRAGER_IJ, where erf(kapa r) and its
    derivatives matter (kapa r of order 1).  The blocks come out of
    cancelling terms of the size of the unscreened pair at the same
    separation, so the bound, 1e-12, is relative to that pair."""
    rng = np.random.default_rng(int(100 * ai + 10 * aj) + 1)
    for sep in list(rng.uniform(0.05, 0.95, 30) * (ai + aj)):
        R = unit(rng) * sep
        ref = o.regular_rotne_prager_ij(R, ai, aj)
        got = call60(ovl.ovl_regular60, R, ai, aj)
        fs = o.rotne_prager_ij_fts(R, ai, aj)
        for name, a, b, f in zip(NAMES, ref, got, fs):
            assert np.abs(a - b).max() <= 1e-12 * max(np.abs(a).max(), np.abs(f).max()), (name, sep)


@pytest.mark.parametrize("method", [1, 2])
@pytest.mark.parametrize("ai,aj", RADII)
def test_device_correction_matches_oracle(ovl, ai, aj, method):
    """overlap.cuh (Yamakawa forms, the generated image at lambda = 0 plus
    the closed-form sign term) against the oracle's Fortran-order
    restatement, over overlapping and fully-inside separations.  The
    correction cancels towards contact and its free-space part grows like
    r^-5 towards r = 0, so the bound, 1e-12, is relative to the largest
    block it is formed from (at r = 0.01 the oracle's full 3 x 3 TR keeps
    ~7e-13 of that scale on its diagonal, which the 60-value form holds as
    exact zeros)."""
    rng = np.random.default_rng(int(100 * ai + 10 * aj))
    seps = list(rng.uniform(0.02, 0.999, 40) * (ai + aj)) + [abs(ai - aj) * 0.5 + 0.01]
    if method == 1:
        seps.append(ai + aj)  # (method 2 is NaN at exact contact, as in the reference)
    for sep in seps:
        R = unit(rng) * sep
        ref = o.overlap_correction_ij(method, R, ai, aj)
        got = call60(ovl.ovl_correction60, R, ai, aj, method)
        yam = o.yamakawa_ij(R, ai, aj) if method == 1 else o.regular_rotne_prager_ij(R, ai, aj)
        fs = o.rotne_prager_ij_fts(R, ai, aj)
        for name, a, b, y, f in zip(NAMES, ref, got, yam, fs):
            scale = max(np.abs(y).max(), np.abs(f).max(), 1e-300)
            assert np.abs(a - b).max() <= 1e-12 * scale, (name, sep)


def test_device_free_space_matches_green_chain(ovl):
    rng = np.random.default_rng(13)
    for ai, aj in RADII:
        for sep in (0.3, 1.0, 1.9):
            R = unit(rng) * sep * (ai + aj)
            ref = o.rotne_prager_ij_fts(R, ai, aj)
            got = call60(ovl.ovl_free_space60, R, ai, aj)
            for name, a, b in zip(NAMES, ref, got):
                assert np.abs(a - b).max() <= 1e-13 * np.abs(a).max(), name


@pytest.mark.parametrize("method", [1, 2])
def test_oracle_assembly_applies_the_correction(method):
    """PER_GRPERY_INV_FRI with correction_method 1 or 2: the overlapping
    pair's blocks move by the correction / (pi mu_f), the others stay; an
    unknown method only counts the overlapping pairs."""
    L, mu = 10.0, o.mu_f_dimensionless(1.0)
    pos = np.array([[1.0, 1.0, 1.0], [2.2, 1.5, 0.6], [6.0, 6.5, 5.0]])
    radii = np.array([1.0, 0.8, 1.0])
    out = {}
    for cm in (0, method, 3):
        lat = o.set_lattice_skew(0.0, [L, L, L], 1.0)
        out[cm] = o.per_grpery_inv_fri(pos, radii, lat, 1e-10, mu, correction_method=cm)
    (G0, n0), (G1, n1), (G2, n2) = out[0], out[method], out[3]
    assert n0 == 0 and n1 == 0 and n2 == 1
    assert np.array_equal(G0, G2)
    N = 3
    rows = lambda p: [3 * p + i for i in range(3)] + [3 * N + 3 * p + i for i in range(3)] + \
        [6 * N + 5 * p + m for m in range(5)]
    diff = G1 - G0
    # only the (0, 1) and (1, 0) pair blocks change
    mask = np.zeros_like(diff, dtype=bool)
    for a, b in ((0, 1), (1, 0)):
        mask[np.ix_(rows(a), rows(b))] = True
    assert np.all(diff[~mask] == 0)
    R = pos[0] - pos[1]
    TT, RR, TR, QQ, Gb, Hb = o.overlap_correction_ij(method, R, radii[0], radii[1])
    s = np.pi * mu
    assert np.allclose(diff[np.ix_(rows(0)[:3], rows(1)[:3])], TT / s, rtol=0, atol=1e-14)
    assert np.allclose(diff[np.ix_(rows(0)[6:], rows(1)[6:])], QQ / s, rtol=0, atol=1e-14)
    assert np.abs(G1 - G1.T).max() <= 1e-14 * np.abs(G1).max()


@pytest.mark.parametrize("a", [1.0, 0.7])
def test_yamakawa_equal_spheres_are_the_published_forms(a):
    """Equal spheres of radius a overlapping at r < 2a: the Rotne-Prager-
    Yamakawa translational and rotational mobilities (in the units of the
    pair kernels, before 1/(pi mu_f)):
      TT = 1/(6a) [(1 - 9r/(32a)) I + 3r/(32a) rr],
      RR = 1/(8a^3) [(1 - 27r/(32a) + 5r^3/(64a^3)) I + (9r/(32a) - 3r^3/(64a^3)) rr]."""
    rng = np.random.default_rng(15)
    for r in (0.1 * a, 0.9 * a, 1.7 * a, 1.999 * a):
        u = unit(rng)
        TT, RR, _, _, _, _ = o.yamakawa_ij(u * r, a, a)
        rr = np.outer(u, u)
        tt = ((1 - 9 * r / (32 * a)) * np.eye(3) + 3 * r / (32 * a) * rr) / (6 * a)
        rot = ((1 - 27 * r / (32 * a) + 5 * r ** 3 / (64 * a ** 3)) * np.eye(3)
               + (9 * r / (32 * a) - 3 * r ** 3 / (64 * a ** 3)) * rr) / (8 * a ** 3)
        assert np.abs(TT - tt).max() <= 1e-15 * np.abs(tt).max()
        assert np.abs(RR - rot).max() <= 1e-14 * np.abs(rot).max()
