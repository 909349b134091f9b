"""The generated closed forms (csrc/ewald_gen.cuh) against the oracle's
restatement of PER_ROTNE_PRAGER_IJ (src/Ewald_summation.f90:196-423).

The header is compiled for the host (g++) and summed image by image in the
same order as the CUDA kernel, so this checks the symbolic rewrite on its
own, without a GPU.  Tolerance: 1e-12 of the largest entry of each block."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from oracle import oracle as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "csrc")
SRC = os.path.join(ROOT, "tests", "cpp", "gen_check.cpp")


@pytest.fixture(scope="module")
def genlib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("gen") / "libgencheck.so")
    subprocess.check_call(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", CSRC, "-o", out, SRC])
    return ctypes.CDLL(out)


def unpack(v):
    TT = np.zeros((3, 3)); RR = np.zeros((3, 3)); TR = np.zeros((3, 3)); QQ = np.zeros((5, 5))
    sym = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    for q, (i, j) in enumerate(sym):
        TT[i, j] = TT[j, i] = v[q]
        RR[i, j] = RR[j, i] = v[6 + q]
    for q, (i, j) in enumerate([(0, 1), (0, 2), (1, 2)]):
        TR[i, j], TR[j, i] = v[12 + q], -v[12 + q]
    q = 15
    for a in range(5):
        for b in range(a, 5):
            QQ[a, b] = QQ[b, a] = v[q]
            q += 1
    G = np.array(v[30:45]).reshape(3, 5)
    H = np.array(v[45:60]).reshape(3, 5)
    return TT, RR, TR, QQ, G, H


def gen_block(genlib, lat, R, ai, aj, include_k=True):
    out = np.zeros(60)
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    genlib.gen_pair_block(d(R), lat.LR, lat.LI, ctypes.c_double(lat.LV), ctypes.c_double(lat.lammda),
                          ctypes.c_int(lat.NR), ctypes.c_int(lat.NI), ctypes.c_double(ai), ctypes.c_double(aj),
                          ctypes.c_double(1 - 0.2 * lat.phi), ctypes.c_int(int(include_k)), d(out))
    return unpack(out)


@pytest.mark.parametrize("T", [0.0, 0.37])
@pytest.mark.parametrize("radii", [(1.0, 1.0), (1.0, 0.5)])
def test_generated_pair_block_matches_oracle(genlib, T, radii):
    rng = np.random.default_rng(7)
    L = 9.632
    lat = o.set_lattice_skew(T, [L, L, L], 1.0)
    o.calc_lattice_inverse(lat, 1e-10, np.ones(64))
    for _ in range(4):
        R = rng.uniform(-L / 2, L / 2, 3)
        R, _d = o.per_skew_correction(lat, R)
        ref = o.per_rotne_prager_ij(lat, R, radii[0], radii[1], include_k=True)
        got = gen_block(genlib, lat, R, radii[0], radii[1])
        names = ["TT", "RR", "TR", "QQ", "G", "H"]
        for name, a, b in zip(names, (ref[0], ref[1], ref[2], ref[3], ref[4], ref[5]), got):
            scale = max(np.abs(a).max(), 1e-300)
            assert np.abs(a - b).max() <= 1e-12 * scale, (name, np.abs(a - b).max(), scale)


def test_generated_free_space_block_matches_oracle(genlib):
    lat = o.Lattice()
    lat.lammda, lat.NR, lat.NI, lat.phi, lat.LV = 0.0, 0, 0, 0.0, 1.0
    for sep in (2.0001, 2.5, 7.0):
        R = np.array([sep * 0.6, -sep * 0.8, 0.0])
        ref = o.per_rotne_prager_ij(lat, R, 1.0, 1.0, include_k=False)
        got = gen_block(genlib, lat, R, 1.0, 1.0, include_k=False)
        for a, b in zip(ref, got):
            assert np.abs(a - b).max() <= 1e-13 * max(np.abs(a).max(), 1e-300)


@pytest.mark.parametrize("ai,aj", [(1.0, 1.0), (1.0, 0.6), (0.7, 1.3)])
def test_real_epilogue_table_matches_direct(genlib, ai, aj):
    """The table form of the real-space epilogue (coefficients per
    (output, moment) pair, as the equal-radius mixed kernel applies it)
    equals the generated epilogue to rounding."""
    rng = np.random.default_rng(int(100 * ai + 10 * aj))
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    for _ in range(5):
        acc = rng.normal(size=97) * np.exp(rng.uniform(-3, 3, 97))
        direct, table = np.zeros(60), np.zeros(60)
        genlib.gen_real_epilogue_both(d(acc), ctypes.c_double(ai), ctypes.c_double(aj), ctypes.c_double(0.9),
                                      d(direct), d(table))
        assert np.abs(direct - table).max() <= 1e-13 * max(np.abs(direct).max(), 1.0)
        assert np.abs(direct).max() > 0
