"""Host-side checks that need no GPU: the C-ABI library loads and exports
every entry point include/rsd_capi.h declares; the lattice routines (host
code) match the oracle; inputs are validated; seeded configurations are
deterministic and respect their minimum gap."""
import ctypes
import os
import re

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "rsd_capi.h")).read()
    return sorted(set(re.findall(r"\b(rsd_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported(rsd):
    lib = rsd.library()
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("T", [0.0, 0.13, 0.5, 0.99, 3.7])
def test_lattice_matches_oracle(rsd, T):
    L = 9.632
    radii = np.ones(64)
    a = rsd.SET_LATTICE_SKEW(T, [L, L, L], 1.0)
    rsd.CALC_LATTICE_INVERSE(a, 1e-10, radii)
    b = o.set_lattice_skew(T, [L, L, L], 1.0)
    o.calc_lattice_inverse(b, 1e-10, radii)
    assert np.allclose(a.LR[:], b.LR[:], rtol=0, atol=0)
    assert np.allclose(a.LI[:], b.LI[:], rtol=1e-15, atol=0)
    assert a.LV == b.LV and a.lammda == b.lammda and a.phi == b.phi
    assert (a.NR, a.NI) == (b.NR, b.NI)


def test_zero_strain_images(rsd):
    """Cubic box at zero strain: NR = NI = 3 for EWS_ERR = 1e-10."""
    L = 25.7919
    a = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    rsd.CALC_LATTICE_INVERSE(a, 1e-10, np.ones(2048))
    assert (a.NR, a.NI) == (3, 3)


def test_bad_arguments_are_rejected(rsd):
    lat = rsd.Lattice()
    with pytest.raises(rsd.RSDError):
        rsd.CALC_LATTICE_INVERSE(lat, 1e-10, np.ones(4))  # LV = 0
    with pytest.raises(rsd.RSDError):
        rsd.LubTab("/nonexistent/lubdat")


def test_context_without_gpu_fails_cleanly(rsd):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rsd.RSDError):
        rsd.Context(0)


def test_seeded_packing_deterministic_and_gapped(rsd):
    p1, r1, L1 = rsd.configs.packing(64, 0.30, 0.01, seed=20261000)
    p2, r2, L2 = rsd.configs.packing(64, 0.30, 0.01, seed=20261000)
    assert np.array_equal(p1, p2) and L1 == L2
    assert rsd.configs.min_gap(p1, L1) >= 0.01 - 1e-12
    p3, _, L3 = rsd.configs.packing(128, 0.45, 1e-3, seed=20262000, sweeps=5)
    assert rsd.configs.min_gap(p3, L3) >= 1e-3 - 1e-12


def test_box_edges_match_the_workloads(rsd):
    assert abs(rsd.configs.box_edge(64, 0.30) - 9.6320) < 1e-4
    assert abs(rsd.configs.box_edge(512, 0.45) - 16.8286) < 1e-4
    assert abs(rsd.configs.box_edge(1000, 0.50) - 20.3098) < 1e-4
    assert abs(rsd.configs.box_edge(2048, 0.50) - 25.7919) < 1e-4


def test_new_entry_points_check_their_arguments_without_a_device(rsd):
    """hydro_SD_FTS, DMDX_CAL and the Brownian velocity reject a missing
    context or array with RSD_EARG before any device work."""
    lib = rsd.library()
    z = np.zeros(64)
    p = z.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    info = ctypes.c_int32(0)
    lat = rsd.Lattice()
    assert lib.rsd_hydro_sd_fts(None, 1, p, p, p, p, p, p, p, p, p, p, ctypes.byref(info)) == rsd.RSD_EARG
    assert lib.rsd_hydro_sd_fts(None, 1, p, p, p, p, p, p, p, p, None, p, ctypes.byref(info)) == rsd.RSD_EARG
    assert lib.rsd_dmdx_cal(None, 1, p, p, ctypes.byref(lat), 1e-10, 0.3, 0, p, p) == rsd.RSD_EARG
    assert lib.rsd_brownian_velocity(None, 1, p, p, p, ctypes.byref(lat), 1e-10, 0.3, 0, p, 1.0, 1e-3, p,
                                     ctypes.byref(info)) == rsd.RSD_EARG
