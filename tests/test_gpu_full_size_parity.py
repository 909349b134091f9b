"""One step of the benchmarked workload at its full size against the oracle:
N = 2048, phi = 0.5, minimum gap 1e-4 a, at strain 0.1 (NR = NI = 3), both
precision forms through the C-ABI against the oracle's STEPPER_Stokesian.
The oracle's step at this size takes a few minutes on a machine's CPU
cores, so the test runs only when RSD_FULL_PARITY=1.

Tolerances, relative to the largest entry of each output: the mixed form
1e-8 (the bound it is specified to); the plain FP64 form 1e-9 (the oracle
inverts RPP explicitly three times where the library solves with one
Cholesky factor, each with errors of order cond(RPP) eps sqrt(n), n = 12288,
and cond(RPP) grows like the inverse of the smallest gap)."""
import os

import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(os.environ.get("RSD_FULL_PARITY") != "1",
                                 reason="full-size oracle step takes minutes: set RSD_FULL_PARITY=1")]

MU = o.mu_f_dimensionless(1.0)


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def test_full_size_step_both_forms():
    ge._load_build_module().build()
    rsd = ge.load_package()
    T = 0.1
    pos, radii, L = rsd.configs.sheared_packing(2048, 0.5, 1e-4, 20262600, T, sweeps=100)
    r = o.stepper_stokesian(pos, radii, [L, L, L], T, 5e-4, 1.0, MU, 1e-10, o.LubTab(rsd.lubdat_dir()))
    tab = rsd.LubTab(rsd.lubdat_dir())
    errs = {}
    for name, prec, tol in (("fp64", rsd.PREC_FP64, 1e-9), ("mixed", rsd.PREC_MIXED, 1e-8)):
        g = rsd.STEPPER_Stokesian(rsd.Context(0), tab, pos, radii, T, 5e-4, [L, L, L], 1.0, MU, 1e-10, precision=prec)
        errs[name] = (rel(g["U_pos"], r["U_pos"]), rel(g["SijN"], r["SijN_hyd"]),
                      abs(g["yeta_mu"][0] - r["yeta_mu"][0]) / abs(r["yeta_mu"][0]))
        assert g["info"].NR == 3 and g["info"].NI == 3
        assert max(errs[name]) <= tol, (name, errs[name])
        assert np.abs(g["conf"] - r["conf"]).max() <= 1e-10 * L
    print("N = 2048 against the oracle (U, S, eta_r):", errs)
