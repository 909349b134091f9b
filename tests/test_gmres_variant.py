"""The GMRES variant of the FTS solve, hydro_SD_FTS (src/stepper.f90:476-546,
useGMRESmethod), on the CPU: the oracle's restatement of its splitting
iteration and of gmres_mod's GMRES(2) against the direct resistance solve
of STEPPER_NOGmres.

With gaps of 0.05a the residual of the reference's alternation falls by a
constant factor per iteration and then stalls above its stopping bar
(LINERR 1e-2), held there by the inner GMRES tolerance; the reference then
returns the last velocity iterate and leaves SijN unassigned.  That
velocity equals the direct solution to ~1e-11.  With gaps of 0.01a the
alternation does not contract and its last iterate is far from the
solution.  The C-ABI's rsd_hydro_sd_fts returns the direct solution
(tests/test_gpu_parity.py checks it on the GPU)."""
import importlib.util
import os

import numpy as np

from oracle import oracle as o

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LUBDAT = os.path.join(ROOT, "tests", "golden", "lubdat")


def configs():
    spec = importlib.util.spec_from_file_location(
        "rsd_configs", os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "configs.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def shear_ein(N):
    E = np.zeros((3, 3))
    E[0, 1] = E[1, 0] = 0.5
    return o.ein_trans_y2(E, N)


def lubricated_case(N=8, seed=20260301):
    pos, radii, L = configs().packing(N, 0.25, 0.05, seed=seed)
    mu = o.mu_f_dimensionless(1.0)
    G, _ = o.per_grpery_inv_fri(pos, radii, o.set_lattice_skew(0.0, [L, L, L], 1.0), 1e-10, mu)
    rfu, rfe, rse, _ = o.lubmxcalc(pos, radii, o.set_lattice_skew(0.0, [L, L, L], 1.0), mu, o.LubTab(LUBDAT))
    Fe = np.random.default_rng(seed).normal(size=6 * N) * 0.1
    return G, rfu, rfe, rse, Fe, shear_ein(N), N


def test_gmres_restatement_solves_a_system():
    rng = np.random.default_rng(5)
    n = 40
    X = rng.normal(size=(n, n))
    A = X @ X.T / n + np.eye(n)
    b = rng.normal(size=n)
    x, it, res = o.gmres(np.zeros(n), b, A, 1e-12, 200, 2)
    assert it > 0 and res < 1e-12
    assert np.abs(x - np.linalg.solve(A, b)).max() <= 1e-10 * np.abs(x).max()


def test_splitting_iteration_does_not_contract_near_contact():
    """Gaps of 0.01a (27 spheres, phi = 0.2): the alternation does not
    settle and its last velocity iterate is far from the solution."""
    pos, radii, L = configs().packing(27, 0.2, 0.01, seed=20260400)
    mu = o.mu_f_dimensionless(1.0)
    lat = o.set_lattice_skew(0.0, [L, L, L], 1.0)
    G, _ = o.per_grpery_inv_fri(pos, radii, lat, 1e-10, mu)
    rfu, rfe, rse, _ = o.lubmxcalc(pos, radii, lat, mu, o.LubTab(LUBDAT))
    N = 27
    Fe = np.random.default_rng(12).normal(size=6 * N) * 0.1
    EIN = shear_ein(N)
    APP, APQ, AQQ = o.split_mobility(G, N)
    out = o.hydro_sd_fts(APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN)
    direct = o.stepper_nogmres(G, rfu, rfe, rse, Fe, EIN, Fe, np.zeros((N, 3)))
    assert out["iters"] == -1 and out["err"] > 1e-3
    U = direct["U_par"]
    assert np.abs(out["U_Par"] - U).max() > 1e-2 * np.abs(U).max()


def test_splitting_iteration_stalls_at_the_direct_solution():
    G, rfu, rfe, rse, Fe, EIN, N = lubricated_case()
    assert np.abs(rfu).max() > 0  # near pairs present
    APP, APQ, AQQ = o.split_mobility(G, N)
    trace = []
    out = o.hydro_sd_fts(APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN, trace=trace)
    direct = o.stepper_nogmres(G, rfu, rfe, rse, Fe, EIN, Fe, np.zeros((N, 3)))
    # the residual contracts geometrically, then stalls above LINERR 1e-2
    assert all(trace[k + 1] < 0.6 * trace[k] for k in range(10))
    assert out["iters"] == -1 and out["SijN"] is None and 1e-12 <= out["err"] < 1e-9
    U = direct["U_par"]
    assert np.abs(out["U_Par"] - U).max() <= 1e-10 * np.abs(U).max()
