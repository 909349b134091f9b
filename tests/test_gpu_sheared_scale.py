"""The step on sheared Lees-Edwards lattices and at the workloads' own
sizes, through the C-ABI against the oracle's STEPPER_Stokesian.

Sheared cases: configurations valid at strain T (configs.sheared_packing:
every surface gap in the sheared minimum image is at least g_min) at
T = 0.37, 0.5, 0.81 and 0.97 (skew = T for shear rate 1), where
CALC_LATTICE_INVERSE (csd_post.f90:158-183) gives NR = NI = 4, 4, 5 and 5
instead of 3 at zero strain, so the image sums of Ewald_summation.f90:
241-412 run over the larger cubes; the mixed form rebuilds its own image
sets there (lambda scaled, cubes widened, FP32 classification).

Tolerances, relative to the largest entry of each output:
  plain FP64 step: 1e-11 at N = 64 (cond(RPP) <= ~400 in these cases, so
  cond * eps <= 1e-13) and 1e-10 at N = 512 (cond(RPP) ~ 1.5e3);
  positions 1e-12 L;
  mixed form (FP32 factors + FP64 refinement): 1e-8, the bound the mixed
  form is specified to.
"""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

pytestmark = pytest.mark.gpu

MU = o.mu_f_dimensionless(1.0)
SHEARED = [(64, 0.30, 0.01, 0.37, 20262001), (64, 0.30, 0.01, 0.81, 20262002), (64, 0.45, 1e-3, 0.50, 20262003),
           (64, 0.45, 1e-3, 0.97, 20262004)]
EXPECT_NR = {0.37: 4, 0.50: 4, 0.81: 5, 0.97: 5}


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="module")
def tabs(rsd):
    return rsd.LubTab(rsd.lubdat_dir()), o.LubTab(rsd.lubdat_dir())


@pytest.fixture(scope="module")
def oracle_steps(rsd, tabs):
    """The oracle's step on each sheared case, computed once."""
    out = {}
    for N, phi, gmin, T, seed in SHEARED:
        pos, radii, L = rsd.configs.sheared_packing(N, phi, gmin, seed, T, sweeps=20)
        assert rsd.configs.sheared_min_gap(pos, L, T) >= gmin * (1 - 1e-9)
        r = o.stepper_stokesian(pos, radii, [L, L, L], T, 1e-3, 1.0, MU, 1e-10, tabs[1])
        out[T] = (pos, radii, L, r)
    return out


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.mark.parametrize("T", [c[3] for c in SHEARED])
@pytest.mark.parametrize("form", ["fp64", "mixed_scale_1.0", "mixed_scale_1.75"])
def test_sheared_step_matches_oracle(rsd, tabs, oracle_steps, T, form):
    pos, radii, L, r = oracle_steps[T]
    assert (r["lattice"].NR, r["lattice"].NI) == (EXPECT_NR[T], EXPECT_NR[T])
    ctx = rsd.Context(0)
    if form == "fp64":
        prec, tol = rsd.PREC_FP64, 1e-11
    else:
        prec, tol = rsd.PREC_MIXED, 1e-8
        ctx.set_mixed_lambda_scale(float(form.rsplit("_", 1)[1]))
    g = rsd.STEPPER_Stokesian(ctx, tabs[0], pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=prec)
    info = g["info"]
    assert info.info == 0
    if form == "fp64" or form == "mixed_scale_1.0":
        assert (info.NR, info.NI) == (r["lattice"].NR, r["lattice"].NI)
    if prec == rsd.PREC_MIXED:
        assert info.residual <= 1e-12
    assert rel(g["U_pos"], r["U_pos"]) <= tol
    assert rel(g["SijN"], r["SijN_hyd"]) <= tol
    assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=tol, atol=0)
    assert np.abs(g["conf"] - r["conf"]).max() <= 1e-12 * L


def test_sheared_step_unequal_radii(rsd, tabs):
    """Two radii (1 and 0.7) on the lattice of strain 0.81 (NR = NI = 5), with
    lubrication (pairs by s = r / a_avg, hydro_lub.f90:83): both forms
    against the oracle.  Shrinking radii of a packing valid for a = 1 only
    widens its gaps."""
    T = 0.81
    pos, radii, L = rsd.configs.sheared_packing(48, 0.25, 0.01, 20262010, T, sweeps=20)
    radii = np.where(np.random.default_rng(20262010).random(48) < 0.5, 1.0, 0.7)
    r = o.stepper_stokesian(pos, radii, [L, L, L], T, 1e-3, 1.0, MU, 1e-10, tabs[1])
    for prec, tol in ((rsd.PREC_FP64, 1e-11), (rsd.PREC_MIXED, 1e-8)):
        ctx = rsd.Context(0)
        g = rsd.STEPPER_Stokesian(ctx, tabs[0], pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=prec)
        assert g["info"].info == 0
        assert rel(g["U_pos"], r["U_pos"]) <= tol
        assert rel(g["SijN"], r["SijN_hyd"]) <= tol
        assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=tol, atol=0)


def test_plain_trajectory_100_steps(rsd, tabs):
    """The 64-sphere workload (phi = 0.30, gap >= 0.01 a, dt = 1e-3) over its
    100 steps (strain 0 -> 0.1).  Every step of the oracle's trajectory is
    repeated by both forms from the oracle's own configuration, so the
    comparison is step for step.  Along this trajectory a pair closes to a
    gap of 1.4e-4 a at step 18 (cond(RPP) 5.4e3) and overlaps at step 19
    (mirrored lubrication, as in the reference), so the plain form's bound is
    set per step from the oracle's RPP: max(1e-11, 300 cond(RPP) eps) -- the
    oracle inverts RPP explicitly three times (MATREV, Rheology) where this
    library solves with one Cholesky factor, and each carries errors of order
    cond eps sqrt(n) (n = 384); the mixed form keeps 1e-8.
    The plain form also runs its own trajectory beside it: independent
    trajectories separate as near-contact pairs amplify rounding, so their
    positions are held to 1e-9 L after the 100 steps."""
    w = rsd.configs.WORKLOADS[1]
    pos, radii, L = rsd.configs.packing(w["N"], w["phi"], w["g_min"], rsd.configs.SEED_BASE + 1000)
    ctx_p, ctx_m, ctx_t = rsd.Context(0), rsd.Context(0), rsd.Context(0)
    co, ct, T = pos.copy(), pos.copy(), 0.0
    worst = {"fp64": 0.0, "mixed": 0.0}
    for k in range(w["steps"]):
        r = o.stepper_stokesian(co, radii, [L, L, L], T, w["dt"], 1.0, MU, 1e-10, tabs[1])
        gp = rsd.STEPPER_Stokesian(ctx_p, tabs[0], co, radii, T, w["dt"], [L, L, L], 1.0, MU, 1e-10)
        gm = rsd.STEPPER_Stokesian(ctx_m, tabs[0], co, radii, T, w["dt"], [L, L, L], 1.0, MU, 1e-10,
                                   precision=rsd.PREC_MIXED)
        P = 6 * w["N"]
        cond = np.linalg.cond(np.linalg.inv(r["G"])[:P, :P] + r["rfu"])
        tol_p = max(1e-11, 300.0 * cond * np.finfo(float).eps)
        for name, g, tol in (("fp64", gp, tol_p), ("mixed", gm, 1e-8)):
            e = max(rel(g["U_pos"], r["U_pos"]), rel(g["SijN"], r["SijN_hyd"]))
            worst[name] = max(worst[name], e)
            assert e <= tol, (name, k, e)
            assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=tol, atol=0), (name, k)
        assert np.abs(gp["conf"] - r["conf"]).max() <= max(1e-12, tol_p * 1e-3) * L
        ct = rsd.STEPPER_Stokesian(ctx_t, tabs[0], ct, radii, T, w["dt"], [L, L, L], 1.0, MU, 1e-10)["conf"]
        co, T = r["conf"], T + w["dt"]
    drift = np.abs(ct - co).max() / L
    print("100 steps: largest step error fp64 %.2e, mixed %.2e; own-trajectory drift %.2e L"
          % (worst["fp64"], worst["mixed"], drift))
    assert drift <= 1e-9


def test_workload_512_both_forms(rsd, tabs):
    """The 512-sphere workload (phi = 0.45, gap >= 1e-3 a; n = 5632): two steps
    of each form against the oracle, every velocity and stresslet."""
    w = rsd.configs.WORKLOADS[2]
    pos, radii, L = rsd.configs.packing(w["N"], w["phi"], w["g_min"], rsd.configs.SEED_BASE + 2000, sweeps=20)
    ctx_p, ctx_m = rsd.Context(0), rsd.Context(0)
    cp, cm, co, T = pos.copy(), pos.copy(), pos.copy(), 0.0
    for k in range(2):
        r = o.stepper_stokesian(co, radii, [L, L, L], T, w["dt"], 1.0, MU, 1e-10, tabs[1])
        gp = rsd.STEPPER_Stokesian(ctx_p, tabs[0], cp, radii, T, w["dt"], [L, L, L], 1.0, MU, 1e-10)
        gm = rsd.STEPPER_Stokesian(ctx_m, tabs[0], cm, radii, T, w["dt"], [L, L, L], 1.0, MU, 1e-10,
                                   precision=rsd.PREC_MIXED)
        for g, tol in ((gp, 1e-10), (gm, 1e-8)):
            assert g["info"].info == 0
            assert rel(g["U_pos"], r["U_pos"]) <= tol
            assert rel(g["SijN"], r["SijN_hyd"]) <= tol
            assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=tol, atol=0)
        assert gm["info"].residual <= 1e-12
        assert np.abs(gp["conf"] - r["conf"]).max() <= 1e-12 * L
        cp, cm, co, T = gp["conf"], gm["conf"], r["conf"], T + w["dt"]
