"""CUDA path against the CPU oracle, through the C-ABI.

Tolerances (stated per test):
  grand mobility / lubrication entries: |gpu - oracle| <= 1e-12 * max|oracle|
  (the plain FP64 form must match the reference routines to 1e-12 relative
  on mobility entries);
  solves, relative to the largest entry of each output, from the condition
  numbers of these cases times FP64 rounding (cond * eps):
    MATREV on X X^T / n + I: cond ~ 5, bound 1e-12;
    the resistance chain and the step on the 27- and 64-sphere packings:
    cond(M) <= 50, cond(RPP) <= 90, so cond * eps <= 2e-14; bound 1e-11."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="module")
def ctx(rsd):
    return rsd.Context(0)


@pytest.fixture(scope="module")
def tabs(rsd):
    return rsd.LubTab(rsd.lubdat_dir()), o.LubTab(rsd.lubdat_dir())


MU = o.mu_f_dimensionless(1.0)


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def sheared_safe_packing(rsd, N, phi, gmin, seed, T, gamma=1.0):
    """Packing whose gaps also hold against the sheared images at strain T."""
    pos, radii, L = rsd.configs.packing(N, phi, gmin, seed)
    lat = o.set_lattice_skew(T, [L, L, L], gamma)
    for i in range(N):
        for j in range(i + 1, N):
            _, d = o.per_skew_correction(lat, pos[i] - pos[j])
            if d < 2 + gmin:
                return None
    return pos, radii, L


@pytest.mark.parametrize("N,phi,T", [(2, 0.05, 0.0), (8, 0.1, 0.0), (8, 0.1, 0.37), (27, 0.2, 0.0),
                                     (27, 0.1, 0.81)])
def test_grand_mobility_matches_oracle(rsd, ctx, N, phi, T):
    for seed in range(20260100, 20260140):
        got = sheared_safe_packing(rsd, N, phi, 0.01, seed, T)
        if got is not None:
            break
    pos, radii, L = got
    lat_g = rsd.SET_LATTICE_SKEW(T, [L, L, L], 1.0)
    APP, APQ, AQQ = rsd.PER_GRPERY_INV_FRI(ctx, pos, radii, lat_g, 1e-10, MU)
    lat_o = o.set_lattice_skew(T, [L, L, L], 1.0)
    G, _ = o.per_grpery_inv_fri(pos, radii, lat_o, 1e-10, MU)
    oPP, oPQ, oQQ = o.split_mobility(G, N)
    scale = np.abs(G).max()
    for a, b in ((APP, oPP), (APQ, oPQ), (AQQ, oQQ)):
        assert np.abs(a - b).max() <= 1e-12 * scale
    assert (lat_g.NR, lat_g.NI) == (lat_o.NR, lat_o.NI)


def test_grand_mobility_config1(rsd, ctx):
    w = rsd.configs.WORKLOADS[1]
    pos, radii, L = rsd.configs.packing(w["N"], w["phi"], w["g_min"], rsd.configs.SEED_BASE + 1000)
    lat_g = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    APP, APQ, AQQ = rsd.PER_GRPERY_INV_FRI(ctx, pos, radii, lat_g, 1e-10, MU)
    G, _ = o.per_grpery_inv_fri(pos, radii, o.set_lattice_skew(0.0, [L, L, L], 1.0), 1e-10, MU)
    N = w["N"]
    M = np.block([[APP, APQ], [APQ.T, AQQ]])
    assert np.abs(M - G).max() <= 1e-12 * np.abs(G).max()
    assert np.abs(G[6 * N:, :6 * N] - APQ.T).max() <= 1e-12 * np.abs(G).max()


def test_grand_mobility_unequal_radii(rsd, ctx):
    rng = np.random.default_rng(3)
    N, L = 10, 14.0
    pos = rsd.configs.packing(N, 0.05, 0.5, seed=20260201)[0] * (L / rsd.configs.box_edge(N, 0.05))
    radii = np.where(rng.random(N) < 0.5, 1.0, 0.6)
    lat_g = rsd.SET_LATTICE_SKEW(0.2, [L, L, L], 1.0)
    APP, APQ, AQQ = rsd.PER_GRPERY_INV_FRI(ctx, pos, radii, lat_g, 1e-10, MU)
    G, _ = o.per_grpery_inv_fri(pos, radii, o.set_lattice_skew(0.2, [L, L, L], 1.0), 1e-10, MU)
    oPP, oPQ, oQQ = o.split_mobility(G, N)
    for a, b in ((APP, oPP), (APQ, oPQ), (AQQ, oQQ)):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(G).max()


def _overlap_case(rsd, ctx, method, T):
    """Pairs whose minimum image overlaps: a partial overlap of unequal
    spheres, a small sphere inside a larger one, and a pair that overlaps
    only across the periodic boundary; correction_method `method` against
    the oracle to 1e-12 of the largest entry."""
    N, L = 10, 9.0
    rng = np.random.default_rng(20261210)
    pos = rsd.configs.packing(N, 0.05, 0.5, seed=20260211)[0] * (L / rsd.configs.box_edge(N, 0.05))
    radii = np.where(rng.random(N) < 0.5, 1.0, 0.6)
    radii[:6] = [1.0, 0.8, 1.0, 0.5, 1.0, 1.0]
    pos[1] = pos[0] + np.array([1.1, 0.4, -0.3])
    pos[3] = pos[2] + np.array([0.2, -0.1, 0.15])
    pos[4] = np.array([0.3, 4.0, 4.0])
    pos[5] = np.array([L - 0.9, 4.2, 4.1])
    pos = np.mod(pos, L)
    lat_g = rsd.SET_LATTICE_SKEW(T, [L, L, L], 1.0)
    APP, APQ, AQQ = rsd.PER_GRPERY_INV_FRI(ctx, pos, radii, lat_g, 1e-10, MU, correction_method=method)
    G, nov = o.per_grpery_inv_fri(pos, radii, o.set_lattice_skew(T, [L, L, L], 1.0), 1e-10, MU,
                                  correction_method=method)
    G0, _ = o.per_grpery_inv_fri(pos, radii, o.set_lattice_skew(T, [L, L, L], 1.0), 1e-10, MU)
    assert nov == 0
    scale = np.abs(G).max()
    assert np.abs(G - G0).max() > 1e-6 * scale  # the corrections are applied
    oPP, oPQ, oQQ = o.split_mobility(G, N)
    for a, b in ((APP, oPP), (APQ, oPQ), (AQQ, oQQ)):
        assert np.abs(a - b).max() <= 1e-12 * scale


@pytest.mark.parametrize("T", [0.0, 0.37])
def test_overlap_correction_matches_oracle(rsd, ctx, T):
    """correction_method 1 (Yamakawa, per_GRPY_YZD.f90:98-116)."""
    _overlap_case(rsd, ctx, 1, T)


def test_grand_mobility_device_variant(rsd, ctx):
    import torch
    pos, radii, L = rsd.configs.packing(27, 0.2, 0.01, seed=20260300)
    lat = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    Md = rsd.per_grpery_inv_fri_dev(ctx, torch.tensor(pos, device="cuda"), torch.tensor(radii, device="cuda"), lat,
                                    1e-10, MU).cpu().numpy()
    G, _ = o.per_grpery_inv_fri(pos, radii, o.set_lattice_skew(0.0, [L, L, L], 1.0), 1e-10, MU)
    assert np.abs(Md - G).max() <= 1e-12 * np.abs(G).max()


@pytest.mark.parametrize("nb", [0, 3])
def test_lubrication_matches_oracle(rsd, ctx, tabs, nb):
    tg, to = tabs
    pos, radii, L = rsd.configs.packing(64, 0.30, 0.01, seed=20261000)
    lat_g = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    lat_o = o.set_lattice_skew(0.0, [L, L, L], 1.0)
    rfu, rfe, rse, nc = rsd.lubmxcalc(ctx, tg, pos, radii, lat_g, MU, nb=nb)
    ofu, ofe, ose, onc = o.lubmxcalc(pos, radii, lat_o, MU, to, nb=nb)
    scale = max(np.abs(ofu).max(), np.abs(ofe).max(), np.abs(ose).max())
    for a, b in ((rfu, ofu), (rfe, ofe), (rse, ose)):
        assert np.abs(a - b).max() <= 1e-12 * scale
    assert nc == onc
    assert np.abs(rfu).max() > 0


def test_lubrication_contact_and_near_contact(rsd, ctx, tabs):
    """A pair at s < 2 (mirrored to 4.00001 - s) and pairs in the asymptotic
    (s < 2.1) and tabulated ranges, non-periodic and periodic."""
    tg, to = tabs
    L = 12.0
    pos = np.array([[1.0, 1.0, 1.0], [2.9995, 1.0, 1.0], [1.0, 3.05, 1.2], [6.0, 6.0, 6.0], [6.0, 6.0, 9.7],
                    [11.5, 6.0, 6.0], [0.7, 6.1, 6.0]])
    radii = np.ones(len(pos))
    for period in (False, True):
        lat_g = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
        lat_o = o.set_lattice_skew(0.0, [L, L, L], 1.0)
        rfu, rfe, rse, nc = rsd.lubmxcalc(ctx, tg, pos, radii, lat_g, MU, is_period=period)
        ofu, ofe, ose, onc = o.lubmxcalc(pos, radii, lat_o, MU, to, is_period=period)
        scale = np.abs(ofu).max()
        for a, b in ((rfu, ofu), (rfe, ofe), (rse, ose)):
            assert np.abs(a - b).max() <= 1e-12 * scale
        assert nc == onc == (2 if period else 1)  # particles 5 and 6 touch only through the boundary


@pytest.mark.parametrize("n", [1, 97, 300, 1031])
def test_matrev_matches_lapack(rsd, ctx, n):
    rng = np.random.default_rng(n)
    X = rng.normal(size=(n, n))
    A = X @ X.T / n + np.eye(n)
    got, info = rsd.MATREV(ctx, A)
    ref, rinfo = o.matrev(A)
    assert info == rinfo == 0
    assert rel(got, ref) <= 1e-12  # cond ~ 5


def test_matrev_reports_not_spd(rsd, ctx):
    A = np.eye(200)
    A[150, 150] = -1.0
    _, info = rsd.MATREV(ctx, A)
    _, rinfo = o.matrev(A)
    assert info == rinfo == 151


def test_cholesky_lower_factor(rsd, ctx):
    rng = np.random.default_rng(5)
    X = rng.normal(size=(250, 250))
    A = X @ X.T + 250 * np.eye(250)
    Lf = rsd.CHOLESKY(ctx, A)
    assert np.allclose(Lf, np.tril(Lf)) and rel(Lf @ Lf.T, A) <= 1e-12
    with pytest.raises(rsd.RSDError):
        rsd.CHOLESKY(ctx, -np.eye(10))


def _small_system(rsd, tabs, N=27, phi=0.2, seed=20260400):
    pos, radii, L = rsd.configs.packing(N, phi, 0.01, seed=seed)
    lat = o.set_lattice_skew(0.0, [L, L, L], 1.0)
    G, _ = o.per_grpery_inv_fri(pos, radii, lat, 1e-10, MU)
    rfu, rfe, rse, _ = o.lubmxcalc(pos, radii, lat, MU, tabs[1])
    return pos, radii, L, G, rfu, rfe, rse


def test_mob_to_resist_and_arrangement(rsd, ctx, tabs):
    pos, radii, L, G, rfu, rfe, rse = _small_system(rsd, tabs)
    N = len(radii)
    APP, APQ, AQQ = o.split_mobility(G, N)
    RPP, RPQ, RQQ, info = rsd.MobToResist_FTS(ctx, APP, APQ, AQQ)
    R0, rinfo = o.mob_to_resist_fts(G)
    assert info == rinfo == 0
    for a, b in ((RPP, R0[:6 * N, :6 * N]), (RPQ, R0[:6 * N, 6 * N:]), (RQQ, R0[6 * N:, 6 * N:])):
        assert rel(a, b) <= 1e-11  # cond(M) ~ 18
    mu, info = rsd.arrangement(ctx, RPP + rfu, RPQ + rfe, RQQ + rse)
    RPPi, _ = o.matrev(R0[:6 * N, :6 * N] + rfu)
    mref = (R0[:6 * N, 6 * N:] + rfe).T @ RPPi @ (R0[:6 * N, 6 * N:] + rfe) - (R0[6 * N:, 6 * N:] + rse)
    assert info == 0 and rel(mu, mref) <= 1e-11  # cond(RPP) ~ 55


def test_stepper_nogmres_matches_oracle(rsd, ctx, tabs):
    pos, radii, L, G, rfu, rfe, rse = _small_system(rsd, tabs)
    N = len(radii)
    rng = np.random.default_rng(11)
    Fe = rng.normal(size=6 * N)
    Fe_inter = rng.normal(size=6 * N) * 0.1
    Eij, _, _ = o.init_u_bg(1.0)
    EIN = o.ein_trans_y2(Eij, N)
    APP, APQ, AQQ = o.split_mobility(G, N)
    got = rsd.STEPPER_NOGmres(ctx, APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN, Fe_inter, pos)
    ref = o.stepper_nogmres(G, rfu, rfe, rse, Fe, EIN, Fe_inter, pos)
    assert got["info"] == 0
    for k in ("U_par", "SijN_hyd", "SijN_FP", "SijN_B", "RPP"):
        assert rel(got[k], ref[k]) <= 1e-11, k  # cond(RPP) ~ 55


@pytest.mark.parametrize("workload", ["small", "config1"])
def test_fused_step_matches_oracle(rsd, ctx, tabs, workload):
    if workload == "small":
        pos, radii, L = rsd.configs.packing(27, 0.2, 0.01, seed=20260500)
        dt, steps = 1e-3, 2
    else:
        w = rsd.configs.WORKLOADS[1]
        pos, radii, L = rsd.configs.packing(w["N"], w["phi"], w["g_min"], rsd.configs.SEED_BASE + 1000)
        dt, steps = w["dt"], 2
    conf_g, conf_o, T = pos.copy(), pos.copy(), 0.0
    for s in range(steps):
        g = rsd.STEPPER_Stokesian(ctx, tabs[0], conf_g, radii, T, dt, [L, L, L], 1.0, MU, 1e-10)
        r = o.stepper_stokesian(conf_o, radii, [L, L, L], T, dt, 1.0, MU, 1e-10, tabs[1])
        assert g["info"].info == 0
        # cond(RPP) ~ 30 (27 spheres) and ~ 90 (64 spheres)
        assert rel(g["U_pos"], r["U_pos"]) <= 1e-11
        assert rel(g["SijN"], r["SijN_hyd"]) <= 1e-11
        assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=1e-11, atol=0)
        assert np.abs(g["conf"] - r["conf"]).max() <= 1e-12 * L
        conf_g, conf_o, T = g["conf"], r["conf"], T + dt


def test_errors_are_reported_not_faulted(rsd, ctx):
    pos, radii, L = rsd.configs.packing(8, 0.1, 0.01, seed=20260600)
    lat = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    bad = pos.copy()
    bad[3, 1] = np.nan
    with pytest.raises(rsd.RSDError) as e:
        rsd.PER_GRPERY_INV_FRI(ctx, bad, radii, lat, 1e-10, MU)
    assert e.value.code == rsd.RSD_ENAN
    over = pos.copy()
    over[1] = over[0] + np.array([1.5, 0, 0])
    with pytest.raises(rsd.RSDError) as e:
        rsd.PER_GRPERY_INV_FRI(ctx, over, radii, lat, 1e-10, MU, correction_method=3)
    assert e.value.code == rsd.RSD_EARG
    with pytest.raises(rsd.RSDError) as e:
        rsd.PER_GRPERY_INV_FRI(ctx, pos, radii, lat, 1e-10, -1.0)
    assert e.value.code == rsd.RSD_EARG


@pytest.mark.parametrize("N,phi,gmin,have_fe", [(27, 0.2, 0.01, False), (64, 0.30, 0.01, True), (64, 0.45, 1e-3, False)])
def test_mixed_step_meets_velocity_tolerance(rsd, ctx, tabs, N, phi, gmin, have_fe):
    """Mixed form (FP32 factors + FP64 refinement): velocities and stresslets
    within 1e-8 relative of the FP64 oracle."""
    pos, radii, L = rsd.configs.packing(N, phi, gmin, seed=20260700 + N, sweeps=20)
    Fe = np.random.default_rng(1).normal(size=6 * N) if have_fe else None
    g = rsd.STEPPER_Stokesian(ctx, tabs[0], pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10, Fe=Fe,
                              precision=rsd.PREC_MIXED)
    r = o.stepper_stokesian(pos, radii, [L, L, L], 0.0, 1e-3, 1.0, MU, 1e-10, tabs[1], Fe=Fe)
    assert g["info"].iterations >= 1 and g["info"].residual <= 1e-12
    assert rel(g["U_pos"], r["U_pos"]) <= 1e-8
    assert rel(g["SijN"], r["SijN_hyd"]) <= 1e-8
    assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=1e-8, atol=0)


@pytest.mark.parametrize("scale,split", [(1.0, (4.0, 1)), (1.5, (4.5, 1)), (2.0, (4.5, 2))])
def test_mixed_step_other_splits(rsd, ctx, tabs, scale, split):
    """The mixed form under another Ewald splitting parameter and near/far
    split (the Ewald sum does not depend on them): same 1e-8 bound."""
    N = 64
    pos, radii, L = rsd.configs.packing(N, 0.30, 0.01, seed=20260800, sweeps=20)
    c2 = rsd.Context(0)  # the settings stay on this context
    c2.set_mixed_lambda_scale(scale)
    c2.set_mixed_split(*split)
    g = rsd.STEPPER_Stokesian(c2, tabs[0], pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10,
                              precision=rsd.PREC_MIXED)
    r = o.stepper_stokesian(pos, radii, [L, L, L], 0.0, 1e-3, 1.0, MU, 1e-10, tabs[1])
    assert rel(g["U_pos"], r["U_pos"]) <= 1e-8
    assert rel(g["SijN"], r["SijN_hyd"]) <= 1e-8
    assert np.allclose(g["yeta_mu"], r["yeta_mu"], rtol=1e-8, atol=0)


def test_mixed_step_unequal_radii(rsd, ctx):
    """Unequal radii take the per-moment reciprocal kernels of the mixed
    assembly (equal radii take the per-vector block weights).  Without
    lubrication, the mixed step against the FP64 step (itself checked
    against the oracle above): velocities and stresslets within 1e-8."""
    N = 48
    pos, _, L = rsd.configs.packing(N, 0.15, 0.3, seed=20260900)
    radii = np.where(np.random.default_rng(5).random(N) < 0.5, 1.0, 0.7)
    out = {}
    for prec in (rsd.PREC_FP64, rsd.PREC_MIXED):
        out[prec] = rsd.STEPPER_Stokesian(ctx, None, pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10,
                                          precision=prec, use_lub=False)
    a, b = out[rsd.PREC_MIXED], out[rsd.PREC_FP64]
    assert rel(a["U_pos"], b["U_pos"]) <= 1e-8
    assert rel(a["SijN"], b["SijN"]) <= 1e-8
