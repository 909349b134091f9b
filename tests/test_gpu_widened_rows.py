"""GPU tests of the rows widened last (overlap correction method 2, the
GMRES variant's FTS solve, the Brownian terms, overlap corrections in the
fused step), through the C-ABI against the oracle; tolerances as in
test_gpu_parity.py, stated per test."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o
from tests.test_gpu_parity import MU, _overlap_case, _small_system, rel

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


@pytest.mark.parametrize("T", [0.0, 0.37])
def test_overlap_correction_method_2_matches_oracle(rsd, ctx, T):
    """correction_method 2 (the regularized pair, Regularization.f90) on the
    overlapping pairs of the method-1 case."""
    _overlap_case(rsd, ctx, 2, T)


@pytest.mark.parametrize("case", ["mild", "near_contact"])
def test_hydro_sd_fts_matches_oracle(rsd, ctx, tabs, case):
    """hydro_SD_FTS (the GMRES variant, stepper.f90:476-546) through the
    C-ABI: velocities and stresslets against the direct resistance solve
    (S = mu EIN + RPQ^T RPP^-1 Fe) and, where the reference's splitting
    iteration settles (gaps >= 0.05a), velocities against the oracle's
    restatement of that iteration.  With gaps of 0.01a the iteration does
    not contract and its last iterate is ~14% off (tests/test_gmres_variant
    .py); the C-ABI returns the solution of the equations either way."""
    from tests.test_gmres_variant import lubricated_case
    if case == "mild":
        G, rfu, rfe, rse, Fe, EIN, N = lubricated_case()
    else:
        pos, radii, L, G, rfu, rfe, rse = _small_system(rsd, tabs)
        N = len(radii)
        Fe = np.random.default_rng(12).normal(size=6 * N) * 0.1
        Eij, _, _ = o.init_u_bg(1.0)
        EIN = o.ein_trans_y2(Eij, N)
    APP, APQ, AQQ = o.split_mobility(G, N)
    got = rsd.hydro_SD_FTS(ctx, APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN)
    assert got["info"] == 0
    direct = o.stepper_nogmres(G, rfu, rfe, rse, Fe, EIN, Fe, np.zeros((N, 3)))
    assert rel(got["U_par"], direct["U_par"]) <= 1e-9
    assert rel(got["SijN"], direct["SijN_hyd"] + direct["SijN_FP"]) <= 1e-9
    if case == "mild":
        it = o.hydro_sd_fts(APP, APQ, AQQ, rfu, rfe, rse, Fe, EIN)
        assert rel(got["U_par"], it["U_Par"]) <= 1e-9


def test_brownian_terms_match_oracle(rsd, ctx):
    """DMDX_CAL and the Brownian velocity of STEPPER_Stokesian (stepper.f90:
    72-86, 664-688) for given normal numbers Z.  DMDX divides the difference
    of two assemblies by deta ~ 1e-3, which scales their entry-level
    rounding by 1e3: bound 1e-7 for it, 1e-9 for the velocity (dominated by
    the Cholesky term)."""
    from tests.test_brownian import dilute
    pos, radii, L, lat_fn = dilute()
    N = len(radii)
    Z = np.random.default_rng(21).normal(size=3 * N)
    lat_g = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    d_g = rsd.DMDX_CAL(ctx, pos, radii, lat_g, 1e-10, MU, Z)
    d_o = o.dmdx_cal(pos, radii, lat_fn, 1e-10, MU, Z)
    assert rel(d_g, d_o) <= 1e-7
    G, _ = o.per_grpery_inv_fri(pos, radii, lat_fn(), 1e-10, MU)
    APP = G[:6 * N, :6 * N]
    u_g = rsd.brownian_velocity(ctx, APP, pos, radii, rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0), 1e-10, MU, Z,
                                0.7, 1e-3)
    u_o, info = o.brownian_velocity(APP, pos, radii, lat_fn, 1e-10, MU, Z, 0.7, 1e-3)
    assert info == 0 and rel(u_g, u_o) <= 1e-9


def test_fused_step_with_overlap_correction(rsd, tabs):
    """The fused step with Context.set_correction_method(2): one particle
    moved to r = 1.9a of another (it also touches a third); the FP64 form
    against the oracle's STEPPER_Stokesian with the same correction (1e-9),
    the mixed form against the FP64 form (1e-8).  (Method 1 makes this
    mobility indefinite, as the reference's own formulas do.)"""
    N = 27
    pos, radii, L = rsd.configs.packing(N, 0.2, 0.01, seed=20260500)
    pos[1] = np.mod(pos[0] + np.array([1.9, 0.0, 0.0]), L)
    c = rsd.Context(0)
    c.set_correction_method(2)
    g = rsd.STEPPER_Stokesian(c, tabs[0], pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10)
    r = o.stepper_stokesian(pos, radii, [L, L, L], 0.0, 1e-3, 1.0, MU, 1e-10, tabs[1], correction_method=2)
    assert g["info"].info == 0 and r["info_m"] == 0
    assert rel(g["U_pos"], r["U_pos"]) <= 1e-9
    assert rel(g["SijN"], r["SijN_hyd"]) <= 1e-9
    assert np.abs(g["conf"] - r["conf"]).max() <= 1e-12 * L
    m = rsd.STEPPER_Stokesian(c, tabs[0], pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10,
                              precision=rsd.PREC_MIXED)
    assert rel(m["U_pos"], g["U_pos"]) <= 1e-8 and rel(m["SijN"], g["SijN"]) <= 1e-8
    r0 = o.stepper_stokesian(pos, radii, [L, L, L], 0.0, 1e-3, 1.0, MU, 1e-10, tabs[1])
    assert rel(g["U_pos"], r0["U_pos"]) > 1e-6  # the correction changed the step


def test_driver_loop_on_the_fused_step(rsd, tabs, tmp_path):
    """The driver's time loop (driver.py) over the reference's file formats
    with the fused FP64 step, against the same loop with the oracle's step:
    four steps, positions to 1e-12 of the box."""
    from tests.test_driver_loop import control_for_periodic_fts
    control = control_for_periodic_fts(tmp_path)
    pos, radii, L = rsd.configs.packing(8, 0.2, 0.05, seed=20261100)
    init = str(tmp_path / "initial_config.dat")
    rsd.driver_files.write_initial_config(init, pos, radii, [L, L, L])
    g = rsd.driver.run(control, init, rsd.driver_step(rsd.Context(0), tabs[0], precision=rsd.PREC_FP64),
                       str(tmp_path / "g.VTF"), str(tmp_path / "g_yeta.txt"))

    def ostep(conf, r, T, dt, LB, gamma, mu_f, ews):
        return o.stepper_stokesian(conf, r, LB, T, dt, gamma, mu_f, ews, tabs[1])

    r = rsd.driver.run(control, init, ostep, str(tmp_path / "o.VTF"), str(tmp_path / "o_yeta.txt"))
    assert g["steps"] == r["steps"] == 4
    assert np.abs(g["conf"] - r["conf"]).max() <= 1e-12 * L
