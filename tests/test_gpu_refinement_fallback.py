"""The mixed form's refinement when the stationary iteration cannot finish:
the flexible GMRES fallback, the RSD_ENOCONV status when that too misses the
bound, and the driver step's FP64 fallback.  The stationary iteration is cut
short with the step's iteration cap (max_iter), which stands in for a
diverging iteration: both leave the residual above 100 x tol and take the
same path.  32 spheres at strain 0.37 (NR = NI = 4), against the oracle's
step to the mixed form's 1e-8."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

pytestmark = pytest.mark.gpu

MU = o.mu_f_dimensionless(1.0)
T = 0.37


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="module")
def case(rsd):
    pos, radii, L = rsd.configs.sheared_packing(32, 0.3, 0.01, 20262300, T, sweeps=20)
    ref = o.stepper_stokesian(pos, radii, [L, L, L], T, 1e-3, 1.0, MU, 1e-10, o.LubTab(rsd.lubdat_dir()))
    return rsd.LubTab(rsd.lubdat_dir()), pos, radii, L, ref


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def test_stationary_cut_short_falls_back_to_gmres(rsd, case):
    tab, pos, radii, L, ref = case
    ctx = rsd.Context(0)
    g = rsd.STEPPER_Stokesian(ctx, tab, pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=rsd.PREC_MIXED,
                              max_iter=1)
    info = g["info"]
    assert info.fallback == 1 and info.iterations > 1
    assert info.residual <= 1e-10
    assert rel(g["U_pos"], ref["U_pos"]) <= 1e-8
    assert rel(g["SijN"], ref["SijN_hyd"]) <= 1e-8
    # a normal step on the same context takes no fallback
    g = rsd.STEPPER_Stokesian(ctx, tab, pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=rsd.PREC_MIXED)
    assert g["info"].fallback == 0 and g["info"].residual <= 1e-10


def test_unconverged_refinement_is_reported(rsd, case):
    tab, pos, radii, L, ref = case
    ctx = rsd.Context(0)
    ctx.set_refinement(1)  # flexible GMRES alone, one iteration: cannot reach the bound
    with pytest.raises(rsd.RSDError) as e:
        rsd.STEPPER_Stokesian(ctx, tab, pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=rsd.PREC_MIXED,
                              max_iter=1)
    assert e.value.code == rsd.RSD_ENOCONV
    ctx.set_refinement(0)
    g = rsd.STEPPER_Stokesian(ctx, tab, pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=rsd.PREC_MIXED)
    assert rel(g["U_pos"], ref["U_pos"]) <= 1e-8


def test_driver_step_takes_the_fp64_form_when_the_mixed_solve_fails(rsd, case):
    tab, pos, radii, L, ref = case
    ctx = rsd.Context(0)
    ctx.set_refinement(1)
    seen = []
    step = rsd.driver_step(ctx, tab, rsd.PREC_MIXED, fp64_fallback=True, on_fallback=lambda t, why: seen.append(t),
                           max_iter=1)
    out = step(pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10)
    assert seen == [T]
    direct = rsd.STEPPER_Stokesian(rsd.Context(0), tab, pos, radii, T, 1e-3, [L, L, L], 1.0, MU, 1e-10)
    assert rel(out["U_pos"], direct["U_pos"]) <= 1e-13
    assert rel(out["U_pos"], ref["U_pos"]) <= 1e-11
