"""Bounded device waits run out without a fault (failure detection on the
GPU): the mixed form's tensor-core GEMMs wait on mbarriers and its
refinement's triangular sweeps wait on per-block counters, each with a
bound.  With the bound set far below what the work needs, the step must
return RSD_ETIMEOUT (a status, not a fault), the kernels must leave the GPU
clean -- tensor memory freed, issued copies and MMAs drained, sweep counters
reset by the next call -- and the next step on the same context, with the
default bounds back, must match the oracle to the mixed form's 1e-8.
N = 256 (order 2816, six 512-blocks), so that the sweeps' tasks wait on
blocks that other CTAs are still publishing."""
import numpy as np
import pytest

import __graft_entry__ as ge
from oracle import oracle as o

pytestmark = pytest.mark.gpu

MU = o.mu_f_dimensionless(1.0)


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.fixture(scope="module")
def case(rsd):
    tg, to = rsd.LubTab(rsd.lubdat_dir()), o.LubTab(rsd.lubdat_dir())
    pos, radii, L = rsd.configs.packing(256, 0.30, 0.01, seed=20262100, sweeps=20)
    ref = o.stepper_stokesian(pos, radii, [L, L, L], 0.0, 1e-3, 1.0, MU, 1e-10, to)
    return tg, pos, radii, L, ref


@pytest.mark.parametrize("which", ["tensor_core_gemm", "triangular_sweeps"])
def test_wait_runs_out_then_context_recovers(rsd, case, which):
    tg, pos, radii, L, ref = case
    ctx = rsd.Context(0)
    if which == "tensor_core_gemm":
        ctx.set_wait_limits(tc_wait_ns=1, tri_spin_polls=0)  # 1 ns: the first TMA load cannot land in time
    else:
        ctx.set_wait_limits(tc_wait_ns=0, tri_spin_polls=1)  # one poll: a sweep's first wait gives up
    for _ in range(2):  # twice: a second timed-out call starts from the first one's state
        with pytest.raises(rsd.RSDError) as e:
            rsd.STEPPER_Stokesian(ctx, tg, pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10,
                                  precision=rsd.PREC_MIXED)
        assert e.value.code == rsd.RSD_ETIMEOUT, str(e.value)
        assert "timed out" in str(e.value)
    ctx.set_wait_limits(0, 0)
    g = rsd.STEPPER_Stokesian(ctx, tg, pos, radii, 0.0, 1e-3, [L, L, L], 1.0, MU, 1e-10, precision=rsd.PREC_MIXED)
    assert g["info"].info == 0 and g["info"].residual <= 1e-12
    assert rel(g["U_pos"], ref["U_pos"]) <= 1e-8
    assert rel(g["SijN"], ref["SijN_hyd"]) <= 1e-8
