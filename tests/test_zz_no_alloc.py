"""The allocation-free grand-mobility entry point, through the C-ABI.

rsd_per_grpery_inv_fri_static is for callers that cannot call cudaMalloc
(a host program whose device memory is all in its own pool, loops that
cannot take cudaMalloc's device synchronisation).  Its only scratch is a
static device array shared by all calls, so this test makes two calls in a
row with different sizes and
lattices -- the second must not see the first one's table -- and compares
each with the allocating entry point rsd_per_grpery_inv_fri_dev, to the
1e-12 relative tolerance of the mobility parity tests.  It also checks that
a request beyond the array's limit is refused with RSD_ELIMIT.  Kept in a
file collected after the parity files so that a first-failure stop has run
them; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rsd():
    ge._load_build_module().build()
    return ge.load_package()


def _static(rsd, pos_t, radii_t, lat, ews, mu, out):
    import torch
    torch.cuda.synchronize()
    N = radii_t.shape[0]
    rc = rsd.library().rsd_per_grpery_inv_fri_static(N, pos_t.data_ptr(), radii_t.data_ptr(), ctypes.byref(lat), ews,
                                                     mu, out.data_ptr(), 11 * N, None)
    torch.cuda.synchronize()
    return rc


def test_static_entry_point_matches_allocating_one_twice(rsd):
    import torch
    ctx = rsd.Context(0)
    mu = rsd.mu_f_dimensionless(1.0)
    cases = [(64, 0.30, 0.01, 0.0, 20261000), (27, 0.10, 0.01, 0.43, 20261001)]
    for N, phi, gmin, T, seed in cases:
        pos, radii, L = rsd.configs.packing(N, phi, gmin, seed=seed)
        pos_t = torch.tensor(pos, dtype=torch.float64, device="cuda")
        radii_t = torch.tensor(radii, dtype=torch.float64, device="cuda")
        lat_a = rsd.SET_LATTICE_SKEW(T, [L, L, L], 1.0)
        ref = rsd.per_grpery_inv_fri_dev(ctx, pos_t, radii_t, lat_a, 1e-10, mu).cpu().numpy()
        lat_s = rsd.SET_LATTICE_SKEW(T, [L, L, L], 1.0)
        out = torch.full((11 * N, 11 * N), float("nan"), dtype=torch.float64, device="cuda")
        assert _static(rsd, pos_t, radii_t, lat_s, 1e-10, mu, out) == rsd.RSD_OK
        got = out.t().cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
        assert (lat_s.NR, lat_s.NI) == (lat_a.NR, lat_a.NI)
        assert abs(lat_s.phi - lat_a.phi) <= 1e-15


def test_static_entry_point_refuses_beyond_its_limit(rsd):
    import torch
    N = 8
    pos, radii, L = rsd.configs.packing(N, 0.1, 0.01, seed=20261002)
    pos_t = torch.tensor(pos, dtype=torch.float64, device="cuda")
    radii_t = torch.tensor(radii, dtype=torch.float64, device="cuda")
    lat = rsd.SET_LATTICE_SKEW(0.0, [L, L, L], 1.0)
    out = torch.zeros((11 * N, 11 * N), dtype=torch.float64, device="cuda")
    # EWS_ERR = 1e-200 asks for NI = 13: 9841 reciprocal vectors in the half space
    assert _static(rsd, pos_t, radii_t, lat, 1e-200, rsd.mu_f_dimensionless(1.0), out) == rsd.RSD_ELIMIT
    assert float(out.abs().max()) == 0.0
