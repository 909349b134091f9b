"""Brownian terms of STEPPER_Stokesian with BROWN (src/stepper.f90:72-86,
664-688) in the oracle, on the CPU: the finite-difference drift DMDX_CAL
and the Brownian velocity for given standard normal numbers Z (the
reference draws them with GAUSS; the C-ABI takes them as input, checked on
the GPU by tests/test_gpu_parity.py)."""
import numpy as np

from oracle import oracle as o
from tests.test_gmres_variant import configs

MU = o.mu_f_dimensionless(1.0)


def dilute(N=8, seed=20260700):
    """A dilute packing and a function returning a fresh lattice of its box
    (the oracle's assembly fills the lattice it is given)."""
    pos, radii, L = configs().packing(N, 0.05, 0.5, seed=seed)
    return pos, radii, L, (lambda: o.set_lattice_skew(0.0, [L, L, L], 1.0))


def test_deta_is_the_single_precision_literal():
    # REAL*8 deta; PARAMETER(deta=0.001): the literal is default real
    assert o.DMDX_DETA == float(np.float32(0.001)) and o.DMDX_DETA != 0.001


def test_dmdx_of_a_single_sphere_is_zero():
    pos, radii, _, lat = dilute(N=1)
    Z = np.random.default_rng(1).normal(size=3)
    assert np.all(o.dmdx_cal(pos, radii, lat, 1e-10, MU, Z) == 0.0)


def test_dmdx_is_quadratic_in_z():
    """(A(x + c deta Z/2) - A(x - c deta Z/2)) c Z / deta = c^2 (dA.Z) Z +
    O(deta^2): halving Z quarters DMDX."""
    pos, radii, _, lat = dilute()
    Z = np.random.default_rng(2).normal(size=3 * len(radii))
    d1 = o.dmdx_cal(pos, radii, lat, 1e-10, MU, Z)
    d2 = o.dmdx_cal(pos, radii, lat, 1e-10, MU, 0.5 * Z)
    assert np.abs(d1).max() > 0
    assert np.abs(4.0 * d2 - d1).max() <= 1e-5 * np.abs(d1).max()


def test_brownian_velocity_of_zero_noise_is_zero():
    pos, radii, _, lat = dilute()
    G, _ = o.per_grpery_inv_fri(pos, radii, lat(), 1e-10, MU)
    u, info = o.brownian_velocity(G[:6 * len(radii), :6 * len(radii)], pos, radii, lat, 1e-10, MU,
                                  np.zeros(3 * len(radii)), 1.0, 1e-3)
    assert info == 0 and np.all(u == 0.0)
