"""The host contact forces (the stand-in for the reference's DEM contact
engine, contact.py): equal and opposite along the line of centres, the
Bossis-Brady exponential outside contact and the linear branch inside,
found through the sheared minimum image, and zero beyond range."""
import importlib.util
import os
import sys
import types

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def mods():
    pkg = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300")
    host = types.ModuleType("rsd_host_c")
    host.__path__ = [pkg]
    sys.modules["rsd_host_c"] = host
    out = {}
    for name in ("configs", "contact"):
        spec = importlib.util.spec_from_file_location("rsd_host_c." + name, os.path.join(pkg, name + ".py"))
        mod = importlib.util.module_from_spec(spec)
        sys.modules["rsd_host_c." + name] = mod
        spec.loader.exec_module(mod)
        out[name] = mod
    return out


def test_pair_force_law(mods):
    C = mods["contact"]
    L = 10.0
    for h in (0.002, 0.03, -0.004):
        pos = np.array([[1.0, 1.0, 1.0], [1.0 + 2.0 + h, 1.0, 1.0]])
        sc = C.SoftContact(2, L, f0=50.0, delta=0.01)
        Fe = sc.forces(pos, 0.0)
        F0 = 50.0 * 6.0
        mag = F0 * np.exp(-h / 0.01) if h >= 0 else F0 * (1 - h / 0.01)
        assert np.allclose(Fe[3:6], [mag, 0, 0]) and np.allclose(Fe[0:3], [-mag, 0, 0])
        assert np.all(Fe[6:] == 0.0)
        assert sc.min_gap == pytest.approx(h)


def test_beyond_range_and_through_the_sheared_image(mods):
    C = mods["contact"]
    L = 10.0
    far = C.SoftContact(2, L, delta=0.01).forces(np.array([[1.0, 1.0, 1.0], [3.2, 1.0, 1.0]]), 0.0)
    assert not far.any()
    # the lattice vector along z carries skew L in x: particle 1 touches
    # particle 0 only through that image, (0, 0, 2.01) away
    skew = 0.3
    p0 = np.array([4.0, 5.0, 5.0])
    p1 = p0 + np.array([0.0, 0.0, 2.01]) - np.array([skew * L, 0.0, L])
    sc = C.SoftContact(2, L, delta=0.01)
    Fe = sc.forces(np.array([p0, p1]), skew)  # strain = skew at shear rate 1
    assert sc.min_gap == pytest.approx(0.01, abs=1e-12)
    assert np.allclose(Fe[3:6], [0.0, 0.0, 6.0 * 100.0 * np.exp(-1.0)])
    assert np.allclose(Fe[0:3], -Fe[3:6])
    # without the skew the nearest image is far away: no force
    assert not C.SoftContact(2, L, delta=0.01).forces(np.array([p0, p1]), 0.0).any()
