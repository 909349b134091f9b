"""Host logic of the ensemble (no GPU): the workload's draws, the size
classes, and the largest-first assignment to workers."""
import importlib.util
import os
import sys
import types

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def ensemble_module():
    pkg = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300")
    host = types.ModuleType("rsd_host_e")
    host.__path__ = [pkg]
    sys.modules["rsd_host_e"] = host
    spec = importlib.util.spec_from_file_location("rsd_host_e.ensemble", os.path.join(pkg, "ensemble.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["rsd_host_e.ensemble"] = mod
    spec.loader.exec_module(mod)
    return mod


def test_draws_are_seeded_and_in_range():
    E = ensemble_module()
    a, b = E.replica_specs(256, 123), E.replica_specs(256, 123)
    assert a == b
    N = np.array([s["N"] for s in a])
    phi = np.array([s["phi"] for s in a])
    g = np.array([s["gamma"] for s in a])
    assert N.min() >= 32 and N.max() <= 256 and len(set(N)) > 100
    assert phi.min() >= 0.10 and phi.max() <= 0.50
    assert g.min() >= 0.1 and g.max() <= 10.0 and np.median(np.log(g)) < 1.0
    assert len({s["seed"] for s in a}) == 256


def test_size_classes_cover_the_range():
    E = ensemble_module()
    assert [E.size_class(N) for N in (32, 63, 64, 127, 128, 191, 192, 256)] == [0, 0, 1, 1, 2, 2, 3, 3]


def test_largest_first_assignment_balances_the_load():
    E = ensemble_module()
    costs = [float(c) ** 3 for c in np.random.default_rng(1).integers(32, 257, 256)]
    groups = E.lpt_assign(costs, 16)
    assert sorted(i for g in groups for i in g) == list(range(256))
    loads = [sum(costs[i] for i in g) for g in groups]
    # LPT is within 4/3 of the optimum, and the optimum is at least the mean load
    assert max(loads) <= 4.0 / 3.0 * max(np.mean(loads), max(costs))
