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


def test_autotune_table_picks_the_fastest_setting_per_class(tmp_path):
    """The tuner times each candidate on the largest replica of each size
    class, keeps the fastest in the table (written as JSON), and the
    workers apply that class's setting before each replica's step.  The
    step here is a stand-in whose duration depends on the settings."""
    import json
    import time

    import torch
    E = ensemble_module()

    class Ctx:
        def __init__(self):
            self.tc, self.rp, self.fs = 1, 1, 1
            self.applied = []

        def set_tensor_cores(self, v):
            self.tc = v

        def set_mixed_real_passes(self, v):
            self.rp = v

        def set_factor_schedule(self, v):
            self.fs = v

    def fastest(N):  # the setting the stand-in makes fastest for a replica of N spheres
        return (0, 1, 1) if N < 64 else ((1, 2, 0) if N < 192 else (1, 1, 1))

    class Rsd:
        PREC_MIXED = 1

        @staticmethod
        def stepper_stokesian_dev(ctx, tab, conf, radii, T, dt, LB, gamma, mu, ews, U, S, precision=0):
            N = conf.shape[0]
            ctx.applied.append((N, ctx.tc, ctx.rp, ctx.fs))
            time.sleep(0.001 if (ctx.tc, ctx.rp, ctx.fs) == fastest(N) else 0.006)
            return np.zeros(5), None

        @staticmethod
        def _sync_ctx(ctx):
            pass

    specs = [dict(N=N, phi=0.3, gamma=1.0, seed=k) for k, N in enumerate((40, 60, 100, 150, 200, 250))]
    ens = E.Ensemble.__new__(E.Ensemble)
    ens.rsd, ens.specs, ens.dt, ens.ews, ens.mu = Rsd(), specs, 1e-3, 1e-10, 1.0
    ens.dev = torch.device("cpu")
    ens.conf = [torch.zeros((s["N"], 3)) for s in specs]
    ens.radii = [torch.ones(s["N"]) for s in specs]
    ens.L, ens.T = [10.0] * len(specs), [0.0] * len(specs)
    ens.U = [None] * len(specs)
    ens.S = [None] * len(specs)
    ens.ctx, ens.tab, ens.table = [Ctx()], [None], {}
    path = tmp_path / "table.json"
    table = ens.autotune(str(path), reps=2)
    assert json.loads(path.read_text()) == json.loads(json.dumps(table))
    for k, N in ((0, 60), (1, 100), (2, 150), (3, 250)):  # each class is timed on its largest replica
        t = table[str(k)]
        assert t["N"] == N and (t["tensor_cores"], t["real_passes"], t["factor_schedule"]) == fastest(N)
    # every candidate was tried on every class
    tried = {(n, tc, rp, fs) for n, tc, rp, fs in ens.ctx[0].applied}
    assert all((60, c["tensor_cores"], c["real_passes"], c["factor_schedule"]) in tried for c in E.CANDIDATES)
    # the workers apply each replica's class setting
    ctx = Ctx()
    for N in (40, 150, 250):
        ens._settings(ctx, N)
        assert (ctx.tc, ctx.rp, ctx.fs) == fastest(N)
