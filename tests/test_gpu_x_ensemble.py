"""The ensemble of uneven replicas (ensemble.py) on the GPU: eight replicas
drawn from the ensemble workload's distribution (N up to 96 here, so that
the oracle keeps up), each with its own volume fraction and shear rate,
stepped twice by concurrent workers; every replica's velocities and
stresslets after each step against the oracle's single-system
STEPPER_Stokesian from the same state, to the mixed form's 1e-8; and the
autotuner's table (one setting per size class present)."""
import json

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


def test_ensemble_replicas_match_the_oracle(rsd, tmp_path):
    E = rsd.ensemble
    specs = E.replica_specs(8, 20263100, n_range=(32, 96))
    packs = [rsd.configs.packing(s["N"], s["phi"], 1e-3, s["seed"], sweeps=20) for s in specs]
    ens = E.Ensemble(rsd, specs, packs, dt=1e-3, workers=3)
    table = ens.autotune(str(tmp_path / "table.json"))
    assert json.load(open(tmp_path / "table.json")) == table
    assert set(table) == {str(E.size_class(s["N"])) for s in specs}
    for k, v in table.items():
        assert {k: v[k] for k in E.CANDIDATES[0]} in E.CANDIDATES
    tab = o.LubTab(rsd.lubdat_dir())
    for step in range(2):
        before = [c.cpu().numpy().copy() for c in ens.conf]
        T0 = list(ens.T)
        ens.run(1)
        for r, s in enumerate(specs):
            L = ens.L[r]
            ref = o.stepper_stokesian(before[r], packs[r][1], [L, L, L], T0[r], 1e-3, s["gamma"], MU, 1e-10, tab)
            assert rel(ens.U[r].cpu().numpy(), ref["U_pos"]) <= 1e-8, (step, r, s)
            assert rel(ens.S[r].cpu().numpy(), ref["SijN_hyd"]) <= 1e-8, (step, r, s)
            assert np.abs(ens.conf[r].cpu().numpy() - ref["conf"]).max() <= 1e-10 * L
            assert abs(ens.yeta[r][0] - ref["yeta_mu"][0]) <= 1e-8 * abs(ref["yeta_mu"][0])
