"""The committed generated headers are what their generators write: each
generator is run into a temporary file and compared with the header byte
for byte (ewald_gen.cuh from gen_ewald.py, overlap_gen.cuh from
gen_overlap.py, dsf_tables.cuh from gen_dsf_tables.py).  Needs sympy (and
its mpmath); about a minute."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "regularized-stokesian-dynamics_gb300", "csrc")

pytest.importorskip("sympy")


def load(name):
    if CSRC not in sys.path:
        sys.path.insert(0, CSRC)
    spec = importlib.util.spec_from_file_location(name, os.path.join(CSRC, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("gen,header,entry", [("gen_ewald", "ewald_gen.cuh", "gen"),
                                              ("gen_overlap", "overlap_gen.cuh", "main"),
                                              ("gen_dsf_tables", "dsf_tables.cuh", "main")])
def test_header_matches_its_generator(tmp_path, capsys, gen, header, entry):
    mod = load(gen)
    out = tmp_path / header
    mod.OUT = str(out)
    getattr(mod, entry)()
    assert out.read_bytes() == open(os.path.join(CSRC, header), "rb").read()
