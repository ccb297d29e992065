"""The NN-potential oracle (oracle/nn_properties.py) against the reference's own
calculate_properties outputs (tests/golden/nn_*.npz, tests/golden/make_golden_nn.py)."""
import numpy as np
import pytest

from oracle import nn_properties as NO
from tests import goldens as G


@pytest.mark.parametrize("name", G.nn_names())
def test_oracle_calculate_properties_matches_reference(name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    desc = dict(x=d["x"], dxdr=d["dxdr"], seq=d["seq"], rdxdr=d["rdxdr_atom"], elements=list(atoms.symbols))
    e, f, s = NO.calculate_properties(nets, drange, sorted(nets), desc, bforce=True, bstress=True)
    assert G.rel_err(e, d["energies"]) < 1e-13
    assert G.rel_err(f, d["forces"]) < 1e-12
    assert G.rel_err(s, d["stress"]) < 1e-12


def test_voigt_reduction_matches_fixture():
    # the per-atom rows stored in the fixture are the reference caller's reduction
    atoms, meta, d = G.load("nacl_snap")
    _, _, dn, _, _ = G.load_nn("nn_nacl_snap")
    out = NO.voigt_atom(d["rdxdr"], d["seq"], len(atoms.positions))
    assert np.array_equal(out, dn["rdxdr_atom"])
