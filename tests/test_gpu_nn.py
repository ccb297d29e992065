"""The NN potential's prediction side on the GPU against the reference's own
calculate_properties (tests/golden/nn_*.npz) and the oracle.

- NeuralNetworkPotential.calculate_properties (so4_contract_dxdr) on the reference's
  descriptors: energies, forces, stress to 1e-11 relative;
- the same from descriptors of the CUDA plain path (FP64) to 1e-9;
- PyXtalFFCalculator, plain route: the reference calculator's result keys, ASE
  stress order and sign; adjoint route (FP32 B and adjoint) to FP32 tolerance;
- so4_contract_dxdr at a larger two-species case against a numpy scatter of the
  same dxdr, bitwise-repeatable, and an asymmetric pair list reported.
"""
import numpy as np
import pytest
import torch

from oracle import nn_properties as NO
from pyxtal_ff_gb300 import engine
from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.ase_calculator import ASE_GPA, ForceField, PyXtalFFCalculator
from pyxtal_ff_gb300.nn import NeuralNetworkPotential
from tests import goldens as G

pytestmark = pytest.mark.gpu


def _ff(meta, nets, drange):
    desc = {"type": meta["kind"], "Rc": meta["rcut"], "cutoff": meta.get("cutoff", "cosine"),
            "parameters": {"lmax": meta["lmax"], "rfac": meta.get("rfac0", 0.99363),
                           "normalize_U": meta.get("normalize_U", False)},
            "weights": meta.get("weights"), "base_potential": None}
    return ForceField(desc, NeuralNetworkPotential(nets, drange))


@pytest.mark.parametrize("name", G.nn_names())
def test_calculate_properties_on_reference_descriptors(cuda_device, name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    pot = NeuralNetworkPotential(nets, drange)
    desc = dict(x=d["x"], dxdr=d["dxdr"], seq=d["seq"], rdxdr=d["rdxdr_atom"], elements=list(atoms.symbols))
    e, f, s = pot.calculate_properties(desc, bforce=True, bstress=True)
    assert G.rel_err(e, d["energies"]) < 1e-12
    assert G.rel_err(f, d["forces"]) < 1e-11
    assert G.rel_err(s, d["stress"]) < 1e-11
    e2, f2, s2 = pot.calculate_properties(desc, bforce=False, bstress=False)
    assert np.array_equal(e2, e) and not f2.any() and not s2.any()


@pytest.mark.parametrize("name", G.nn_names())
def test_calculator_plain_route_matches_reference(cuda_device, name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    calc = PyXtalFFCalculator(ff=_ff(meta, nets, drange))
    en = calc.get_potential_energy(atoms)
    r = calc.results
    assert abs(en - d["energies"].sum()) <= 1e-9 * max(1.0, abs(d["energies"].sum()))
    assert G.rel_err(r["energies"], d["energies"]) < 1e-9
    assert G.rel_err(calc.get_forces(atoms), d["forces"]) < 1e-9
    assert G.rel_err(r["stress_ml"], d["stress"]) < 1e-9
    expect = -(d["stress"] * ASE_GPA)[[0, 1, 2, 5, 4, 3]]
    assert G.rel_err(calc.get_stress(atoms), expect) < 1e-9
    for k in ("free_energy", "energy_ml", "forces_ml", "stress_zbl", "energy_zbl", "forces_zbl"):
        assert k in r
    # unchanged atoms: no recomputation; the 'pyxtal' style keeps GPa in the reference order
    calc2 = PyXtalFFCalculator(style="pyxtal", ff=_ff(meta, nets, drange))
    assert G.rel_err(calc2.get_stress(atoms), d["stress"]) < 1e-9


@pytest.mark.parametrize("name", ["nn_si16_snap", "nn_si432_snap"])
def test_calculator_adjoint_route(cuda_device, name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    calc = PyXtalFFCalculator(ff=_ff(meta, nets, drange), route="adjoint")
    calc.calculate(atoms)
    r = calc.results
    assert G.rel_err(r["energies"], d["energies"]) < 1e-5
    assert G.rel_err(r["forces"], d["forces"]) < 1e-4
    assert G.rel_err(r["stress_ml"], d["stress"]) < 1e-4


def test_calculator_adjoint_route_md_loop_replays_graph(cuda_device):
    """Repeated calls on one layout (an MD loop) replay a captured step; every step equals
    a fresh calculator's uncaptured result bit for bit."""
    atoms, meta, d, nets, drange = G.load_nn("nn_si16_snap")
    calc = PyXtalFFCalculator(ff=_ff(meta, nets, drange), route="adjoint")
    base = atoms.positions.copy()
    rng = np.random.default_rng(3)
    for _ in range(4):
        atoms.positions = base + rng.normal(0, 0.01, size=base.shape)
        calc.calculate(atoms)
        ref = PyXtalFFCalculator(ff=calc.parameters["ff"], route="adjoint")
        ref.calculate(atoms)
        for k in ("energies", "energy", "forces", "stress"):
            assert np.array_equal(calc.results[k], ref.results[k]), k
    assert calc._step is not None


def test_contract_dxdr_large_two_species(cuda_device):
    from pyxtal_ff_gb300.calculator import Batch, SO4Calculator
    structs = [S.sio2_random(n_si=150, seed=7), S.diamond_si(2, 2, 3, sigma=0.1, rng=np.random.default_rng(8))]
    batch = Batch(structs)
    calc = SO4Calculator(lmax=2, rcut=4.5, kind="SNAP", weights={"Si": 1.0, "O": 0.6}, rfac0=0.99363)
    dsc = calc.descriptors(batch)
    nb = dsc["neighbors"]
    rda = engine.rdxdr_atom(dsc["rdxdr"], nb.pair_ptr, nb.natoms)
    beta = torch.from_numpy(np.random.default_rng(9).normal(size=tuple(dsc["x"].shape))).cuda()
    f1, s1 = engine.contract_dxdr(beta, nb.pair_ptr, nb.seq, nb.atom_struct, nb.atom_ptr_dev, dxdr=dsc["dxdr"],
                                  rdxdr_atom=rda)
    f2, s2 = engine.contract_dxdr(beta, nb.pair_ptr, nb.seq, nb.atom_struct, nb.atom_ptr_dev, dxdr=dsc["dxdr"],
                                  rdxdr_atom=rda)
    assert torch.equal(f1, f2) and torch.equal(s1, s2)
    # numpy scatter of the same arrays
    seq = nb.seq.cpu().numpy()
    pp = nb.pair_ptr.cpu().numpy()
    centre = np.repeat(np.arange(nb.natoms), np.diff(pp))
    base = batch.atom_ptr[:-1][np.repeat(np.arange(batch.nstruct), np.diff(batch.atom_ptr))]
    j = seq[:, 1] + base[centre]
    b = beta.cpu().numpy()
    contrib = np.einsum("pk,pkc->pc", b[centre], dsc["dxdr"].cpu().numpy())
    fr = np.zeros((nb.natoms, 3))
    np.add.at(fr, j, -contrib)
    sa = -np.einsum("ik,ikv->iv", b, rda.cpu().numpy())
    sr = np.stack([sa[batch.atom_ptr[s]:batch.atom_ptr[s + 1]].sum(0) for s in range(batch.nstruct)])
    assert G.rel_err(f1.cpu().numpy(), fr) < 1e-12
    assert G.rel_err(s1.cpu().numpy(), sr) < 1e-12
    # the same through the oracle's dense form for the second structure (single species, small)
    a0, a1 = int(batch.atom_ptr[1]), int(batch.atom_ptr[2])
    p0, p1 = int(pp[a0]), int(pp[a1])
    sub = dict(x=dsc["x"][a0:a1].cpu().numpy(), dxdr=dsc["dxdr"][p0:p1].cpu().numpy(), seq=seq[p0:p1].copy(),
               rdxdr=rda[a0:a1].cpu().numpy(), elements=["Si"] * (a1 - a0))
    lin = torch.nn.Sequential(torch.nn.Linear(dsc["x"].shape[1], 1)).double()
    dr = {"Si": np.stack([np.zeros(dsc["x"].shape[1]), np.ones(dsc["x"].shape[1])], 1)}
    eo, fo, so = NO.calculate_properties({"Si": lin}, dr, ["Si"], sub, bforce=True, bstress=True)
    pot = NeuralNetworkPotential({"Si": lin}, dr)
    eg, fg, sg = pot.calculate_properties(sub, bforce=True, bstress=True)
    assert G.rel_err(eg, eo) < 1e-13 and G.rel_err(fg, fo) < 1e-12 and G.rel_err(sg, so) < 1e-12


def test_contract_dxdr_reports_asymmetric_pairs(cuda_device):
    atoms, meta, d, nets, drange = G.load_nn("nn_si16_snap")
    seq = d["seq"].copy()
    # drop one off-diagonal pair: its reverse pair then has no partner
    k = int(np.nonzero(seq[:, 0] != seq[:, 1])[0][3])
    keep = np.ones(len(seq), bool)
    keep[k] = False
    pot = NeuralNetworkPotential(nets, drange)
    desc = dict(x=d["x"], dxdr=d["dxdr"][keep], seq=seq[keep], rdxdr=d["rdxdr_atom"], elements=list(atoms.symbols))
    with pytest.raises(ValueError):
        pot.calculate_properties(desc, bforce=True, bstress=False)
