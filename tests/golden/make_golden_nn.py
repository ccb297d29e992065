"""Generate the NN-potential golden vectors (tests/golden/nn_*.npz) by running the
REFERENCE's own ``NeuralNetwork.calculate_properties``
(pyxtal_ff/models/neuralnetwork.py:579-678) on descriptors the reference's SO4/SNAP
code computed.

Runs only where the reference tree is readable; its root must be given in
$PYXTAL_FF_REF.  Besides the descriptor stand-ins of
make_golden.py (numba, ASE, float range), the NN module needs stand-ins for what
this container lacks and calculate_properties never calls: matplotlib (plotting),
``pyxtal_ff.models.optimizers.regressor`` (training) and
``pyxtal_ff.utilities.elements`` (element data).  The NeuralNetwork object is
created without its constructor and given the four attributes calculate_properties
reads -- elements, models, drange, unit -- as a loaded checkpoint gives them
(load_checkpoint, :838-893).

Per case: the descriptor inputs as the reference's caller passes them (x, dxdr,
seq, elements, and rdxdr reduced per atom to Voigt order, utilities/__init__.py:226-233),
the per-element networks (layer sizes, activation names, weights), drange, and the
reference's outputs (energies, forces, stress); and the LAMMPS ML-IAP text files the
reference writes for that potential (NeuralNetwork.save_weights_to_txt, :719-836)
and for a linear potential with random coefficients
(PR.save_weights_to_txt, polynomialregression.py:286-345).

    python tests/golden/make_golden_nn.py
"""
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import make_golden  # noqa: E402
from pyxtal_ff_gb300 import structures as S  # noqa: E402



def _install_nn_stubs():
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    plt = types.ModuleType("matplotlib.pyplot")
    plt.style = types.SimpleNamespace(use=lambda *a, **k: None)
    gs = types.ModuleType("matplotlib.gridspec")
    gs.GridSpec = object
    tk = types.ModuleType("matplotlib.ticker")
    mpl.pyplot, mpl.gridspec, mpl.ticker = plt, gs, tk
    for name, mod in (("matplotlib", mpl), ("matplotlib.pyplot", plt), ("matplotlib.gridspec", gs),
                      ("matplotlib.ticker", tk)):
        sys.modules[name] = mod
    models = types.ModuleType("pyxtal_ff.models")
    models.__path__ = [os.path.join(make_golden.reference_root(), "pyxtal_ff", "models")]
    sys.modules["pyxtal_ff.models"] = models
    opt = types.ModuleType("pyxtal_ff.models.optimizers")
    opt.__path__ = []
    reg = types.ModuleType("pyxtal_ff.models.optimizers.regressor")
    reg.Regressor = object
    sys.modules["pyxtal_ff.models.optimizers"] = opt
    sys.modules["pyxtal_ff.models.optimizers.regressor"] = reg
    util = types.ModuleType("pyxtal_ff.utilities")
    util.__path__ = []
    el = types.ModuleType("pyxtal_ff.utilities.elements")
    el.Element = object
    sys.modules["pyxtal_ff.utilities"] = util
    sys.modules["pyxtal_ff.utilities.elements"] = el


def _voigt_atom(rdxdr, seq, n):
    """Per-pair (P, nB, 3, 3) -> per-atom (n, nB, 6): sum over the pairs of each centre,
    then the entries (0, 4, 8, 1, 2, 5) of the flattened 3x3."""
    out = np.zeros((n, rdxdr.shape[1], 3, 3))
    np.add.at(out, seq[:, 0], rdxdr)
    return out.reshape(n, rdxdr.shape[1], 9)[:, :, [0, 4, 8, 1, 2, 5]]


def _nets(torch, elements, nB, spec, seed):
    """spec: element -> (hidden sizes, activation names incl. the output layer)."""
    torch.manual_seed(seed)
    nets, arch = {}, {}
    for e in elements:
        hidden, acts = spec[e]
        sizes = [nB] + list(hidden) + [1]
        layers = []
        for i, act in enumerate(acts):
            layers.append(torch.nn.Linear(sizes[i], sizes[i + 1]))
            if act != "Linear":
                layers.append(getattr(torch.nn, act)())
        nets[e] = torch.nn.Sequential(*layers).double()
        arch[e] = dict(sizes=sizes, acts=list(acts))
    return nets, arch


def _drange(x, elements, symbols, pad):
    d = {}
    for e in elements:
        xe = x[np.array(symbols) == e]
        lo, hi = xe.min(0), xe.max(0)
        w = np.maximum(hi - lo, 1e-3)
        d[e] = np.stack([lo - pad * w, hi + pad * w], axis=1)
    return d


def _cases():
    nacl = dict(np.load(os.path.join(HERE, "nacl_snap.npz")))
    si16 = dict(np.load(os.path.join(HERE, "si16_triclinic_snap.npz")))
    si432 = S.diamond_si(3, 3, 6, sigma=0.06, rng=np.random.default_rng(31))
    return [
        ("nn_nacl_snap", nacl, None, {"Cl": ([6, 5], ["Tanh", "Sigmoid", "Linear"]),
                                      "Na": ([7], ["Tanh", "Linear"])}, 3),
        ("nn_si16_snap", si16, None, {"Si": ([8, 8], ["Tanh", "Tanh", "Linear"])}, 4),
        # more than 400 atoms: the reference's per-atom np.where branch
        ("nn_si432_snap", None, (si432, dict(kind="SNAP", lmax=1, rcut=2.6, weights={"Si": 1.0}, rfac0=0.99363)),
         {"Si": ([5], ["Softplus", "Linear"])}, 5),
    ]


def main():
    so4, snap, _ = make_golden.load_reference()
    _install_nn_stubs()
    import importlib
    import torch
    nnmod = importlib.import_module("pyxtal_ff.models.neuralnetwork")
    prmod = importlib.import_module("pyxtal_ff.models.polynomialregression")
    torch.set_default_dtype(torch.float64)
    for name, fix, run, spec, seed in _cases():
        if fix is None:
            atoms, p = run
            out, dt, *_ = make_golden.run_case(so4, snap, atoms, p)
            fix = dict(positions=atoms.positions, cell=atoms.get_cell(), pbc=np.asarray(atoms.pbc, dtype=np.int32),
                       numbers=atoms.numbers, x=out["x"], seq=out["seq"], dxdr=out["dxdr"], rdxdr=out["rdxdr"],
                       meta=json.dumps(dict(p, derivative=True, stress=True)))
        symbols = [S.CHEMICAL_SYMBOLS[int(z)] for z in fix["numbers"]]
        n, nB = fix["x"].shape
        elements = sorted(set(symbols))
        nets, arch = _nets(torch, elements, nB, spec, seed)
        drange = _drange(fix["x"], elements, symbols, 0.05)
        desc = dict(x=np.asarray(fix["x"]), dxdr=np.asarray(fix["dxdr"]), seq=np.asarray(fix["seq"]),
                    rdxdr=_voigt_atom(np.asarray(fix["rdxdr"]), np.asarray(fix["seq"]), n), elements=symbols)
        pot = nnmod.NeuralNetwork.__new__(nnmod.NeuralNetwork)
        pot.elements, pot.models, pot.drange, pot.unit = elements, nets, drange, "eV"
        energies, forces, stress = pot.calculate_properties(desc, bforce=True, bstress=True)
        d = dict(positions=fix["positions"], cell=fix["cell"], pbc=fix["pbc"], numbers=fix["numbers"],
                 descriptor_meta=str(fix["meta"]), x=desc["x"], dxdr=desc["dxdr"], seq=desc["seq"],
                 rdxdr_atom=desc["rdxdr"], energies=energies, forces=forces, stress=stress,
                 arch=json.dumps(arch, sort_keys=True))
        for e in elements:
            d["drange_" + e] = drange[e]
            for k, v in nets[e].state_dict().items():
                d["w_%s_%s" % (e, k)] = v.detach().numpy()
        # the LAMMPS export of the same potential, and of a linear one
        meta = json.loads(str(fix["meta"]))
        des_info = {"type": meta["kind"], "Rc": meta["rcut"], "weights": meta.get("weights"),
                    "parameters": {"lmax": meta["lmax"], "rfac": meta.get("rfac0", 0.99363)}}
        with tempfile.TemporaryDirectory() as tmp:
            pot.path = tmp + "/"
            pot.hiddenlayers = {e: arch[e]["sizes"][1:] for e in elements}
            pot.activation = {e: arch[e]["acts"] for e in elements}
            pot.no_of_descriptors = nB
            pot.save_weights_to_txt(des_info)
            d["nn_weights_txt"] = open(tmp + "/NN_weights.txt").read()
            d["descriptor_param_txt"] = open(tmp + "/DescriptorParam.txt").read()
            pr = prmod.PR.__new__(prmod.PR)
            pr.path, pr.elements, pr.d_max = tmp + "/", elements, nB
            pr.coef_ = np.random.default_rng(seed).normal(size=len(elements) * (nB + 1))
            pr.save_weights_to_txt(des_info)
            d["pr_coef"] = pr.coef_
            d["pr_weights_txt"] = open(tmp + "/PR_weights.txt").read()
            d["pr_descriptor_param_txt"] = open(tmp + "/DescriptorParam.txt").read()
        d["des_info"] = json.dumps(des_info, sort_keys=True)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print("%-16s atoms %4d  nB %3d  E %.6f  |F|max %.3e  S %s" % (name, n, nB, energies.sum(), np.abs(forces).max(),
                                                                    np.array2string(stress, precision=4)), flush=True)


if __name__ == "__main__":
    main()
