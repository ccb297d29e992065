"""Generate tests/golden/pr_design.npz by running the REFERENCE's own linear potential
(class PR, pyxtal_ff/models/polynomialregression.py) on the descriptors stored in
tests/golden/nn_*.npz (which the reference's SNAP code computed):

- parse_descriptors(train=False) (:438-682) and calculate_properties (:374-411) per
  case, with the random coefficients stored there (pr_coef);
- parse_descriptors(train=True) over a two-structure database (the NaCl and Si16
  cases, elements Cl, Na, Si; only the second in the stress group), written with the
  standard-library shelve module as the reference reads it;
- the same for order 2 (quadratic features of the first d_max descriptors).

Runs in the build container only (the reference tree must be readable); stand-ins as
in make_golden_nn.py.

    python tests/golden/make_golden_pr.py
"""
import os
import shelve
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import make_golden  # noqa: E402
import make_golden_nn  # noqa: E402
from pyxtal_ff_gb300 import structures as S  # noqa: E402


def _desc(name):
    d = dict(np.load(os.path.join(HERE, name + ".npz")))
    symbols = [S.CHEMICAL_SYMBOLS[int(z)] for z in d["numbers"]]
    return d, dict(x=d["x"], dxdr=d["dxdr"], seq=d["seq"], rdxdr=d["rdxdr_atom"], elements=symbols)


def main():
    make_golden.load_reference()
    make_golden_nn._install_nn_stubs()
    import importlib
    prmod = importlib.import_module("pyxtal_ff.models.polynomialregression")
    out = {}
    for name in ("nn_nacl_snap", "nn_si16_snap", "nn_si432_snap"):
        d, desc = _desc(name)
        pr = prmod.PR.__new__(prmod.PR)
        pr.elements = sorted(set(desc["elements"]))
        pr.quadratic, pr.d_max, pr.coef_ = False, None, d["pr_coef"]
        X = pr.parse_descriptors({"0": desc}, fc=True, sc=True, train=False)
        e, f, s = pr.calculate_properties(desc, bforce=True, bstress=True)
        key = name[3:]
        out[key + "_X"], out[key + "_energies"], out[key + "_forces"], out[key + "_stress"] = X, e, f, s
        print(key, X.shape, e.sum(), flush=True)
    # order 2 (quadratic): the same per case, on the first few descriptors (d_max) so the
    # fixture stays small, with random coefficients
    for name, dmax in (("nn_nacl_snap", 6), ("nn_si16_snap", 5), ("nn_si432_snap", 5)):
        d, desc = _desc(name)
        pr = prmod.PR.__new__(prmod.PR)
        pr.elements = sorted(set(desc["elements"]))
        pr.quadratic, pr.d_max = True, dmax
        nq = (dmax * dmax + 3 * dmax) // 2
        pr.coef_ = np.random.default_rng(7).normal(size=len(pr.elements) * (1 + nq))
        X = pr.parse_descriptors({"0": desc}, fc=True, sc=True, train=False)
        e, f, s_ = pr.calculate_properties(desc, bforce=True, bstress=True)
        key = "quad_" + name[3:]
        out[key + "_X"], out[key + "_energies"], out[key + "_forces"], out[key + "_stress"] = X, e, f, s_
        out[key + "_coef"], out[key + "_dmax"] = pr.coef_, np.int64(dmax)
        print(key, X.shape, flush=True)
    # training matrix over two structures
    with tempfile.TemporaryDirectory() as tmp:
        db = shelve.open(os.path.join(tmp, "train"))
        for i, (name, group) in enumerate((("nn_nacl_snap", "A"), ("nn_si16_snap", "B"))):
            _, desc = _desc(name)
            desc["group"] = group
            db[str(i)] = desc
        db.close()
        pr = prmod.PR.__new__(prmod.PR)
        pr.path = tmp + "/"
        pr.elements = ["Cl", "Na", "Si"]
        pr.quadratic, pr.d_max = False, None
        pr.no_of_structures, pr.no_of_atoms, pr.stress_components = 2, 8 + 16, 6
        pr.stress_group = ["B"]
        X = pr.parse_descriptors("train", fc=True, sc=True, train=True)
        out["train_X"] = X
        print("train", X.shape, flush=True)
        pr.quadratic, pr.d_max = True, 6
        X = pr.parse_descriptors("train", fc=True, sc=True, train=True)
        out["quad_train_X"] = X
        print("quad train", X.shape, flush=True)
    np.savez_compressed(os.path.join(HERE, "pr_design.npz"), **out)


if __name__ == "__main__":
    main()
