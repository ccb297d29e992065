"""Loader for the golden vectors in tests/golden/ (made by tests/golden/make_golden.py
from the reference itself).  Shared by the CPU oracle tests and the GPU parity tests."""
import glob
import json
import os

import numpy as np

from pyxtal_ff_gb300.structures import Atoms

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    """Descriptor cases (tests/golden/make_golden.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("reference_tables", "nn_", "pr_")))


def nn_names():
    """NN-potential cases (tests/golden/make_golden_nn.py)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "nn_*.npz")))


def load_nn(name):
    """atoms, descriptor parameters, the fixture dict, and per element its network
    (torch, FP64, the reference's layer layout) and drange."""
    import torch
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    meta = json.loads(str(d.pop("descriptor_meta")))
    arch = json.loads(str(d.pop("arch")))
    atoms = Atoms(d["numbers"], d["positions"], d["cell"], pbc=d["pbc"].astype(bool))
    nets, drange = {}, {}
    for e, a in arch.items():
        layers = []
        for i, act in enumerate(a["acts"]):
            layers.append(torch.nn.Linear(a["sizes"][i], a["sizes"][i + 1]))
            if act != "Linear":
                layers.append(getattr(torch.nn, act)())
        net = torch.nn.Sequential(*layers).double()
        pre = "w_%s_" % e
        net.load_state_dict({k[len(pre):]: torch.from_numpy(v) for k, v in d.items() if k.startswith(pre)})
        nets[e] = net
        drange[e] = d["drange_" + e]
    return atoms, meta, d, nets, drange


def load(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    meta = json.loads(str(d.pop("meta")))
    atoms = Atoms(d.pop("numbers"), d.pop("positions"), d.pop("cell"), pbc=d.pop("pbc").astype(bool))
    return atoms, meta, d


def tables():
    return dict(np.load(os.path.join(GOLDEN, "reference_tables.npz")))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        raise AssertionError("shape %s != %s" % (a.shape, b.shape))
    if b.size == 0:
        return 0.0
    scale = np.max(np.abs(b))
    diff = np.max(np.abs(a - b))
    return float(diff / scale) if scale > 0 else float(diff)


def compare_to_golden(out, d, tol):
    """Compare a reference-style output dict with one golden case; returns {key: rel err}."""
    errs = {"x": rel_err(out["x"], d["x"])}
    if "seq" in d:
        assert np.array_equal(np.asarray(out["seq"]), d["seq"]), "seq differs"
    seq = np.asarray(d["seq"]) if "seq" in d else None
    if "dxdr" in d:
        errs["dxdr"] = rel_err(out["dxdr"], d["dxdr"])
    if "dxdr_head" in d:
        dx = np.asarray(out["dxdr"])
        n = d["x"].shape[0]
        errs["dxdr_head"] = rel_err(dx[seq[:, 0] < 2], d["dxdr_head"])
        errs["dxdr_by_j"] = rel_err(np.stack([dx[seq[:, 1] == m].sum(0) for m in range(n)]), d["dxdr_by_j"])
        proj = np.random.default_rng(99).standard_normal(dx.shape[1:])
        errs["dxdr_proj"] = rel_err(np.einsum("pkc,kc->p", dx, proj), d["dxdr_proj"])
    if "rdxdr" in d:
        errs["rdxdr"] = rel_err(out["rdxdr"], d["rdxdr"])
    if "rdxdr_head" in d:
        rd = np.asarray(out["rdxdr"])
        n = d["x"].shape[0]
        errs["rdxdr_head"] = rel_err(rd[seq[:, 0] < 2], d["rdxdr_head"])
        errs["rdxdr_atom"] = rel_err(np.stack([rd[seq[:, 0] == m].sum(0) for m in range(n)]), d["rdxdr_atom"])
        proj = np.random.default_rng(98).standard_normal(rd.shape[1:])
        errs["rdxdr_proj"] = rel_err(np.einsum("pkab,kab->p", rd, proj), d["rdxdr_proj"])
    bad = {k: v for k, v in errs.items() if not (v <= tol)}
    assert not bad, "relative errors above %g: %s" % (tol, bad)
    return errs


def descriptor_kwargs(meta):
    kw = dict(kind=meta["kind"], lmax=meta["lmax"], rcut=meta["rcut"], cutoff=meta.get("cutoff", "cosine"),
              normalize_U=meta.get("normalize_U", False), derivative=meta["derivative"], stress=meta["stress"])
    if meta["kind"] == "SNAP":
        kw.update(weights=meta["weights"], rfac0=meta["rfac0"])
    if meta.get("atom_ids") is not None:
        kw["atom_ids"] = range(meta["atom_ids"])
    return kw
