"""Generate the golden vectors in tests/golden/ by running the REFERENCE itself.

This script runs only where the reference source tree is readable; its root
(the directory holding ``pyxtal_ff/``) must be given in $PYXTAL_FF_REF.  It imports the
reference's own descriptor modules unchanged --
``pyxtal_ff/descriptors/SO4.py``, ``SNAP.py``, ``angular_momentum.py``,
``utils.py`` -- with three stand-ins for what this container lacks:

* numba (not installed): ``njit`` becomes the identity decorator and
  ``prange`` becomes ``range``, so the numba kernels run as plain CPython;
* ASE (not installed; ``ase.neighborlist.NeighborList``, ASE >= 3.22.1):
  a brute-force numpy neighbour list that returns every periodic image with
  |pos[j] + o.cell - pos[i]| < cutoff_i + cutoff_j, excluding (i, o=0), in
  (j, o) lexicographic order (the intra-group order is the one detail ASE's
  own order is not pinned on);
* Python 3 range(): the reference calls ``range(0, l/2, 1)`` with a float
  in compute_bi / compute_dbidrj (SO4.py:1101-1102, 1141-1142, ...); that runs
  under numba but not CPython, so a module-level ``range`` that accepts
  integral floats is injected into the two modules' globals (the source files
  are not modified).

Outputs: one compressed .npz per case with the inputs (positions, cell, pbc,
numbers, parameters) and the reference's outputs (x, dxdr, rdxdr, seq), plus
reference.npz with the reference's factorial table and CG lists.  Large cases
keep x and seq in full, the pair arrays of the first centres, and per-atom /
whole-array reductions of the rest.

    PYXTAL_FF_REF=<reference root> python tests/golden/make_golden.py [--only name ...]
"""
import argparse
import builtins
import json
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from pyxtal_ff_gb300 import structures as S  # noqa: E402

def reference_root():
    """The reference's source root, from $PYXTAL_FF_REF (required: there is no default)."""
    ref = os.environ.get("PYXTAL_FF_REF")
    if not ref or not os.path.isdir(os.path.join(ref, "pyxtal_ff", "descriptors")):
        raise SystemExit("set PYXTAL_FF_REF to the reference's source root (the directory holding pyxtal_ff/)")
    return ref


# --------------------------------------------------------------------------- stubs
def _install_numba_stub():
    nb = types.ModuleType("numba")

    class _Type:
        def __call__(self, *a, **k):
            return self

        def __getitem__(self, k):
            return self

    for name in ("f8", "f4", "i8", "i4", "c16", "c8", "b1", "void", "int64", "float64", "complex128"):
        setattr(nb, name, _Type())

    def njit(*args, **kwargs):
        if len(args) == 1 and isinstance(args[0], types.FunctionType):
            return args[0]
        return lambda f: f

    nb.njit = njit
    nb.jit = njit
    nb.prange = range
    nb.types = types.SimpleNamespace()
    sys.modules["numba"] = nb


class _StubNeighborList:
    """Brute-force stand-in for ase.neighborlist.NeighborList (bothways, no self)."""

    def __init__(self, cutoffs, self_interaction=False, bothways=True, skin=0.0):
        assert not self_interaction and bothways
        self.cutoffs = np.asarray(cutoffs, dtype=np.float64)

    def update(self, atoms):
        pos = np.asarray(atoms.positions, dtype=np.float64)
        cell = np.asarray(atoms.get_cell(), dtype=np.float64)
        pbc = np.broadcast_to(np.asarray(atoms.pbc, dtype=bool), (3,))
        inv = np.linalg.inv(cell)
        frac = pos @ inv
        d = 1.0 / np.linalg.norm(inv, axis=0)  # plane spacings
        n = len(pos)
        self._idx, self._off = [], []
        for i in range(n):
            js, offs = [], []
            for j in range(n):
                rc = self.cutoffs[i] + self.cutoffs[j]
                rng = []
                for k in range(3):
                    if pbc[k]:
                        df = frac[i, k] - frac[j, k]
                        lo = int(np.floor(df - rc / d[k])) - 1
                        hi = int(np.ceil(df + rc / d[k])) + 1
                        rng.append(range(lo, hi + 1))
                    else:
                        rng.append(range(0, 1))
                for o0 in rng[0]:
                    for o1 in rng[1]:
                        for o2 in rng[2]:
                            if j == i and o0 == 0 and o1 == 0 and o2 == 0:
                                continue
                            sc = (o0 * cell[0] + o1 * cell[1]) + o2 * cell[2]
                            r = (pos[j] + sc) - pos[i]
                            rr = np.sqrt((r[0] * r[0] + r[1] * r[1]) + r[2] * r[2])
                            if rr < rc:
                                js.append(j)
                                offs.append((o0, o1, o2))
            self._idx.append(np.array(js, dtype=np.int64))
            self._off.append(np.array(offs, dtype=np.int64).reshape(-1, 3))

    def get_neighbors(self, i):
        return self._idx[i], self._off[i]


def _install_ase_stub():
    ase = types.ModuleType("ase")
    nlm = types.ModuleType("ase.neighborlist")
    nlm.NeighborList = _StubNeighborList
    ase.neighborlist = nlm
    sys.modules["ase"] = ase
    sys.modules["ase.neighborlist"] = nlm


def _int_range(*args):
    conv = []
    for a in args:
        if isinstance(a, float):
            if not a.is_integer():
                raise TypeError("non-integral range bound %r" % a)
            a = int(a)
        conv.append(a)
    return builtins.range(*conv)


def load_reference():
    ref = reference_root()
    _install_numba_stub()
    _install_ase_stub()
    pkg = types.ModuleType("pyxtal_ff")
    pkg.__path__ = [os.path.join(ref, "pyxtal_ff")]
    sub = types.ModuleType("pyxtal_ff.descriptors")
    sub.__path__ = [os.path.join(ref, "pyxtal_ff", "descriptors")]
    sys.modules["pyxtal_ff"] = pkg
    sys.modules["pyxtal_ff.descriptors"] = sub
    import importlib
    so4 = importlib.import_module("pyxtal_ff.descriptors.SO4")
    snap = importlib.import_module("pyxtal_ff.descriptors.SNAP")
    am = importlib.import_module("pyxtal_ff.descriptors.angular_momentum")
    so4.range = _int_range
    snap.range = _int_range
    return so4, snap, am


# --------------------------------------------------------------------------- cases
def _cases():
    c = []
    nacl = S.nacl_cluster(1.0)
    c.append(("nacl_so4", nacl, dict(kind="SO4", lmax=2, rcut=6.0)))
    c.append(("nacl_snap", nacl, dict(kind="SNAP", lmax=2, rcut=6.0, weights={"Na": 0.3, "Cl": 0.7}, rfac0=0.99363)))
    si8 = S.diamond_si(1, 1, 1, sigma=0.05, rng=np.random.default_rng(11))
    c.append(("si8_images_so4", si8, dict(kind="SO4", lmax=3, rcut=4.9)))
    tri = S.diamond_si(1, 1, 2, sigma=0.08, strain=0.04, rng=np.random.default_rng(12))
    c.append(("si16_triclinic_snap", tri, dict(kind="SNAP", lmax=2, rcut=4.0, weights={"Si": 1.0}, rfac0=0.99363)))
    for cut in ("tanh", "poly1", "poly2", "poly3", "poly4", "exp"):
        c.append(("si8_cut_%s" % cut, si8, dict(kind="SO4", lmax=1, rcut=3.5, cutoff=cut)))
    c.append(("si8_normU_snap", si8, dict(kind="SNAP", lmax=2, rcut=3.5, weights={"Si": 0.8}, rfac0=0.9,
                                          normalize_U=True)))
    ragged = S.Atoms([14, 8, 14], [[1.0, 1.0, 1.0], [2.6, 1.2, 0.9], [0.2, 3.6, 1.0]], 14.0 * np.eye(3), pbc=True)
    c.append(("ragged_so4", ragged, dict(kind="SO4", lmax=2, rcut=3.0)))
    c.append(("si8_prefix_so4", si8, dict(kind="SO4", lmax=2, rcut=4.2, atom_ids=3)))
    c.append(("si8_noderiv_so4", si8, dict(kind="SO4", lmax=2, rcut=4.2, derivative=False, stress=False)))
    c.append(("si8_nostress_so4", si8, dict(kind="SO4", lmax=2, rcut=4.2, derivative=True, stress=False)))
    sio2 = S.sio2_random(n_si=8, density=2.2, dmin=1.4, seed=5)
    c.append(("sio2_24_lmax4_snap", sio2, dict(kind="SNAP", lmax=4, rcut=5.0, weights={"Si": 1.0, "O": 0.5},
                                               rfac0=0.99363, big=True)))
    cfg0 = S.diamond_si(2, 2, 2, sigma=0.05, rng=np.random.default_rng(0))
    c.append(("si64_lmax3_snap_w1", cfg0, dict(kind="SNAP", lmax=3, rcut=4.9, weights={"Si": 1.0}, rfac0=1.0, big=True)))
    c.append(("si64_lmax3_so4", cfg0, dict(kind="SO4", lmax=3, rcut=4.9, big=True)))
    return c


def run_case(so4, snap, atoms, p):
    p = dict(p)
    big = p.pop("big", False)
    kind = p.pop("kind")
    atom_ids = p.pop("atom_ids", None)
    deriv = p.pop("derivative", True)
    stress = p.pop("stress", True)
    common = dict(lmax=p["lmax"], rcut=p["rcut"], derivative=deriv, stress=stress,
                  normalize_U=p.get("normalize_U", False), cutoff_function=p.get("cutoff", "cosine"))
    if kind == "SO4":
        f = so4.SO4_Bispectrum(**common)
    else:
        f = snap.SO4_Bispectrum(p["weights"], rfac0=p["rfac0"], **common)
    t0 = time.time()
    out = f.calculate(atoms, atom_ids=None if atom_ids is None else range(atom_ids))
    dt = time.time() - t0
    return out, dt, big, kind, atom_ids, deriv, stress


def save_case(name, atoms, p, out, dt, big, kind, atom_ids, deriv, stress):
    meta = dict(p)
    meta.pop("big", None)
    meta.update(kind=kind, derivative=deriv, stress=stress, atom_ids=atom_ids, seconds=round(dt, 3))
    d = dict(positions=atoms.positions, cell=atoms.get_cell(), pbc=np.asarray(atoms.pbc, dtype=np.int32),
             numbers=atoms.numbers, meta=json.dumps(meta, sort_keys=True), x=np.ascontiguousarray(out["x"]))
    if "seq" in out:
        d["seq"] = out["seq"]
    if out.get("dxdr") is not None:
        dx = np.ascontiguousarray(out["dxdr"])
        if big:
            seq = out["seq"]
            head = np.nonzero(seq[:, 0] < 2)[0]
            d["dxdr_head"] = dx[head]
            n = out["x"].shape[0]
            d["dxdr_by_j"] = np.stack([dx[seq[:, 1] == m].sum(0) for m in range(n)])
            rngp = np.random.default_rng(99).standard_normal(dx.shape[1:])
            d["dxdr_proj"] = np.einsum("pkc,kc->p", dx, rngp)
        else:
            d["dxdr"] = dx
    if out.get("rdxdr") is not None:
        rd = np.ascontiguousarray(out["rdxdr"])
        if big:
            seq = out["seq"]
            head = np.nonzero(seq[:, 0] < 2)[0]
            d["rdxdr_head"] = rd[head]
            n = out["x"].shape[0]
            d["rdxdr_atom"] = np.stack([rd[seq[:, 0] == m].sum(0) for m in range(n)])
            rngp = np.random.default_rng(98).standard_normal(rd.shape[1:])
            d["rdxdr_proj"] = np.einsum("pkab,kab->p", rd, rngp)
        else:
            d["rdxdr"] = rd
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)


def save_reference_tables(am, so4):
    facts = np.array([am.factorial(n) for n in range(0, 40)])
    d = dict(factorial=facts)
    for twol in range(0, 11):
        ldim = twol + 1
        cnt = 0
        for l1 in range(ldim):
            for l2 in range(l1 + 1):
                for l in range(l1 - l2, min(twol, l1 + l2) + 1, 2):
                    cnt += (l1 + 1) * (l2 + 1)
        cg = np.zeros(cnt)
        so4.init_clebsch_gordan(twol, cg)
        d["cglist_%d" % twol] = cg
    np.savez_compressed(os.path.join(HERE, "reference_tables.npz"), **d)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*")
    args = ap.parse_args()
    so4, snap, am = load_reference()
    if not args.only or "tables" in args.only:
        save_reference_tables(am, so4)
        print("reference_tables.npz")
    for name, atoms, p in _cases():
        if args.only and name not in args.only:
            continue
        res = run_case(so4, snap, atoms, p)
        save_case(name, atoms, p, *res)
        print("%-24s %7.2f s  x%s" % (name, res[1], res[0]["x"].shape), flush=True)


if __name__ == "__main__":
    main()
