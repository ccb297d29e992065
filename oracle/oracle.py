"""ctypes wrapper of the C oracle (test infrastructure only).

``descriptor()`` returns the reference's output dict
(``pyxtal_ff/descriptors/SO4.py:190-206``) computed by the FP64 CPU
restatement in so4_oracle.c: ``x``, ``dxdr``, ``rdxdr``, ``seq``,
``elements``.  ``forces_virial()`` contracts the same dB/dr with dE/dB on the
fly, the way the reference's consumers contract ``dxdr`` and ``rdxdr``
(``pyxtal_ff/models/neuralnetwork.py:492,497``), without storing them.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class _NL(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("nimg", C.c_int64), ("npair", C.c_int64),
        ("img_ptr", C.POINTER(C.c_int64)), ("img_j", C.POINTER(C.c_int32)),
        ("img_off", C.POINTER(C.c_int32)), ("img_r", C.POINTER(C.c_double)),
        ("pair_ptr", C.POINTER(C.c_int64)), ("seq", C.POINTER(C.c_int64)),
        ("pair_img", C.POINTER(C.c_int64)), ("nsite", C.POINTER(C.c_int64)),
    ]


class _Params(C.Structure):
    _fields_ = [("twol", C.c_int), ("cutoff_id", C.c_int), ("normalize_u", C.c_int),
                ("rcut", C.c_double), ("rfac0", C.c_double), ("vol", C.c_double)]


CUTOFF_IDS = {"cosine": 1, "tanh": 2, "poly1": 3, "poly2": 4, "poly3": 5, "poly4": 6, "exp": 7}


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.so4o_nl_build.restype = C.POINTER(_NL)
        L.so4o_nl_build.argtypes = [C.c_int, C.c_int, dp, dp, ip, C.c_double]
        L.so4o_nl_free.argtypes = [C.POINTER(_NL)]
        L.so4o_compute.restype = C.c_int
        L.so4o_compute.argtypes = [C.POINTER(_Params), C.POINTER(_NL), C.c_int, dp, dp, dp,
                                   dp, dp, dp, dp, dp, dp, C.c_int]
        L.so4o_sizes.argtypes = [C.c_int, ip]
        L.so4o_tables.argtypes = [C.c_int, C.c_int, dp, ip, ip, ip, ip, ip, dp]
        L.so4o_factorial.restype = C.c_double
        L.so4o_factorial.argtypes = [C.c_int]
        L.so4o_sfac.restype = C.c_double
        L.so4o_sfac.argtypes = [C.c_double, C.c_double, C.c_int]
        L.so4o_dsfac.restype = C.c_double
        L.so4o_dsfac.argtypes = [C.c_double, C.c_double, C.c_int]
        _lib = L
    return _lib


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def sizes(twol):
    out = np.zeros(5, dtype=np.int32)
    if lib().so4o_sizes(int(twol), _p(out, C.c_int)):
        raise ValueError("unsupported twol")
    return dict(idxu=int(out[0]), idxz=int(out[1]), idxcg=int(out[2]), nB=int(out[3]), idxu_half=int(out[4]))


def tables(twol, normalize_u=False):
    s = sizes(twol)
    ld = twol + 1
    cg = np.zeros(s["idxcg"]); idxb = np.zeros((s["nB"], 3), np.int32)
    idxz = np.zeros((s["idxz"], 10), np.int32); iub = np.zeros(ld, np.int32)
    izb = np.zeros((ld, ld, ld), np.int32); icb = np.zeros((ld, ld, ld), np.int32)
    un = np.zeros(s["idxu"])
    lib().so4o_tables(int(twol), int(bool(normalize_u)), _p(cg), _p(idxb, C.c_int), _p(idxz, C.c_int),
                      _p(iub, C.c_int), _p(izb, C.c_int), _p(icb, C.c_int), _p(un))
    return dict(cglist=cg, idxb=idxb, idxz=idxz, idxu_block=iub, idxz_block=izb, idxcg_block=icb, unorm=un)


def factorial(n):
    return lib().so4o_factorial(int(n))


class NeighborList:
    """Oracle neighbour list: CSR images per centre and the reference's seq."""

    def __init__(self, pos, cell, pbc, rc, n_center=None):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(3, 3)
        pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(3))
        n = len(pos)
        nc = n if n_center is None else int(n_center)
        ptr = lib().so4o_nl_build(n, nc, _p(pos), _p(cell), _p(pbc, C.c_int), float(rc))
        if not ptr:
            raise ValueError("oracle neighbour list: invalid input (singular cell or bad sizes)")
        self._ptr = ptr
        nl = ptr.contents
        self.n = nl.n
        self.nimg, self.npair = nl.nimg, nl.npair

        def arr(p, count, dt):
            if count == 0:
                return np.zeros(0, dtype=dt)
            return np.ctypeslib.as_array(p, shape=(count,)).astype(dt, copy=True)

        self.img_ptr = arr(nl.img_ptr, nc + 1, np.int64)
        self.img_j = arr(nl.img_j, self.nimg, np.int32)
        self.img_off = arr(nl.img_off, 3 * self.nimg, np.int32).reshape(-1, 3)
        self.img_r = arr(nl.img_r, 3 * self.nimg, np.float64).reshape(-1, 3)
        self.pair_ptr = arr(nl.pair_ptr, nc + 1, np.int64)
        self.seq = arr(nl.seq, 2 * self.npair, np.int64).reshape(-1, 2)
        self.pair_img = arr(nl.pair_img, self.npair + 1, np.int64)
        self.nsite = arr(nl.nsite, nc, np.int64)

    def __del__(self):
        try:
            if self._ptr:
                lib().so4o_nl_free(self._ptr)
                self._ptr = None
        except Exception:
            pass


def _weights(kind, numbers, symbols, weights):
    if kind == "SO4":
        w_nb = numbers.astype(np.float64)
        w_site = numbers.astype(np.float64)
    else:
        w_nb = np.array([float(weights[s]) for s in symbols], dtype=np.float64)
        w_site = np.ones(len(numbers), dtype=np.float64)
    return np.ascontiguousarray(w_nb), np.ascontiguousarray(w_site)


def compute(pos, cell, pbc, numbers, symbols, *, kind="SO4", lmax=3, rcut=3.5, weights=None,
            rfac0=None, cutoff="cosine", normalize_U=False, n_center=None, want_dxdr=True,
            want_rdxdr=True, beta=None, nthreads=0, nl=None):
    """Low-level oracle call.  Returns (nl, x, dxdr, rdxdr, forces, vir)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    cell = np.ascontiguousarray(cell, dtype=np.float64).reshape(3, 3)
    twol = int(round(2 * lmax))
    if nl is None:
        nl = NeighborList(pos, cell, pbc, rcut, n_center)
    nB = sizes(twol)["nB"]
    nc = nl.n
    w_nb, w_site = _weights(kind, np.asarray(numbers), symbols, weights)
    prm = _Params(twol, CUTOFF_IDS[cutoff], int(bool(normalize_U)), float(rcut),
                  float(1.0 if kind == "SO4" else (0.99363 if rfac0 is None else rfac0)),
                  abs(float(np.linalg.det(cell))))
    x = np.zeros((nc, nB))
    dxdr = np.zeros((nl.npair, nB, 3)) if want_dxdr else None
    rdxdr = np.zeros((nl.npair, nB, 3, 3)) if want_rdxdr else None
    forces = vir = None
    if beta is not None:
        beta = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, dtype=np.float64), (nc, nB)))
        forces = np.zeros((len(pos), 3))
        vir = np.zeros((3, 3))
    rc = lib().so4o_compute(C.byref(prm), nl._ptr, len(pos), _p(pos), _p(w_nb), _p(w_site),
                            _p(x), _p(dxdr), _p(rdxdr), _p(beta), _p(forces), _p(vir), int(nthreads))
    if rc:
        raise ValueError("oracle compute failed (status %d)" % rc)
    return nl, x, dxdr, rdxdr, forces, vir


def descriptor(atoms, *, kind="SO4", lmax=3, rcut=3.5, weights=None, rfac0=None, cutoff="cosine",
               normalize_U=False, derivative=True, stress=False, atom_ids=None, nthreads=0):
    """The reference's calculate() output dict, from the oracle."""
    from pyxtal_ff_gb300.structures import as_arrays
    pos, cell, pbc, numbers, symbols = as_arrays(atoms)
    n_center = None if atom_ids is None else len(list(atom_ids))
    nl, x, dxdr, rdxdr, _, _ = compute(pos, cell, pbc, numbers, symbols, kind=kind, lmax=lmax, rcut=rcut,
                                       weights=weights, rfac0=rfac0, cutoff=cutoff, normalize_U=normalize_U,
                                       n_center=n_center, want_dxdr=derivative, want_rdxdr=stress,
                                       nthreads=nthreads)
    out = {"x": x, "dxdr": dxdr if derivative else None, "elements": list(symbols),
           "rdxdr": rdxdr if stress else None}
    if derivative:
        out["seq"] = nl.seq
    return out


def forces_virial(atoms, beta, *, kind="SO4", lmax=3, rcut=3.5, weights=None, rfac0=None,
                  cutoff="cosine", normalize_U=False, nthreads=0, nl=None):
    """Energy, forces (-dE/dr) and the contracted virial for E = sum_i beta_i . x_i.

    vir = sum_i beta_i . sum_{pairs of i} rdxdr[pair]  (3x3, eV/A^3);
    the reference's stress is -vir in Voigt order [xx,yy,zz,xy,xz,yz] x 160.21766 GPa.
    """
    from pyxtal_ff_gb300.structures import as_arrays
    pos, cell, pbc, numbers, symbols = as_arrays(atoms)
    nl, x, _, _, f, vir = compute(pos, cell, pbc, numbers, symbols, kind=kind, lmax=lmax, rcut=rcut,
                                  weights=weights, rfac0=rfac0, cutoff=cutoff, normalize_U=normalize_U,
                                  want_dxdr=False, want_rdxdr=False, beta=beta, nthreads=nthreads, nl=nl)
    beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), x.shape)
    energy = float(np.sum(beta * x))
    return dict(x=x, energy=energy, forces=f, virial=vir, nl=nl)
