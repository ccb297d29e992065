"""Host orchestration of the CUDA path: device tables, the GPU neighbour list and
the descriptor / adjoint launches.  Device memory comes from torch (the caller
side of the C ABI); the library itself allocates nothing but its tables.

A batch is any list of structures: their atoms are concatenated, structure s
owning atoms [atom_ptr[s], atom_ptr[s+1]).  Every launch goes on torch's current
CUDA stream.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import Geom, Params, Tuning, check, lib

CUTOFF_IDS = {"cosine": 1, "tanh": 2, "poly1": 3, "poly2": 4, "poly3": 5, "poly4": 6, "exp": 7}


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def require_cuda():
    """Raise unless a CUDA device is present: the path has no CPU fallback."""
    if not torch.cuda.is_available():
        raise RuntimeError("pyxtal_ff_gb300 needs a CUDA GPU (GB300, sm_103a); there is no CPU fallback")


# ---------------------------------------------------------------------- tables
class Tables:
    """Device-resident CG / rootpq / index tables for one (twol, normalize_U), built for
    one tuning of the FP32 kernels' launch shapes (None: the defaults; see so4_tuning)."""

    def __init__(self, twol, normalize_u=False, tuning=None):
        h = C.c_void_p()
        if tuning is None:
            check(lib().so4_tables_create(int(twol), int(bool(normalize_u)), C.byref(h)), "so4_tables_create")
        else:
            t6 = tuple(tuning) + (0,) * (6 - len(tuning))
            tn = Tuning(*(int(v) for v in t6[:6]))
            check(lib().so4_tables_create_tuned(int(twol), int(bool(normalize_u)), C.byref(tn), C.byref(h)),
                  "so4_tables_create_tuned")
        self.handle = h
        tn = Tuning()
        check(lib().so4_tables_get_tuning(h, C.byref(tn)), "so4_tables_get_tuning")
        # (wkmax, rev_threads, utot_warps, rev_pair, zw_atoms, zw_threads), resolved
        self.tuning = (tn.wkmax, tn.rev_threads, tn.utot_warps, tn.rev_pair, tn.zw_atoms, tn.zw_threads)
        s = (C.c_int * 8)()
        check(lib().so4_tables_sizes(h, s), "so4_tables_sizes")
        self.twol = int(twol)
        self.n_u, self.n_half, self.n_z, self.nB, self.n_cg, self.n_blk, self.n_bsec, self.n_wsub = [int(v) for v in s]

    def export(self):
        ld = self.twol + 1
        cg = np.zeros(self.n_cg)
        idxb = np.zeros((self.nB, 3), np.int32)
        idxz = np.zeros((self.n_z, 10), np.int32)
        iub = np.zeros(ld, np.int32)
        izb = np.zeros((ld, ld, ld), np.int32)
        icb = np.zeros((ld, ld, ld), np.int32)
        check(lib().so4_tables_export(self.handle, cg.ctypes.data, idxb.ctypes.data, idxz.ctypes.data,
                                      iub.ctypes.data, izb.ctypes.data, icb.ctypes.data), "so4_tables_export")
        return dict(cglist=cg, idxb=idxb, idxz=idxz, idxu_block=iub, idxz_block=izb, idxcg_block=icb)

    def __del__(self):
        try:
            if self.handle:
                lib().so4_tables_destroy(self.handle)
                self.handle = None
        except Exception:
            pass


_TABLES = {}


def tables(twol, normalize_u=False, tuning=None):
    """The tables of (twol, normalize_u) on the current device, built once per tuning
    ((wkmax, rev_threads, utot_warps[, rev_pair]) with 0 for a default, or None for all
    defaults)."""
    tkey = None if tuning is None else tuple(int(v) for v in tuning)
    key = (int(twol), bool(normalize_u), torch.cuda.current_device(), tkey)
    t = _TABLES.get(key)
    if t is None:
        t = Tables(twol, normalize_u, tkey)
        _TABLES[key] = t
    return t


def params(twol, rcut, rfac0, cutoff):
    return Params(int(twol), CUTOFF_IDS[cutoff], float(rcut), float(rfac0))


# ---------------------------------------------------------------- neighbours
@dataclass
class Neighbors:
    natoms: int
    nstruct: int
    nimg: int
    npair: int
    atom_ptr: np.ndarray       # host (S+1,)
    vol: np.ndarray            # host (S,)
    geom: torch.Tensor         # device bytes
    nbins: int
    atom_struct: torch.Tensor  # (N,) i32
    atom_ptr_dev: torch.Tensor  # (S+1,) i32
    img_ptr: torch.Tensor      # (N+1,) i32
    img_j: torch.Tensor        # (M,) i32
    img_off: torch.Tensor      # (M,3) i32
    img_r: torch.Tensor        # (M,3) f64
    pair_ptr: torch.Tensor     # (N+1,) i32
    seq: torch.Tensor          # (P,2) i64
    pair_img: torch.Tensor     # (P+1,) i32
    nsite: torch.Tensor        # (N,) i32
    img_pair: torch.Tensor     # (M,) i32
    img_rev: torch.Tensor      # (M,) i32
    no_neighbor: bool          # some atom has no image within rcut


def geometry(cells, pbc, atom_ptr, rcut):
    cells = np.ascontiguousarray(np.asarray(cells, dtype=np.float64).reshape(-1, 9))
    pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(-1, 3))
    atom_ptr = np.ascontiguousarray(np.asarray(atom_ptr, dtype=np.int32))
    S = len(cells)
    geo = (Geom * max(S, 1))()
    nb = C.c_int()
    rc = lib().so4_geometry(cells.ctypes.data, pbc.ctypes.data, atom_ptr.ctypes.data, S, float(rcut), geo,
                            C.byref(nb))
    if rc == _lib.SO4_ERR_NONFINITE:
        raise ValueError("cell contains NaN or Inf")
    if rc == _lib.SO4_ERR_ARG:
        raise ValueError("singular cell with periodic boundary conditions, or invalid rcut")
    check(rc, "so4_geometry")
    raw = np.frombuffer(bytes(geo), dtype=np.uint8)[: C.sizeof(Geom) * S]
    vol = np.array([geo[s].vol for s in range(S)])
    return raw, vol, int(nb.value)


_NL_CAPACITY = {}  # (natoms, nbins, rcut) -> (image capacity, pair capacity) seen last time
_LAYOUTS = {}      # batch layout -> device copies of its geometry (read-only, shared)


@dataclass
class Layout:
    """What the neighbour list needs of a batch besides the positions, on the device."""
    natoms: int
    nstruct: int
    atom_ptr: np.ndarray
    vol: np.ndarray
    geom: torch.Tensor
    nbins: int
    atom_struct: torch.Tensor
    atom_ptr_dev: torch.Tensor
    rcut: float


def layout(cells, pbc, atom_ptr, rcut, device="cuda"):
    """Geometry of a batch (cells, pbc, atom ranges) uploaded once per distinct layout."""
    dev = torch.device(device)
    cells = np.ascontiguousarray(np.asarray(cells, dtype=np.float64).reshape(-1, 3, 3))
    pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(-1, 3))
    atom_ptr = np.ascontiguousarray(np.asarray(atom_ptr, dtype=np.int64))
    key = (str(dev), float(rcut), cells.tobytes(), pbc.tobytes(), atom_ptr.tobytes())
    lay = _LAYOUTS.get(key)
    if lay is not None:
        return lay
    N, S = int(atom_ptr[-1]), len(atom_ptr) - 1
    raw, vol, nbins = geometry(cells, pbc, atom_ptr, rcut)
    counts = np.diff(atom_ptr)
    lay = Layout(N, S, atom_ptr, vol, torch.from_numpy(raw.copy()).to(dev), nbins,
                 torch.from_numpy(np.repeat(np.arange(S, dtype=np.int32), counts)).to(dev),
                 torch.from_numpy(atom_ptr.astype(np.int32)).to(dev), float(rcut))
    if len(_LAYOUTS) >= 16:
        _LAYOUTS.pop(next(iter(_LAYOUTS)))
    _LAYOUTS[key] = lay
    return lay


@dataclass
class NeighborBuffers:
    """Device arrays of one neighbour list with room for cap_m images and cap_p pairs."""
    cap_m: int
    cap_p: int
    ws: torch.Tensor
    img_ptr: torch.Tensor
    img_j: torch.Tensor
    img_off: torch.Tensor
    img_r: torch.Tensor
    pair_ptr: torch.Tensor
    seq: torch.Tensor
    pair_img: torch.Tensor
    nsite: torch.Tensor
    img_pair: torch.Tensor
    img_rev: torch.Tensor

    slot_cap: int = 0   # > 0: the one-pass count + keys mode (so4_nl_count_keys / so4_nl_sort)

    @staticmethod
    def allocate(lay: Layout, cap_m, cap_p, device, workspace=None, slot_cap=0):
        dev, N = torch.device(device), lay.natoms
        ws_bytes = lib().so4_nl_workspace_size(N, lay.nbins, max(cap_m, N * slot_cap))
        ws = workspace if (workspace is not None and workspace.numel() >= ws_bytes) else \
            torch.empty(ws_bytes, dtype=torch.uint8, device=dev)
        i32 = dict(dtype=torch.int32, device=dev)
        return NeighborBuffers(cap_m, cap_p, ws, torch.empty(N + 1, **i32), torch.empty(cap_m, **i32),
                               torch.empty((cap_m, 3), **i32), torch.empty((cap_m, 3), dtype=torch.float64, device=dev),
                               torch.empty(N + 1, **i32), torch.empty((cap_p, 2), dtype=torch.int64, device=dev),
                               torch.empty(cap_p + 1, **i32), torch.empty(max(N, 1), **i32),
                               torch.empty(cap_m, **i32), torch.empty(cap_m, **i32), int(slot_cap))

    def summary_dev(self):
        """The device copy of {images, pairs, status bits} that enqueue_neighbors leaves."""
        return self.ws[16:28].view(torch.int32)

    def max_count_dev(self):
        """Largest per-atom image count (slot mode only)."""
        return self.ws[32:36].view(torch.int32)


def enqueue_neighbors(lay: Layout, pos, bufs: NeighborBuffers, summary=None, lite=False):
    """Launch the three neighbour-list passes for positions pos (N,3) f64 on the device
    into bufs, and the summary; with summary (a ctypes int[3]) the call waits and
    fills it, else nothing synchronises (the summary stays on the device).  lite: skip
    the pair arrays (seq, pair_img, nsite, img_pair), keeping what the adjoint reads."""
    L, st, N, S = lib(), _stream(), lay.natoms, lay.nstruct
    b = bufs
    if b.slot_cap > 0:
        check(L.so4_nl_count_keys(_ptr(lay.geom), S, lay.nbins, _ptr(pos), _ptr(lay.atom_struct), N, lay.rcut,
                                  b.slot_cap, _ptr(b.img_ptr), _ptr(b.ws), b.ws.numel(), st), "so4_nl_count_keys")
        check(L.so4_nl_sort(_ptr(lay.geom), S, lay.nbins, _ptr(pos), _ptr(lay.atom_struct), N, _ptr(b.img_ptr),
                            b.cap_m, b.slot_cap, _ptr(b.img_j), _ptr(b.img_off), _ptr(b.img_r), _ptr(b.pair_ptr),
                            _ptr(b.ws), b.ws.numel(), st), "so4_nl_sort")
    else:
        check(L.so4_nl_count(_ptr(lay.geom), S, lay.nbins, _ptr(pos), _ptr(lay.atom_struct), N, lay.rcut,
                             _ptr(b.img_ptr), _ptr(b.ws), b.ws.numel(), st), "so4_nl_count")
        check(L.so4_nl_fill(_ptr(lay.geom), S, lay.nbins, _ptr(pos), _ptr(lay.atom_struct), N, lay.rcut,
                            _ptr(b.img_ptr), b.cap_m, _ptr(b.img_j), _ptr(b.img_off), _ptr(b.img_r),
                            _ptr(b.pair_ptr), _ptr(b.ws), b.ws.numel(), st), "so4_nl_fill")
    pairs = not lite
    check(L.so4_nl_pairs(_ptr(lay.geom), S, _ptr(lay.atom_struct), N, _ptr(b.img_ptr), b.cap_m, _ptr(b.img_j),
                         _ptr(b.img_off), _ptr(b.pair_ptr), b.cap_p, _ptr(b.seq if pairs else None),
                         _ptr(b.pair_img if pairs else None), _ptr(b.nsite if pairs else None),
                         _ptr(b.img_pair if pairs else None), _ptr(b.img_rev), _ptr(b.ws), b.ws.numel(), st),
          "so4_nl_pairs")
    check(L.so4_nl_summary(_ptr(b.img_ptr), _ptr(b.pair_ptr), N, _ptr(b.ws), b.ws.numel(), st, summary),
          "so4_nl_summary")


def check_summary(M, P, bits, cap_m=None, cap_p=None):
    """False if a neighbour list overflowed its buffers; else raise for its status bits
    (non-finite positions, an offset beyond the encodable range, an asymmetric list)."""
    if (cap_m is not None and M > cap_m) or (cap_p is not None and P > cap_p) or (bits & (1 << _lib.SO4_ERR_SLOTS)):
        return False
    if bits & (1 << _lib.SO4_ERR_NONFINITE):
        raise ValueError("positions contain NaN or Inf")
    for code in (_lib.SO4_ERR_CAPACITY, _lib.SO4_ERR_REVERSE):  # capacity here: an image offset beyond 511 cells
        if bits & (1 << code):
            raise _lib.SO4Error(code, "neighbour list")
    return True


def capacity_for(lay: Layout):
    """Image / pair capacity for a layout: the last count seen with 10 % room, else 64 per atom."""
    N = lay.natoms
    return _NL_CAPACITY.get((N, lay.nbins, lay.rcut), (max(64 * N, 1), max(64 * N, 1) + N))


def note_capacity(lay: Layout, M, P):
    _NL_CAPACITY[(lay.natoms, lay.nbins, lay.rcut)] = (max(int(M * 1.1) + 16, 1), max(int(P * 1.1) + 16, 1))


def neighbors_view(lay: Layout, b: NeighborBuffers, M, P, bits=0):
    """A Neighbors record over buffers b holding M images and P pairs (M, P may be the
    capacities when the true counts are still on the device)."""
    return Neighbors(lay.natoms, lay.nstruct, M, P, lay.atom_ptr, lay.vol, lay.geom, lay.nbins, lay.atom_struct,
                     lay.atom_ptr_dev, b.img_ptr, b.img_j[:M], b.img_off[:M], b.img_r[:M], b.pair_ptr, b.seq[:P],
                     b.pair_img[: P + 1], b.nsite[: lay.natoms], b.img_pair[:M], b.img_rev[:M],
                     bool(bits & (1 << _lib.SO4_ERR_NO_NEIGHBOR)))


def build_neighbors(pos, cells, pbc, atom_ptr, rcut, device="cuda", workspace=None):
    """GPU neighbour list of a batch.  pos: (N,3) f64 tensor on the device (or a
    numpy array), cells (S,3,3), pbc (S,3), atom_ptr (S+1,) host arrays.

    The image and pair arrays are sized from the counts of the previous call with
    the same shape (a first call uses an estimate); one synchronising read returns
    the true totals and the status, and an undersized call is repeated with room."""
    dev = torch.device(device)
    if not isinstance(pos, torch.Tensor):
        pos = torch.from_numpy(np.ascontiguousarray(pos, dtype=np.float64))
    pos = pos.to(dev, dtype=torch.float64).contiguous()
    lay = layout(cells, pbc, atom_ptr, rcut, dev)
    if pos.shape != (lay.natoms, 3):
        raise ValueError("positions must be (N,3) for N = atom_ptr[-1]")
    cap_m, cap_p = capacity_for(lay)
    summary = (C.c_int * 3)()
    for _attempt in range(3):
        bufs = NeighborBuffers.allocate(lay, cap_m, cap_p, dev, workspace)
        enqueue_neighbors(lay, pos, bufs, summary)
        M, P, bits = int(summary[0]), int(summary[1]), int(summary[2])
        if check_summary(M, P, bits, cap_m, cap_p):
            break
        cap_m, cap_p = max(cap_m, int(M * 1.25) + 16), max(cap_p, int(P * 1.25) + 16)
    else:
        raise _lib.SO4Error(_lib.SO4_ERR_CAPACITY, "neighbour list")
    note_capacity(lay, M, P)
    return neighbors_view(lay, bufs, M, P, bits)


# ----------------------------------------------------------------- compute
def site_weights(kind, numbers, symbols, weights=None):
    """(w_nb, w_site) per atom: SO4.py uses atomic numbers for both
    (SO4.py:244, 271); SNAP.py uses weights[symbol] and 1 (SNAP.py:273, 299-301)."""
    numbers = np.asarray(numbers)
    if kind == "SO4":
        w = numbers.astype(np.float64)
        return w, w.copy()
    w_nb = np.array([float(weights[s]) for s in symbols], dtype=np.float64)
    return w_nb, np.ones(len(numbers), dtype=np.float64)


def plain(tab, prm, nb: Neighbors, pos, w_nb, w_site, precision=0, want_deriv=True, want_stress=True):
    """x (N,nB), dxdr (P,nB,3), rdxdr (P,nB,3,3) on the device; FP64 (precision 0) or FP32 (1)."""
    dev = pos.device
    dt = torch.float64 if precision == 0 else torch.float32
    x = torch.empty((max(nb.natoms, 1), tab.nB), dtype=dt, device=dev)
    dxdr = torch.empty((max(nb.npair, 1), tab.nB, 3), dtype=dt, device=dev) if want_deriv else None
    rdxdr = torch.empty((max(nb.npair, 1), tab.nB, 3, 3), dtype=dt, device=dev) if (want_deriv and want_stress) else None
    ws = torch.empty(lib().so4_plain_workspace_size(tab.handle, nb.natoms), dtype=torch.uint8, device=dev)
    check(lib().so4_plain(tab.handle, C.byref(prm), int(precision), _ptr(nb.geom), _ptr(nb.atom_struct), nb.natoms,
                          _ptr(pos), _ptr(w_nb), _ptr(w_site), _ptr(nb.img_ptr), _ptr(nb.img_j), _ptr(nb.img_r),
                          _ptr(nb.pair_ptr), _ptr(nb.pair_img), _ptr(nb.nsite), int(want_deriv),
                          int(want_deriv and want_stress), _ptr(x), _ptr(dxdr), _ptr(rdxdr), _ptr(ws), ws.numel(),
                          _stream()), "so4_plain")
    x = x[: nb.natoms]
    if dxdr is not None:
        dxdr = dxdr[: nb.npair]
    if rdxdr is not None:
        rdxdr = rdxdr[: nb.npair]
    return x, dxdr, rdxdr


def rdxdr_atom(rdxdr, pair_ptr, natoms):
    """Per-atom Voigt stress rows (natoms, nB, 6) from per-pair rdxdr (P, nB, 3, 3) whose
    pairs are grouped by centre (pair_ptr), as the reference's caller forms them
    (pyxtal_ff/utilities/__init__.py:226-233)."""
    nB = rdxdr.shape[1]
    out = torch.empty((max(natoms, 1), nB, 6), dtype=rdxdr.dtype, device=rdxdr.device)
    prec = 0 if rdxdr.dtype == torch.float64 else 1
    check(lib().so4_rdxdr_atom(prec, _ptr(rdxdr.contiguous()), _ptr(pair_ptr), natoms, nB, _ptr(out), _stream()),
          "so4_rdxdr_atom")
    return out[:natoms]


def contract_dxdr(beta, pair_ptr, seq, atom_struct, atom_ptr, dxdr=None, rdxdr_atom=None, status=None, out=None):
    """Forces (N, 3) and per-structure stress sums (S, 6) from the plain path's dxdr /
    per-atom rdxdr and beta = dE/dx (so4_contract_dxdr):
      forces[m] = -sum over pairs p with seq[p, 1] == m of beta[i(p)] . dxdr[p]
      stress[s] = -sum over the atoms i of s of beta[i] . rdxdr_atom[i]   (no unit factor)
    Either output is None when its input is.  All arrays on one device, one dtype.
    Without `status` the call reads the status word back and raises ValueError for a
    pair without its reverse; with a zeroed device int32 `status` it does not
    synchronise and leaves the bits there.  `out` = (forces, stress_atom, stress) reuses
    caller buffers of shapes (N, 3), (N, 6), (S, 6)."""
    natoms, nB = beta.shape
    nstruct = int(atom_ptr.numel()) - 1
    dev, dt = beta.device, beta.dtype
    prec = 0 if dt == torch.float64 else 1
    if out is not None:
        forces, sa, stress = out
        forces = forces if dxdr is not None else None
        sa, stress = (sa, stress) if rdxdr_atom is not None else (None, None)
    else:
        forces = torch.empty((max(natoms, 1), 3), dtype=dt, device=dev) if dxdr is not None else None
        sa = torch.empty((max(natoms, 1), 6), dtype=dt, device=dev) if rdxdr_atom is not None else None
        stress = torch.empty((max(nstruct, 1), 6), dtype=dt, device=dev) if rdxdr_atom is not None else None
    own = status is None
    if own:
        status = torch.zeros(1, dtype=torch.int32, device=dev)
    keep = [t.contiguous() if t is not None else None for t in (beta, pair_ptr, seq, atom_struct, atom_ptr, dxdr,
                                                                  rdxdr_atom)]
    check(lib().so4_contract_dxdr(prec, natoms, nB, nstruct, _ptr(keep[3]), _ptr(keep[4]), _ptr(keep[1]),
                                  _ptr(keep[2]), _ptr(keep[5]), _ptr(keep[0]), _ptr(keep[6]), _ptr(forces), _ptr(sa),
                                  _ptr(stress), _ptr(status), _stream()), "so4_contract_dxdr")
    bits = int(status.item()) if own else 0
    if bits & (1 << _lib.SO4_ERR_REVERSE):
        raise ValueError("so4_contract_dxdr: a pair has no reverse pair (the pair list is not symmetric)")
    return (forces[:natoms] if forces is not None else None), (stress[:nstruct] if stress is not None else None)


def design_forces(X, ncols, nB, nelem, species, pair_ptr, seq, atom_struct, atom_ptr, dxdr, force_row):
    """Force rows of the linear design matrix X (so4_design_forces), in place."""
    natoms = int(species.numel())
    status = torch.zeros(1, dtype=torch.int32, device=X.device)
    check(lib().so4_design_forces(natoms, nB, nelem, _ptr(atom_struct), _ptr(atom_ptr), _ptr(pair_ptr), _ptr(seq),
                                  _ptr(species), _ptr(dxdr), _ptr(force_row), int(ncols), _ptr(X), _ptr(status),
                                  _stream()), "so4_design_forces")
    bits = int(status.item())
    if bits & (1 << _lib.SO4_ERR_REVERSE):
        raise ValueError("so4_design_forces: a pair has no reverse pair (the pair list is not symmetric)")
    if bits & (1 << _lib.SO4_ERR_ARG):
        raise ValueError("so4_design_forces: an element index is out of range")


def design_struct(X, ncols, nB, nelem, species, atom_ptr, x, rdxdr_atom, energy_row, stress_row):
    """Energy (count, sum x) and stress (-sum rdxdr_atom) rows per structure (so4_design_struct)."""
    nstruct = int(atom_ptr.numel()) - 1
    check(lib().so4_design_struct(nstruct, nB, nelem, _ptr(atom_ptr), _ptr(species), _ptr(x), _ptr(rdxdr_atom),
                                  _ptr(energy_row), _ptr(stress_row), int(ncols), _ptr(X), _stream()),
          "so4_design_struct")


def design_forces_q(X, ncols, nB, feat, nelem, species, pair_ptr, seq, atom_struct, atom_ptr, x, dxdr, force_row):
    """Force rows of the design matrix for the features feat (F, 2) i32 (so4_design_forces_q)."""
    natoms = int(species.numel())
    status = torch.zeros(1, dtype=torch.int32, device=X.device)
    check(lib().so4_design_forces_q(natoms, nB, int(feat.shape[0]), nelem, _ptr(feat), _ptr(atom_struct),
                                    _ptr(atom_ptr), _ptr(pair_ptr), _ptr(seq), _ptr(species), _ptr(x), _ptr(dxdr),
                                    _ptr(force_row), int(ncols), _ptr(X), _ptr(status), _stream()),
          "so4_design_forces_q")
    bits = int(status.item())
    if bits & (1 << _lib.SO4_ERR_REVERSE):
        raise ValueError("so4_design_forces_q: a pair has no reverse pair (the pair list is not symmetric)")
    if bits & (1 << _lib.SO4_ERR_ARG):
        raise ValueError("so4_design_forces_q: an element index is out of range")


def design_struct_q(X, ncols, nB, feat, nelem, species, atom_ptr, x, rdxdr_atom, energy_row, stress_row):
    """Energy and stress rows per structure for the features feat (so4_design_struct_q)."""
    nstruct = int(atom_ptr.numel()) - 1
    check(lib().so4_design_struct_q(nstruct, nB, int(feat.shape[0]), nelem, _ptr(feat), _ptr(atom_ptr), _ptr(species),
                                    _ptr(x), _ptr(rdxdr_atom), _ptr(energy_row), _ptr(stress_row), int(ncols),
                                    _ptr(X), _stream()), "so4_design_struct_q")


def forward32(tab, prm, nb: Neighbors, w_nb, w_site):
    """FP32 B (N,nB) and U_tot (N, n_half, 2) for the adjoint."""
    dev = w_nb.device
    x = torch.empty((max(nb.natoms, 1), tab.nB), dtype=torch.float32, device=dev)
    utot = torch.empty((max(nb.natoms, 1), tab.n_half, 2), dtype=torch.float32, device=dev)
    ws = torch.empty(max(lib().so4_forward32_workspace_size(tab.handle, nb.natoms), 1), dtype=torch.uint8, device=dev)
    check(lib().so4_forward32(tab.handle, C.byref(prm), nb.natoms, _ptr(w_nb), _ptr(w_site), _ptr(nb.img_ptr),
                              _ptr(nb.img_j), _ptr(nb.img_r), _ptr(utot), _ptr(x), _ptr(ws), ws.numel(), _stream()),
          "so4_forward32")
    return x[: nb.natoms], utot[: nb.natoms]


def adjoint32(tab, prm, nb: Neighbors, w_nb, utot, beta, workspace=None, eatom=None):
    """forces (N,3) f64 = -dE/dr and virial (S,3,3) f64 = sum r (x) dE/dr, for beta = dE/dB.
    With eatom (N,) the per-structure energy (S,) f64 = its fixed-order sum is returned too."""
    dev = utot.device
    beta = beta.to(torch.float32).contiguous()
    if eatom is not None:
        y = torch.empty((max(nb.natoms, 1), tab.n_half, 2), dtype=torch.float32, device=dev)
        g = torch.empty((max(nb.nimg, 1), 3), dtype=torch.float32, device=dev)
        L, st = lib(), _stream()
        check(L.so4_adjoint_y32(tab.handle, nb.natoms, _ptr(utot), _ptr(beta), _ptr(y), st), "so4_adjoint_y32")
        check(L.so4_adjoint_deidrj32(tab.handle, C.byref(prm), nb.natoms, _ptr(w_nb), _ptr(nb.img_ptr),
                                     _ptr(nb.img_j), _ptr(nb.img_r), nb.nimg, _ptr(y), _ptr(g), st),
              "so4_adjoint_deidrj32")
        return gather(nb, g, eatom.to(torch.float32).contiguous())
    forces = torch.empty((max(nb.natoms, 1), 3), dtype=torch.float64, device=dev)
    virial = torch.empty((max(nb.nstruct, 1), 3, 3), dtype=torch.float64, device=dev)
    need = lib().so4_adjoint_workspace_size(tab.handle, nb.natoms, nb.nimg)
    ws = workspace if (workspace is not None and workspace.numel() >= need) else torch.empty(need, dtype=torch.uint8, device=dev)
    check(lib().so4_adjoint32(tab.handle, C.byref(prm), nb.nstruct, _ptr(nb.atom_struct), _ptr(nb.atom_ptr_dev),
                              nb.natoms, _ptr(w_nb), _ptr(nb.img_ptr), _ptr(nb.img_j), _ptr(nb.img_r),
                              _ptr(nb.img_rev), nb.nimg, _ptr(utot), _ptr(beta), _ptr(forces), _ptr(virial),
                              _ptr(ws), ws.numel(), _stream()), "so4_adjoint32")
    return forces[: nb.natoms], virial[: nb.nstruct]


def gather(nb: Neighbors, g, eatom=None):
    """forces (N,3), virial (S,3,3) and, with eatom (N,) f32, energy (S,) -- all f64 and in a
    fixed summation order -- from the per-image dE/dr g (M,3) f32."""
    dev = g.device
    N = nb.natoms
    forces = torch.empty((max(N, 1), 3), dtype=torch.float64, device=dev)
    virial = torch.empty((max(nb.nstruct, 1), 3, 3), dtype=torch.float64, device=dev)
    energy = torch.empty(max(nb.nstruct, 1), dtype=torch.float64, device=dev) if eatom is not None else None
    part = torch.empty(lib().so4_gather_workspace_size(N), dtype=torch.uint8, device=dev)
    check(lib().so4_adjoint_gather(N, nb.nstruct, _ptr(nb.atom_ptr_dev), _ptr(nb.img_ptr), _ptr(nb.img_rev),
                                   _ptr(nb.img_r), _ptr(g), _ptr(eatom), _ptr(part), _ptr(forces), _ptr(virial),
                                   _ptr(energy), _stream()), "so4_adjoint_gather")
    return forces[:N], virial[: nb.nstruct], (energy[: nb.nstruct] if energy is not None else None)


def adjoint32_staged(tab, prm, nb: Neighbors, w_nb, utot, beta, mark=None, first=0):
    """adjoint32 as its three C-ABI stages (Y build, per-image contraction, gather) with
    caller-visible buffers; mark(i) is called between stages (for timing)."""
    dev = utot.device
    beta = beta.to(torch.float32).contiguous()
    N, M = nb.natoms, nb.nimg
    y = torch.empty((max(N, 1), tab.n_half, 2), dtype=torch.float32, device=dev)
    g = torch.empty((max(M, 1), 3), dtype=torch.float32, device=dev)
    L, st = lib(), _stream()
    check(L.so4_adjoint_y32(tab.handle, N, _ptr(utot), _ptr(beta), _ptr(y), st), "so4_adjoint_y32")
    if mark:
        mark(first + 1)
    check(L.so4_adjoint_deidrj32(tab.handle, C.byref(prm), N, _ptr(w_nb), _ptr(nb.img_ptr), _ptr(nb.img_j),
                                 _ptr(nb.img_r), M, _ptr(y), _ptr(g), st), "so4_adjoint_deidrj32")
    if mark:
        mark(first + 2)
    forces, virial, _ = gather(nb, g)
    return forces, virial


def jvp32(tab, prm, nb: Neighbors, w_nb, utot, v=None, G=None, workspace=None):
    """dB (N, nB) f32: the JVP of B along dr_m = (v_j - v_i) + G_s^T r_m (v (N,3), G (S,3,3) f64)."""
    dev = utot.device
    dB = torch.empty((max(nb.natoms, 1), tab.nB), dtype=torch.float32, device=dev)
    need = lib().so4_jvp_workspace_size(tab.handle, nb.natoms)
    ws = workspace if (workspace is not None and workspace.numel() >= need) else torch.empty(need, dtype=torch.uint8, device=dev)
    v = v.to(torch.float64).contiguous() if v is not None else None
    G = G.to(torch.float64).contiguous() if G is not None else None
    check(lib().so4_jvp32(tab.handle, C.byref(prm), _ptr(nb.atom_struct), nb.natoms, _ptr(w_nb), _ptr(nb.img_ptr),
                          _ptr(nb.img_j), _ptr(nb.img_r), _ptr(utot), _ptr(v), _ptr(G), _ptr(dB), _ptr(ws), ws.numel(),
                          _stream()), "so4_jvp32")
    return dB[: nb.natoms]


def adjoint_linear32(tab, prm, nb: Neighbors, w_nb, w_site, beta, workspace=None):
    """B (N,nB) f32, forces (N,3) f64, virial (S,3,3) f64 and energy (S,) f64 = sum beta.B for an
    energy linear in B (beta = dE/dB fixed), in one fused pass (Z computed once)."""
    dev = w_nb.device
    beta = beta.to(torch.float32).contiguous()
    x = torch.empty((max(nb.natoms, 1), tab.nB), dtype=torch.float32, device=dev)
    forces = torch.empty((max(nb.natoms, 1), 3), dtype=torch.float64, device=dev)
    virial = torch.empty((max(nb.nstruct, 1), 3, 3), dtype=torch.float64, device=dev)
    energy = torch.empty(max(nb.nstruct, 1), dtype=torch.float64, device=dev)
    need = lib().so4_linear_workspace_size(tab.handle, nb.natoms, nb.nimg)
    ws = workspace if (workspace is not None and workspace.numel() >= need) else torch.empty(need, dtype=torch.uint8, device=dev)
    check(lib().so4_adjoint_linear32(tab.handle, C.byref(prm), nb.nstruct, _ptr(nb.atom_struct), _ptr(nb.atom_ptr_dev),
                                     nb.natoms, _ptr(w_nb), _ptr(w_site), _ptr(nb.img_ptr), _ptr(nb.img_j),
                                     _ptr(nb.img_r), _ptr(nb.img_rev), nb.nimg, _ptr(beta), _ptr(x), _ptr(forces),
                                     _ptr(virial), _ptr(energy), _ptr(ws), ws.numel(), _stream()),
          "so4_adjoint_linear32")
    return x[: nb.natoms], forces[: nb.natoms], virial[: nb.nstruct], energy[: nb.nstruct]


def linear_staged(tab, prm, nb: Neighbors, w_nb, w_site, beta, mark=None, first=0):
    """adjoint_linear32 as its C-ABI stages (U_tot; B and Y; per-image dE/dr; gather),
    with mark(i) called between stages (for timing).  Returns (x, forces, virial, energy)."""
    dev = w_nb.device
    beta = beta.to(torch.float32).contiguous()
    N, M = nb.natoms, nb.nimg
    utot = torch.empty((max(N, 1), tab.n_half, 2), dtype=torch.float32, device=dev)
    x = torch.empty((max(N, 1), tab.nB), dtype=torch.float32, device=dev)
    y = torch.empty((max(N, 1), tab.n_half, 2), dtype=torch.float32, device=dev)
    bc = torch.empty((tab.n_bsec, max(N, 1)), dtype=torch.float32, device=dev)
    eatom = torch.empty(max(N, 1), dtype=torch.float32, device=dev)
    g = torch.empty((max(M, 1), 3), dtype=torch.float32, device=dev)
    L, st = lib(), _stream()
    check(L.so4_utot32(tab.handle, C.byref(prm), N, _ptr(w_nb), _ptr(w_site), _ptr(nb.img_ptr), _ptr(nb.img_j),
                       _ptr(nb.img_r), _ptr(utot), st), "so4_utot32")
    if mark:
        mark(first + 1)
    check(L.so4_linear_by32(tab.handle, N, _ptr(utot), _ptr(beta), _ptr(x), _ptr(y), _ptr(bc), _ptr(eatom), st),
          "so4_linear_by32")
    if mark:
        mark(first + 2)
    check(L.so4_adjoint_deidrj32(tab.handle, C.byref(prm), N, _ptr(w_nb), _ptr(nb.img_ptr), _ptr(nb.img_j),
                                 _ptr(nb.img_r), M, _ptr(y), _ptr(g), st), "so4_adjoint_deidrj32")
    if mark:
        mark(first + 3)
    forces, virial, energy = gather(nb, g, eatom)
    return x[:N], forces, virial, energy
