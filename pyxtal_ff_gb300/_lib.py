"""ctypes binding of libso4gb300.so (the C ABI of include/so4_gb300.h).

The library is loaded lazily on first use, never at import, so importing the
package creates no CUDA context and stays fork-safe (the reference's callers
run descriptors in a multiprocessing.Pool, pyxtal_ff/utilities/__init__.py:145).
There is no CPU fallback: if the library is missing, every entry point raises.
"""
import ctypes as C
import os

from . import build_ext

SO4_OK = 0
SO4_ERR_ARG = 1
SO4_ERR_UNSUPPORTED = 2
SO4_ERR_CUDA = 3
SO4_ERR_CAPACITY = 4
SO4_ERR_NONFINITE = 5
SO4_ERR_WORKSPACE = 6
SO4_ERR_NO_NEIGHBOR = 7
SO4_ERR_REVERSE = 8
SO4_ERR_TOO_LARGE = 9
SO4_ERR_SLOTS = 10

_MESSAGES = {
    SO4_ERR_ARG: "invalid argument",
    SO4_ERR_UNSUPPORTED: "not supported by the compiled kernels",
    SO4_ERR_CUDA: "a CUDA runtime call failed",
    SO4_ERR_CAPACITY: "an image offset or a count exceeds the encodable range",
    SO4_ERR_NONFINITE: "non-finite positions or cell",
    SO4_ERR_WORKSPACE: "workspace too small",
    SO4_ERR_NO_NEIGHBOR: "an atom has no neighbour within rcut",
    SO4_ERR_REVERSE: "neighbour list is not symmetric",
    SO4_ERR_TOO_LARGE: "problem exceeds the fixed 64 MiB scratch of so4_adjoint32_noalloc",
    SO4_ERR_SLOTS: "an atom has more images than the per-atom key slots",
}


class SO4Error(RuntimeError):
    def __init__(self, code, where):
        self.code = code
        super().__init__("%s: %s (status %d)" % (where, _MESSAGES.get(code, "error"), code))


def check(code, where):
    if code != SO4_OK:
        if code == SO4_ERR_ARG:
            raise ValueError("%s: %s" % (where, _MESSAGES[code]))
        if code == SO4_ERR_UNSUPPORTED:
            raise NotImplementedError("%s: %s" % (where, _MESSAGES[code]))
        raise SO4Error(code, where)


class Geom(C.Structure):
    _fields_ = [("cell", C.c_double * 9), ("inv", C.c_double * 9), ("vol", C.c_double),
                ("nbin", C.c_int * 3), ("mshift", C.c_int * 3), ("pbc", C.c_int * 3),
                ("bin_base", C.c_int), ("atom_base", C.c_int), ("natoms", C.c_int)]


class Params(C.Structure):
    _fields_ = [("twol", C.c_int), ("cutoff_id", C.c_int), ("rcut", C.c_double), ("rfac0", C.c_double)]


class Tuning(C.Structure):
    """so4_tuning: launch shapes of the FP32 kernels (0 = the default)."""
    _fields_ = [("wkmax", C.c_int), ("rev_threads", C.c_int), ("utot_warps", C.c_int), ("rev_pair", C.c_int),
                ("zw_atoms", C.c_int), ("zw_threads", C.c_int)]


_lib = None
_vp, _i, _sz, _i64, _d = C.c_void_p, C.c_int, C.c_size_t, C.c_int64, C.c_double


def lib():
    """The loaded library; builds it first when the in-tree copy is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    path = build_ext.LIB
    if not os.path.exists(path) or build_ext._stale(path, [os.path.join(build_ext.CSRC, s) for s in build_ext.SOURCES]):
        path = build_ext.build()
    L = C.CDLL(path)
    sig = {
        "so4_version": (C.c_char_p, []),
        "so4_tables_create": (_i, [_i, _i, C.POINTER(_vp)]),
        "so4_tables_create_tuned": (_i, [_i, _i, C.POINTER(Tuning), C.POINTER(_vp)]),
        "so4_tables_get_tuning": (_i, [_vp, C.POINTER(Tuning)]),
        "so4_tables_destroy": (_i, [_vp]),
        "so4_tables_sizes": (_i, [_vp, C.POINTER(_i)]),
        "so4_tables_export": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "so4_geometry": (_i, [_vp, _vp, _vp, _i, _d, _vp, C.POINTER(_i)]),
        "so4_nl_workspace_size": (_sz, [_i, _i, _i64]),
        "so4_nl_count": (_i, [_vp, _i, _i, _vp, _vp, _i, _d, _vp, _vp, _sz, _vp]),
        "so4_nl_fill": (_i, [_vp, _i, _i, _vp, _vp, _i, _d, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_nl_pairs": (_i, [_vp, _i, _vp, _i, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp,
                              _sz, _vp]),
        "so4_status_read": (_i, [_vp, _sz, _vp, C.POINTER(_i)]),
        "so4_nl_count_keys": (_i, [_vp, _i, _i, _vp, _vp, _i, _d, _i, _vp, _vp, _sz, _vp]),
        "so4_nl_sort": (_i, [_vp, _i, _i, _vp, _vp, _i, _vp, _i64, _i, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_nl_bins": (_i, [_vp, _i, _i, _vp, _vp, _i, _i, _vp, _sz, _vp]),
        "so4_nl_count_keys_range": (_i, [_vp, _i, _i, _vp, _vp, _i, _d, _i, _i, _i, _vp, _sz, _vp]),
        "so4_nl_scan_range": (_i, [_i, _i, _i, _i, _i, _vp, _vp, _sz, _vp]),
        "so4_nl_sort_range": (_i, [_vp, _i, _i, _vp, _vp, _i, _i, _i, _vp, _i64, _i, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_nl_summary": (_i, [_vp, _vp, _i, _vp, _sz, _vp, C.POINTER(_i)]),
        "so4_plain_workspace_size": (_sz, [_vp, _i]),
        "so4_plain": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                           _i, _i, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_rdxdr_atom": (_i, [_i, _vp, _vp, _i, _i, _vp, _vp]),
        "so4_contract_dxdr": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "so4_design_forces": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, _vp, _vp, _vp]),
        "so4_design_struct": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, _vp, _vp]),
        "so4_design_forces_q": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, _vp,
                                     _vp, _vp]),
        "so4_design_struct_q": (_i, [_i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_int64, _vp, _vp]),
        "so4_forward32_workspace_size": (_sz, [_vp, _i]),
        "so4_forward32": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_adjoint_workspace_size": (_sz, [_vp, _i, _i64]),
        "so4_adjoint_y32": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
        "so4_adjoint_deidrj32": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _vp, _vp, _i64, _vp, _vp, _vp]),
        "so4_gather_workspace_size": (_sz, [_i]),
        "so4_adjoint_gather": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "so4_launch_count": (C.c_longlong, []),
        "so4_set_pdl": (C.c_int, [C.c_int]),
        "so4_peak_fma": (_i, [_i, _i, _i, _vp, C.POINTER(C.c_double), _vp]),
        "so4_jvp_workspace_size": (_sz, [_vp, _i]),
        "so4_linear_workspace_size": (_sz, [_vp, _i, _i64]),
        "so4_utot32": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "so4_linear_by32": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "so4_adjoint_linear32": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i64,
                                      _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_jvp32": (_i, [_vp, C.POINTER(Params), _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _sz, _vp]),
        "so4_adjoint32_noalloc": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _i64, _vp,
                                       _vp, _vp, _vp, _vp]),
        "so4_adjoint32": (_i, [_vp, C.POINTER(Params), _i, _vp, _vp, _i, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp,
                               _vp, _vp, _vp, _sz, _vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def exported_symbols():
    """Names the C ABI header declares (used by the load test)."""
    hdr = os.path.join(os.path.dirname(build_ext.HERE), "include", "so4_gb300.h")
    import re
    names = re.findall(r"^\s*(?:int|size_t|long long|const char \*)\s*\**\s*(so4_\w+)\s*\(", open(hdr).read(),
                       re.M)
    return sorted(set(names))
