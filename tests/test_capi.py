"""The C-ABI library builds, loads and exports every symbol include/so4_gb300.h declares
(no compute calls: this runs without a GPU)."""
import ctypes as C

import numpy as np
import pytest

from pyxtal_ff_gb300 import _lib


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = _lib.exported_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_string():
    assert b"sm_103a" in _lib.lib().so4_version()


def test_geometry_host_function():
    from pyxtal_ff_gb300 import engine
    cells = np.stack([5.43 * np.eye(3), 20.0 * np.eye(3)])
    raw, vol, nbins = engine.geometry(cells, [[1, 1, 1], [1, 1, 0]], [0, 8, 10], 4.9)
    g = (_lib.Geom * 2).from_buffer_copy(raw.tobytes())
    assert np.allclose(vol, [5.43 ** 3, 8000.0])
    assert list(g[0].nbin) == [1, 1, 1] and list(g[0].mshift) == [1, 1, 1]
    assert list(g[1].nbin) == [4, 4, 1] and list(g[1].mshift) == [1, 1, 0]
    assert g[1].bin_base == 1 and nbins == 17 and g[1].atom_base == 8


def test_geometry_rejects_bad_cells():
    from pyxtal_ff_gb300 import engine
    with pytest.raises(ValueError):
        engine.geometry(np.zeros((1, 3, 3)), [[1, 1, 1]], [0, 1], 4.0)
    with pytest.raises(ValueError):
        engine.geometry(np.full((1, 3, 3), np.nan), [[1, 1, 1]], [0, 1], 4.0)
    with pytest.raises(ValueError):
        engine.geometry(np.eye(3)[None], [[1, 1, 1]], [0, 1], -1.0)


def test_workspace_size_queries_grow():
    L = _lib.lib()
    a = L.so4_nl_workspace_size(100, 10, 0)
    b = L.so4_nl_workspace_size(100, 10, 10000)
    assert b > a >= 256


def test_tables_need_no_gpu_for_argument_errors():
    h = C.c_void_p()
    assert _lib.lib().so4_tables_create(-1, 0, C.byref(h)) == _lib.SO4_ERR_ARG
    assert _lib.lib().so4_tables_create(40, 0, C.byref(h)) == _lib.SO4_ERR_UNSUPPORTED
