"""so4_adjoint32_noalloc: the adjoint for callers that cannot allocate device memory.

Callers such as an MD engine's force plugin (handed only input and output
buffers) or code running while a pre-reserved pool owns the GPU's memory cannot
call cudaMalloc when they need forces.  This entry point takes its scratch from
a fixed 64 MiB device array instead of a workspace.  The test calls it through
the C ABI twice in a row (the second call reuses the array left by the first)
and checks forces and virial against so4_adjoint32 within the FP32 adjoint
tolerance used by the other GPU tests (2e-4 relative); it also checks that an
oversized problem is rejected.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from pyxtal_ff_gb300 import _lib, engine
from pyxtal_ff_gb300 import structures as S

pytestmark = pytest.mark.gpu

TOL = 2e-4


def _rel(a, b):
    a, b = a.cpu().numpy(), b.cpu().numpy()
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _setup(lmax=4, rc=5.0):
    structs = [S.diamond_si(3, 3, 2, sigma=0.1, rng=np.random.default_rng(21)), S.sio2_random(n_si=8, seed=22)]
    pos = np.concatenate([s.positions for s in structs])
    cells = np.stack([s.get_cell() for s in structs])
    pbc = np.ones((2, 3), np.int32)
    ptr = np.concatenate([[0], np.cumsum([len(s) for s in structs])])
    numbers = np.concatenate([s.numbers for s in structs])
    symbols = sum([list(s.symbols) for s in structs], [])
    tab = engine.tables(2 * lmax)
    prm = engine.params(2 * lmax, rc, 0.99363, "cosine")
    nb = engine.build_neighbors(torch.from_numpy(pos).cuda(), cells, pbc, ptr, rc)
    w_nb, w_site = engine.site_weights("SNAP", numbers, symbols, {"Si": 1.0, "O": 0.5})
    w_nb, w_site = torch.from_numpy(w_nb).cuda(), torch.from_numpy(w_site).cuda()
    x, utot = engine.forward32(tab, prm, nb, w_nb, w_site)
    return tab, prm, nb, w_nb, utot


def _noalloc(tab, prm, nb, w_nb, utot, beta):
    forces = torch.empty((nb.natoms, 3), dtype=torch.float64, device="cuda")
    virial = torch.empty((nb.nstruct, 3, 3), dtype=torch.float64, device="cuda")
    p = engine._ptr
    rc = _lib.lib().so4_adjoint32_noalloc(tab.handle, C.byref(prm), nb.nstruct, p(nb.atom_struct),
                                          p(nb.atom_ptr_dev), nb.natoms, p(w_nb), p(nb.img_ptr), p(nb.img_j),
                                          p(nb.img_r), p(nb.img_rev), nb.nimg, p(utot), p(beta), p(forces),
                                          p(virial), engine._stream())
    assert rc == _lib.SO4_OK, rc
    return forces, virial


def test_noalloc_matches_workspace_adjoint_on_two_calls(cuda_device):
    tab, prm, nb, w_nb, utot = _setup()
    for seed in (1, 2):
        beta = torch.from_numpy(np.random.default_rng(seed).normal(0, 0.01, size=(nb.natoms, tab.nB))).float().cuda()
        f_ref, v_ref = engine.adjoint32(tab, prm, nb, w_nb, utot, beta)
        f, v = _noalloc(tab, prm, nb, w_nb, utot, beta)
        torch.cuda.synchronize()
        assert _rel(f, f_ref) < TOL and _rel(v, v_ref) < TOL


def test_noalloc_rejects_problems_beyond_its_scratch(cuda_device):
    tab, prm, nb, w_nb, utot = _setup(lmax=2, rc=4.0)
    too_many_images = (64 << 20) // 12 + 1
    rc = _lib.lib().so4_adjoint32_noalloc(tab.handle, C.byref(prm), 1, None, None, 10, None, None, None, None, None,
                                          too_many_images, None, None, None, None, None)
    assert rc == _lib.SO4_ERR_TOO_LARGE
