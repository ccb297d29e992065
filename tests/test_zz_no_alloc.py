"""so4_adjoint32_noalloc: the adjoint for callers that cannot allocate device memory.

Callers such as an MD engine's force plugin (handed only input and output
buffers) or code running while a pre-reserved pool owns the GPU's memory cannot
call cudaMalloc when they need forces.  This entry point takes its scratch from
a fixed 64 MiB device array instead of a workspace.

The test calls it through the C ABI.  A first call on a larger problem (another
layout of the scratch) leaves the array dirty; then two calls in a row on the
test problem must give forces and virial bitwise equal to so4_adjoint32 (both run
the same deterministic kernels in the same order, so any scratch-carving or
offset error shows), and neither torch's allocator nor the device's free memory
may change across those calls.  An oversized problem must be rejected.  The file
is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from pyxtal_ff_gb300 import _lib, engine
from pyxtal_ff_gb300 import structures as S

pytestmark = pytest.mark.gpu


def _setup(structs, lmax=4, rc=5.0):
    pos = np.concatenate([s.positions for s in structs])
    cells = np.stack([s.get_cell() for s in structs])
    pbc = np.ones((len(structs), 3), np.int32)
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


def _beta(nb, tab, seed):
    return torch.from_numpy(np.random.default_rng(seed).normal(0, 0.01, size=(nb.natoms, tab.nB))).float().cuda()


def _noalloc(tab, prm, nb, w_nb, utot, beta, forces, virial):
    p = engine._ptr
    rc = _lib.lib().so4_adjoint32_noalloc(tab.handle, C.byref(prm), nb.nstruct, p(nb.atom_struct),
                                          p(nb.atom_ptr_dev), nb.natoms, p(w_nb), p(nb.img_ptr), p(nb.img_j),
                                          p(nb.img_r), p(nb.img_rev), nb.nimg, p(utot), p(beta), p(forces),
                                          p(virial), engine._stream())
    assert rc == _lib.SO4_OK, rc


def _outputs(nb):
    return (torch.empty((nb.natoms, 3), dtype=torch.float64, device="cuda"),
            torch.empty((nb.nstruct, 3, 3), dtype=torch.float64, device="cuda"))


def test_noalloc_matches_workspace_adjoint_on_two_calls(cuda_device):
    # a larger problem first: the array then holds another layout's data when the test problem runs
    big = _setup([S.diamond_si(4, 4, 3, sigma=0.1, rng=np.random.default_rng(23))])
    bf, bv = _outputs(big[2])
    _noalloc(*big, _beta(big[2], big[0], 3), bf, bv)
    tab, prm, nb, w_nb, utot = _setup([S.diamond_si(3, 3, 2, sigma=0.1, rng=np.random.default_rng(21)),
                                       S.sio2_random(n_si=8, seed=22)])
    betas = [_beta(nb, tab, seed) for seed in (1, 2)]
    refs = [engine.adjoint32(tab, prm, nb, w_nb, utot, b) for b in betas]
    outs = [_outputs(nb) for _ in betas]
    torch.cuda.synchronize()
    alloc0, free0 = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    for b, (f, v) in zip(betas, outs):
        _noalloc(tab, prm, nb, w_nb, utot, b, f, v)
    torch.cuda.synchronize()
    alloc1, free1 = torch.cuda.memory_allocated(), torch.cuda.mem_get_info()[0]
    assert alloc1 == alloc0 and free1 == free0, (alloc0, alloc1, free0, free1)
    for (f, v), (f_ref, v_ref) in zip(outs, refs):
        assert torch.equal(f, f_ref), float((f - f_ref).abs().max())
        assert torch.equal(v, v_ref), float((v - v_ref).abs().max())


def test_noalloc_rejects_problems_beyond_its_scratch(cuda_device):
    tab, prm, nb, w_nb, utot = _setup([S.diamond_si(1, 1, 1, sigma=0.1, rng=np.random.default_rng(24))],
                                      lmax=2, rc=4.0)
    too_many_images = (64 << 20) // 12 + 1
    rc = _lib.lib().so4_adjoint32_noalloc(tab.handle, C.byref(prm), 1, None, None, 10, None, None, None, None, None,
                                          too_many_images, None, None, None, None, None)
    assert rc == _lib.SO4_ERR_TOO_LARGE
