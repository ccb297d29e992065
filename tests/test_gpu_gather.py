"""The gather stage (so4_adjoint_gather): forces, per-structure virial and energy
from per-image dE/dr, against an FP64 numpy sum of the same terms.

Structure sizes are chosen so that structures start and end inside the gather's
8-atom chunks, span several chunks, or hold a single atom, which covers every
branch of the chunk / head bookkeeping.  Forces are compensated FP32 sums
(tolerance 1e-12 of the largest force), the per-atom virial is FP32 before the
FP64 sum over atoms (1e-6 of the largest component), the energy an FP64 sum of
FP32 values (1e-12).
"""
import numpy as np
import pytest
import torch

from pyxtal_ff_gb300 import engine
from pyxtal_ff_gb300 import structures as S

pytestmark = pytest.mark.gpu


def _reference(nb, g, eatom):
    img_ptr = nb.img_ptr.cpu().numpy().astype(np.int64)
    rev = nb.img_rev.cpu().numpy().astype(np.int64)
    r = nb.img_r.cpu().numpy()
    gg = g.cpu().numpy().astype(np.float64)
    e = eatom.cpu().numpy().astype(np.float64)
    N, ptr = nb.natoms, np.asarray(nb.atom_ptr)
    centre = np.repeat(np.arange(N), np.diff(img_ptr))
    forces = np.zeros((N, 3))
    np.add.at(forces, centre, gg - gg[rev])
    vat = np.zeros((N, 3, 3))
    np.add.at(vat, centre, r[:, :, None] * gg[:, None, :])
    vir = np.stack([vat[a0:a1].sum(0) for a0, a1 in zip(ptr[:-1], ptr[1:])])
    en = np.array([e[a0:a1].sum() for a0, a1 in zip(ptr[:-1], ptr[1:])])
    return forces, vir, en


@pytest.mark.parametrize("sizes", [(3, 9, 1, 17, 8, 5, 16, 2), (64,), (1, 1, 1), (8, 8, 7, 9)])
def test_gather_ragged_structures(cuda_device, sizes):
    rng = np.random.default_rng(sum(sizes))
    structs = []
    for n in sizes:
        # n atoms in a cubic box small enough that every atom has neighbours within 4.0 A
        L = 3.0 * max(n, 2) ** (1.0 / 3.0)
        structs.append(S.Atoms([14] * n, rng.uniform(0, L, size=(n, 3)), np.eye(3) * L, pbc=True))
    pos = np.concatenate([s.positions for s in structs])
    cells = np.stack([s.cell for s in structs])
    pbc = np.ones((len(structs), 3), np.int32)
    ptr = np.concatenate([[0], np.cumsum(sizes)])
    nb = engine.build_neighbors(torch.from_numpy(pos).cuda(), cells, pbc, ptr, 4.0)
    g = torch.from_numpy(rng.normal(size=(nb.nimg, 3))).float().cuda()
    eatom = torch.from_numpy(rng.normal(size=nb.natoms)).float().cuda()
    f, v, e = engine.gather(nb, g, eatom)
    f_ref, v_ref, e_ref = _reference(nb, g, eatom)
    assert np.abs(f.cpu().numpy() - f_ref).max() <= 1e-12 * np.abs(f_ref).max()
    assert np.abs(v.cpu().numpy() - v_ref).max() <= 1e-6 * np.abs(v_ref).max()
    assert np.abs(e.cpu().numpy() - e_ref).max() <= 1e-12 * np.abs(e_ref).max()
    # fixed order: a second call is bitwise identical
    f2, v2, e2 = engine.gather(nb, g, eatom)
    assert torch.equal(f, f2) and torch.equal(v, v2) and torch.equal(e, e2)
    # without a per-atom energy the virial and forces are unchanged
    f3, v3, e3 = engine.gather(nb, g)
    assert e3 is None and torch.equal(f, f3) and torch.equal(v, v3)
