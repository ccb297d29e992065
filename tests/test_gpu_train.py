"""Force matching on the adjoint path (512 Si structures of 8-64 atoms, lmax 3).

- The gradient of the training loss w.r.t. the model weights, computed with the
  adjoint forces and the JVP backward (FP32 kernels), matches the same loss built
  from the FP64 plain path (dxdr contracted with dE/dB by the reference's formula,
  differentiated by torch) to 1e-3 relative.
- One optimiser step on the full config (512 structures of 8-64 atoms) runs and a
  few steps reduce the loss.
- The Stillinger-Weber targets: forces are -dE/dr (central differences).
"""
import numpy as np
import pytest
import torch

from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.calculator import Batch, SO4Calculator, contract_plain
from pyxtal_ff_gb300.train import ForceMatching, stillinger_weber

pytestmark = pytest.mark.gpu


def _structs(n, seed):
    return S.si_batch(n, seed=seed, sizes=range(1, 9), max_cells=8, strain=0.04, sigma=0.1)


def test_stillinger_weber_forces_are_energy_gradient(cuda_device):
    structs = _structs(3, 40)
    b = Batch(structs)
    e, f = stillinger_weber(b)
    h = 1e-5
    for a, c in [(0, 0), (5, 2), (b.natoms - 1, 1)]:
        pp, pm = b.positions.copy(), b.positions.copy()
        pp[a, c] += h
        pm[a, c] -= h
        bp, bm = Batch(structs), Batch(structs)
        bp.positions, bm.positions = pp, pm
        fd = -(stillinger_weber(bp)[0].sum() - stillinger_weber(bm)[0].sum()).item() / (2 * h)
        assert abs(fd - f[a, c].item()) < 1e-6 * max(1.0, abs(fd))


def test_training_gradient_matches_fp64_plain_path(cuda_device):
    structs = _structs(24, 41)
    fm = ForceMatching(structs, lmax=3, rcut=4.9, seed=4)
    L = fm.loss()
    grads = torch.autograd.grad(L, list(fm.model.parameters()))
    # FP64 reference: same model in FP64, forces from the plain path's dxdr
    b = fm.batch
    calc = SO4Calculator(lmax=3, rcut=4.9, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
    d = calc.descriptors(b, precision="fp64")
    m64 = type(fm.model)(d["x"].shape[1], 1, seed=4, dtype=torch.float64).cuda()
    m64.load_state_dict({k: v.double() for k, v in fm.model.state_dict().items()})
    xg = d["x"].clone().requires_grad_(True)
    e_atom = m64(xg, fm.species)
    beta = torch.autograd.grad(e_atom.sum(), xg, create_graph=True)[0]
    c = contract_plain(d["x"], d["dxdr"], d["rdxdr"], d["seq"], d["pair_ptr"], b.atom_ptr, beta, b.volumes)
    energy = torch.zeros(b.nstruct, dtype=torch.float64, device="cuda").index_add(0, fm.struct, e_atom)
    L64 = torch.mean(((energy - fm.e_ref) / fm.natoms_s) ** 2) + 0.1 * torch.mean((c["forces"] - fm.f_ref) ** 2)
    g64 = torch.autograd.grad(L64, list(m64.parameters()))
    assert abs(L.item() - L64.item()) <= 1e-4 * abs(L64.item())
    for g, r in zip(grads, g64):
        err = (g.double() - r).abs().max().item() / max(r.abs().max().item(), 1e-30)
        assert err < 1e-3, err


def test_512_structure_training_step_runs_and_loss_decreases(cuda_device):
    structs = _structs(512, 4)
    fm = ForceMatching(structs, lmax=3, rcut=4.9, seed=4, lr=3e-3)
    losses = [fm.step().item() for _ in range(5)]
    print("training atoms", fm.batch.natoms, "losses", ["%.4g" % v for v in losses])
    assert np.all(np.isfinite(losses)) and losses[-1] < losses[0]


def test_captured_training_step_matches_eager(cuda_device):
    # two species so the per-species model path is captured too
    structs = _structs(24, 7) + [S.sio2_random(n_si=4, seed=8)]
    targets = None
    fa = ForceMatching(structs, lmax=3, rcut=4.9, seed=4, lr=3e-3, weights={"Si": 1.0, "O": 0.6})
    targets = (fa.e_ref, fa.f_ref)
    fb = ForceMatching(structs, lmax=3, rcut=4.9, seed=4, lr=3e-3, weights={"Si": 1.0, "O": 0.6}, targets=targets)
    for _ in range(3):
        fa.step()
    fb.capture(warmup=3)  # the warm-up steps are real steps: both models have taken three
    for _ in range(4):
        la, lb = fa.step().item(), fb.step().item()
        assert abs(la - lb) <= 1e-6 * abs(la), (la, lb)
    for pa, pb in zip(fa.model.parameters(), fb.model.parameters()):
        assert (pa - pb).abs().max().item() <= 1e-5 * max(pa.abs().max().item(), 1.0)
