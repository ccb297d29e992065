"""The batched and autograd workloads at full size on the GPU.

- 256 Si supercells (n_i in {1,2,3}, strain U(-0.03,0.03), sigma 0.08, seed 1), lmax 3,
  rcut 4.9: FP32 plain x/dxdr/rdxdr vs the FP64 plain path of the same batch (which is
  itself checked against the oracle at 1e-10), errors reported; four structures also
  against the oracle.
- SiO2 648 atoms (2.2 g/cm^3, seed 2), lmax 4, rcut 5.0, weights Si 1.0 / O 0.5,
  per-species MLP 2x16 tanh (Xavier, seed 3): autograd forces vs central finite
  differences (h = 1e-4 A, FP64 energies) on 20 atoms and vs the FP64 dxdr . dE/dB.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyxtal_ff_gb300 import engine, ops
from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.calculator import Batch, SO4Calculator, contract_plain
from tests import goldens as G

pytestmark = pytest.mark.gpu


def test_256_si_supercells_batched_fp32_plain(cuda_device):
    structs = S.si_batch(256, seed=1, sizes=(1, 2, 3), strain=0.03, sigma=0.08)
    batch = Batch(structs)
    calc = SO4Calculator(lmax=3, rcut=4.9, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
    d64 = calc.descriptors(batch, precision="fp64")
    d32 = calc.descriptors(batch, precision="fp32")
    ex = G.rel_err(d32["x"].cpu().numpy(), d64["x"].cpu().numpy())
    ed = G.rel_err(d32["dxdr"].cpu().numpy(), d64["dxdr"].cpu().numpy())
    er = G.rel_err(d32["rdxdr"].cpu().numpy(), d64["rdxdr"].cpu().numpy())
    print("batched atoms", batch.natoms, "pairs", d64["seq"].shape[0], "rel err x %.2e dxdr %.2e rdxdr %.2e" % (ex, ed, er))
    assert ex < 2e-5 and ed < 2e-4 and er < 2e-4
    pptr = d64["pair_ptr"].cpu().numpy()
    for s in (0, 17, 100, 255):
        a0, a1 = batch.atom_ptr[s], batch.atom_ptr[s + 1]
        ref = O.descriptor(structs[s], kind="SNAP", lmax=3, rcut=4.9, weights={"Si": 1.0}, rfac0=1.0, stress=True)
        assert G.rel_err(d64["x"][a0:a1].cpu().numpy(), ref["x"]) < 1e-10
        assert G.rel_err(d64["dxdr"][pptr[a0]:pptr[a1]].cpu().numpy(), ref["dxdr"]) < 1e-10


class SpeciesMLP(torch.nn.Module):
    """Per-species MLP on B: nB -> 16 -> 16 -> 1, tanh, Xavier-uniform from a seed."""

    def __init__(self, nB, nspecies, seed, dtype=torch.float32):
        super().__init__()
        g = torch.Generator().manual_seed(seed)
        self.layers = torch.nn.ModuleList()
        for _ in range(nspecies):
            seq = torch.nn.Sequential(torch.nn.Linear(nB, 16), torch.nn.Tanh(), torch.nn.Linear(16, 16),
                                      torch.nn.Tanh(), torch.nn.Linear(16, 1))
            for m in seq:
                if isinstance(m, torch.nn.Linear):
                    torch.nn.init.xavier_uniform_(m.weight, generator=g)
                    torch.nn.init.zeros_(m.bias)
            self.layers.append(seq.to(dtype))

    def forward(self, x, species):
        out = torch.zeros(x.shape[0], dtype=x.dtype, device=x.device)
        for s, net in enumerate(self.layers):
            m = species == s
            if m.any():
                out[m] = net(x[m]).squeeze(-1)
        return out


def test_sio2_648_autograd_forces(cuda_device):
    atoms = S.sio2_random(n_si=216, density=2.2, dmin=1.4, seed=2)
    w = {"Si": 1.0, "O": 0.5}
    batch = Batch([atoms], species_order=["O", "Si"])
    species = torch.from_numpy(batch.species).cuda()
    pos = torch.from_numpy(batch.positions).cuda()
    ctx = ops.Context.build(pos, batch.cells, batch.pbc, batch.atom_ptr, batch.numbers, batch.symbols, lmax=4,
                            rcut=5.0, kind="SNAP", weights=w)
    model = SpeciesMLP(55, 2, seed=3).cuda()
    p = pos.clone().requires_grad_(True)
    x = ops.SO4Descriptor.apply(p, ctx)
    E = model(x, species).sum()
    E.backward()
    F_auto = -p.grad.cpu().numpy()
    # FP64 energy for finite differences: FP64 plain B + the same MLP in FP64
    model64 = SpeciesMLP(55, 2, seed=3, dtype=torch.float64).cuda()
    model64.load_state_dict({k: v.double() for k, v in model.state_dict().items()})
    calc = SO4Calculator(lmax=4, rcut=5.0, kind="SNAP", weights=w, rfac0=0.99363)

    def energy64(positions):
        d = calc.descriptors(batch, positions, precision="fp64", derivative=False, stress=False)
        with torch.no_grad():
            return float(model64(d["x"], species).sum())

    h = 1e-4
    rng = np.random.default_rng(20)
    atoms_sel = rng.choice(len(atoms), size=20, replace=False)
    err_fd = 0.0
    for a in atoms_sel:
        for c in range(3):
            pp = batch.positions.copy()
            pm = batch.positions.copy()
            pp[a, c] += h
            pm[a, c] -= h
            fd = -(energy64(pp) - energy64(pm)) / (2 * h)
            err_fd = max(err_fd, abs(fd - F_auto[a, c]))
    # against the FP64 dxdr contracted with the same dE/dB
    d = calc.descriptors(batch, precision="fp64")
    xb = d["x"].clone().requires_grad_(True)
    beta64 = torch.autograd.grad(model64(xb, species).sum(), xb)[0]
    c = contract_plain(d["x"], d["dxdr"], d["rdxdr"], d["seq"], d["pair_ptr"], batch.atom_ptr, beta64, batch.volumes)
    err_dx = float(np.abs(c["forces"].cpu().numpy() - F_auto).max())
    fmax = float(np.abs(F_auto).max())
    print("SiO2 max|F| %.3f eV/A, FD err %.2e, dxdr.beta err %.2e" % (fmax, err_fd, err_dx))
    assert err_dx <= 1e-4 * max(1.0, fmax)
    assert err_fd <= 1e-3 * max(1.0, fmax)
