"""The 32,000-atom workload (diamond Si 20x20x10, a = 5.43 A, sigma 0.1 A from seed 5;
SO4 lmax 4, rcut 5.0 A, unit weight; energy linear in B with coefficients N(0, 0.01)
from seed 6) against the FP64 oracle on every centre.

This is the first size at which image counts, grid sizes and the int32 image offsets
run at scale (0.93 M images), so the neighbour list, the GPU FP64 plain path and the
FP32 adjoint are each compared with the oracle here, not only on small cells:
- neighbour list: image counts per centre, the seq pairs and the FP64 image vectors
  bit-exact;
- FP64 plain path (B, dxdr and per-pair rdxdr, contracted with beta as the
  reference's consumers do): 1e-10 relative on B, forces and stress;
- FP32 adjoint (the captured step of the benchmark): force error <= 1e-4 eV/A and
  stress error <= 1e-3 GPa, B 2e-5 relative, energy 1e-6 relative.
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.calculator import EV_A3_TO_GPA, VOIGT, Batch, LinearModel, SO4Calculator, contract_plain

pytestmark = pytest.mark.gpu

LMAX, RCUT = 4, 5.0
TOL_FP64 = 1e-10
TOL_F32_FORCE, TOL_F32_STRESS = 1e-4, 1e-3   # eV/A, GPa


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(scope="module")
def workload(cuda_device):
    atoms = S.diamond_si(20, 20, 10, sigma=0.1, rng=np.random.default_rng(5))
    calc = SO4Calculator(lmax=LMAX, rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
    coef = np.random.default_rng(6).normal(0.0, 0.01, size=calc.nB)
    beta = np.broadcast_to(coef, (len(atoms), calc.nB))
    ref = O.forces_virial(atoms, beta, kind="SNAP", lmax=LMAX, rcut=RCUT, weights={"Si": 1.0}, rfac0=1.0,
                          nthreads=os.cpu_count() or 1)
    ref["stress"] = -(ref["virial"].reshape(1, 9)[:, VOIGT]) * EV_A3_TO_GPA
    return atoms, calc, coef, ref


def test_neighbour_list_bit_exact_at_32000_atoms(workload):
    atoms, calc, coef, ref = workload
    nl = ref["nl"]
    batch = Batch([atoms])
    nb = calc.neighbors(batch, torch.from_numpy(batch.positions).cuda())
    assert nb.nimg == nl.nimg and nb.npair == nl.npair
    assert np.array_equal(nb.img_ptr.cpu().numpy(), nl.img_ptr)
    assert np.array_equal(nb.seq.cpu().numpy(), nl.seq)
    assert np.array_equal(nb.img_j.cpu().numpy(), nl.img_j)
    assert np.array_equal(nb.img_off.cpu().numpy(), nl.img_off)
    assert np.array_equal(nb.img_r.cpu().numpy().view(np.int64), nl.img_r.view(np.int64))
    assert np.array_equal(nb.pair_img.cpu().numpy()[:-1], nl.pair_img[:-1])
    assert np.array_equal(nb.nsite.cpu().numpy(), nl.nsite)
    rev = nb.img_rev.cpu().numpy()
    assert np.array_equal(rev[rev], np.arange(len(rev)))


def test_fp64_plain_path_vs_oracle_at_32000_atoms(workload):
    atoms, calc, coef, ref = workload
    batch = Batch([atoms])
    d = calc.descriptors(batch, precision="fp64")
    beta = torch.as_tensor(coef, dtype=torch.float64, device="cuda").expand(len(atoms), -1).contiguous()
    c = contract_plain(d["x"], d["dxdr"], d["rdxdr"], d["seq"], d["pair_ptr"], batch.atom_ptr, beta, batch.volumes)
    ex = _rel(d["x"].cpu().numpy(), ref["x"])
    ef = _rel(c["forces"].cpu().numpy(), ref["forces"])
    es = _rel(c["stress"].cpu().numpy(), ref["stress"])
    ee = abs(float(c["energy"].sum()) - ref["energy"]) / abs(ref["energy"])
    print("FP64 plain vs oracle at 32000 atoms: B %.2e forces %.2e stress %.2e energy %.2e" % (ex, ef, es, ee))
    assert ex < TOL_FP64 and ef < TOL_FP64 and es < TOL_FP64 and ee < TOL_FP64


def test_fp32_adjoint_step_vs_oracle_at_32000_atoms(workload):
    atoms, calc, coef, ref = workload
    batch = Batch([atoms])
    step = calc.capture(batch, LinearModel(coef).cuda())
    res = step(torch.from_numpy(batch.positions).cuda())
    torch.cuda.synchronize()
    assert step.check()
    f = res["forces"].cpu().numpy()
    s = res["stress"].cpu().numpy()
    df = float(np.max(np.abs(f - ref["forces"])))
    ds = float(np.max(np.abs(s - ref["stress"])))
    ex = _rel(res["x"].double().cpu().numpy(), ref["x"])
    ee = abs(float(res["energy"].sum()) - ref["energy"]) / abs(ref["energy"])
    print("FP32 adjoint vs oracle at 32000 atoms: force %.2e eV/A, stress %.2e GPa, B %.2e, energy %.2e"
          % (df, ds, ex, ee))
    assert df <= TOL_F32_FORCE and ds <= TOL_F32_STRESS
    assert ex < 2e-5 and ee < 1e-6
