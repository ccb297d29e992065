"""The autotuner on the GPU: the tuned launch shapes against the oracle, and one search.

- so4_tables_create_tuned: out-of-range values -> SO4_ERR_ARG; a CTA shape that is not
  built for this twol -> SO4_ERR_UNSUPPORTED; the resolved tuning reads back.
- Each kernel shape (window units of 3 and 4 entries, 128-thread per-image CTAs, 2 and 8
  centres per U_tot CTA, the per-image pass with two lanes per image or one lane per row
  chain) at lmax 3 and 4: B, forces and
  virial against the oracle's contraction (2e-4 relative; B 2e-5), and the JVP
  against the oracle's dxdr / rdxdr (2e-4).
- autotune_step on a small batch: every evaluated candidate passed its check or was
  rejected, the chosen choice is applied to the calculator, its captured step matches
  the oracle, and a second call is answered from the cache.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyxtal_ff_gb300 import _lib, autotune, engine, ops
from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.calculator import EV_A3_TO_GPA, VOIGT, Batch, LinearModel, SO4Calculator
from tests import goldens as G

pytestmark = pytest.mark.gpu
W = {"Si": 1.0, "O": 0.5}


def _structs():
    return [S.diamond_si(2, 2, 1, sigma=0.1, rng=np.random.default_rng(41)), S.sio2_random(n_si=8, seed=42)]


def test_tuned_tables_validate_their_arguments(cuda_device):
    L = _lib.lib()
    h = C.c_void_p()
    for bad in [(6, 0, 0), (-1, 0, 0), (0, 192, 0), (0, 0, 3)]:
        assert L.so4_tables_create_tuned(8, 0, C.byref(_lib.Tuning(*bad)), C.byref(h)) == _lib.SO4_ERR_ARG
    for unsupported in [(0, 128, 0), (0, 0, 8)]:
        assert L.so4_tables_create_tuned(4, 0, C.byref(_lib.Tuning(*unsupported)), C.byref(h)) == \
            _lib.SO4_ERR_UNSUPPORTED
    assert engine.Tables(8, False, (3, 128, 2, 1)).tuning[:4] == (3, 128, 2, 1)
    assert engine.Tables(8, False, None).tuning[:3] == (5, 256, 4)
    assert engine.Tables(10, False, (4, 0, 0)).tuning == (4, 128, 4, 2, 32, 512)
    assert L.so4_tables_create_tuned(8, 0, C.byref(_lib.Tuning(0, 0, 0, 3)), C.byref(h)) == _lib.SO4_ERR_ARG
    assert L.so4_tables_create_tuned(4, 0, C.byref(_lib.Tuning(0, 0, 0, 1)), C.byref(h)) == _lib.SO4_ERR_UNSUPPORTED


@pytest.mark.parametrize("lmax", [3, 4])
@pytest.mark.parametrize("tuning", [(3, 0, 0, 0), (4, 128, 2, 2), (5, 128, 8, 2), (3, 256, 8, 2), (5, 0, 4, 1),
                                    (4, 0, 2, 1)])
def test_tuned_kernels_match_the_oracle(cuda_device, lmax, tuning):
    structs = _structs()
    pos = np.concatenate([s.positions for s in structs])
    cells = np.stack([s.get_cell() for s in structs])
    pbc = np.ones((2, 3), np.int32)
    ptr = np.concatenate([[0], np.cumsum([len(s) for s in structs])])
    numbers = np.concatenate([s.numbers for s in structs])
    symbols = sum([list(s.symbols) for s in structs], [])
    rc = 4.9
    p = torch.from_numpy(pos).cuda()
    choice = autotune.Choice(wkmax=tuning[0], rev_threads=tuning[1], utot_warps=tuning[2], rev_pair=tuning[3])
    ctx = ops.Context.build(p, cells, pbc, ptr, numbers, symbols, lmax=lmax, rcut=rc, kind="SNAP", weights=W,
                            tuning=choice)
    assert ctx.tab.tuning[0] == tuning[0]
    x, utot = engine.forward32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.w_site)
    beta = np.random.default_rng(7).normal(0, 0.01, size=(len(pos), ctx.tab.nB))
    f, vir = engine.adjoint32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, utot, torch.from_numpy(beta).float().cuda())
    rng = np.random.default_rng(8)
    v = rng.normal(size=(len(pos), 3))
    dB = engine.jvp32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, utot, v=torch.from_numpy(v).cuda()).cpu().numpy()
    f, vir = f.cpu().numpy(), vir.cpu().numpy()
    for s, st in enumerate(structs):
        a0, a1 = ptr[s], ptr[s + 1]
        ref = O.forces_virial(st, beta[a0:a1], kind="SNAP", lmax=lmax, rcut=rc, weights=W, rfac0=0.99363)
        assert G.rel_err(x[a0:a1].cpu().numpy(), ref["x"]) < 2e-5
        assert G.rel_err(f[a0:a1], ref["forces"]) < 2e-4
        assert G.rel_err(vir[s] / ctx.nb.vol[s], ref["virial"]) < 2e-4
        d = O.descriptor(st, kind="SNAP", lmax=lmax, rcut=rc, weights=W, rfac0=0.99363, stress=False)
        exp = np.zeros((a1 - a0, ref["x"].shape[1]))
        for q, (i, j) in enumerate(d["seq"]):
            exp[i] += d["dxdr"][q] @ v[a0 + j]
        assert G.rel_err(dB[a0:a1], exp) < 2e-4


@pytest.mark.parametrize("twol", [6, 8, 10])
def test_every_created_unit_cap_runs_every_window_mode(cuda_device, twol):
    # a unit cap the window kernels cannot stage is refused at creation, never at launch
    L = _lib.lib()
    structs = _structs()
    pos = np.concatenate([s.positions for s in structs])
    cells = np.stack([s.get_cell() for s in structs])
    ptr = np.concatenate([[0], np.cumsum([len(s) for s in structs])])
    numbers = np.concatenate([s.numbers for s in structs])
    symbols = sum([list(s.symbols) for s in structs], [])
    made = 0
    for wk in range(1, 6):
        h = C.c_void_p()
        rc = L.so4_tables_create_tuned(twol, 0, C.byref(_lib.Tuning(wk, 0, 0)), C.byref(h))
        assert rc in (_lib.SO4_OK, _lib.SO4_ERR_UNSUPPORTED)
        if rc != _lib.SO4_OK:
            continue
        L.so4_tables_destroy(h)
        made += 1
        p = torch.from_numpy(pos).cuda()
        ctx = ops.Context.build(p, cells, np.ones((2, 3), np.int32), ptr, numbers, symbols, lmax=twol // 2,
                                rcut=4.5, kind="SNAP", weights=W, tuning=autotune.Choice(wkmax=wk))
        x, utot = engine.forward32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.w_site)
        beta = torch.ones((len(pos), ctx.tab.nB), dtype=torch.float32, device="cuda")
        engine.adjoint32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, utot, beta)
        engine.adjoint_linear32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.w_site, beta)
        if twol <= 8:  # the JVP's window mode stages more slots than fit above twol 8, whatever the cap
            engine.jvp32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, utot,
                         v=torch.ones((len(pos), 3), dtype=torch.float64, device="cuda"))
    assert made >= 3  # the default cap and the tuner's 4 and 3 at least
    torch.cuda.synchronize()


def test_autotune_step_picks_a_checked_choice_and_caches_it(cuda_device, tmp_path):
    structs = [S.diamond_si(3, 3, 3, sigma=0.1, rng=np.random.default_rng(43))]
    batch = Batch(structs)
    calc = SO4Calculator(lmax=3, rcut=4.9, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
    coef = np.random.default_rng(44).normal(0, 0.01, size=calc.nB)
    model = LinearModel(coef).cuda()
    cache = autotune.TuningCache(str(tmp_path / "tuning.json"))
    rep = autotune.autotune_step(calc, batch, model, steps=3, warmup=1, rounds=1, cache=cache)
    assert not rep["cached"] and rep["ms"] > 0
    assert all(e["ms"] is None or e["ms"] > 0 for e in rep["evaluated"])
    chosen = autotune.Choice.from_dict(rep["choice"])
    assert calc.tuning == chosen and calc.tables.tuning[0] == chosen.wkmax
    res = calc.capture(batch, model)(torch.from_numpy(batch.positions).cuda())
    beta = np.broadcast_to(coef, (batch.natoms, calc.nB))
    ref = O.forces_virial(structs[0], beta, kind="SNAP", lmax=3, rcut=4.9, weights={"Si": 1.0}, rfac0=1.0)
    stress = -(ref["virial"].reshape(1, 9)[:, VOIGT]) * EV_A3_TO_GPA
    assert G.rel_err(res["forces"].cpu().numpy(), ref["forces"]) < 2e-4
    assert G.rel_err(res["stress"].cpu().numpy(), stress) < 2e-4
    again = autotune.autotune_step(SO4Calculator(lmax=3, rcut=4.9, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0),
                                   batch, model, cache=cache)
    assert again["cached"] and again["choice"] == rep["choice"]
