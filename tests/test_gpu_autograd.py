"""The adjoint's backward (JVP) and the torch autograd chain.

- JVP vs the oracle: dB_i = sum_pairs dxdr[p] . v_j (dxdr of the reference's
  algorithm, FP64) and the strain part V sum_ab G_ab sum_pairs rdxdr[p][k][a][b].
- SO4Descriptor: positions.grad after E.backward() equals -F of the oracle's
  contraction.
- AdjointForces: dL/dbeta from the JVP equals exact differences of L in beta
  (L is linear in beta, so central differences have no truncation error).
Tolerances: FP32 kernels against FP64, 2e-4 relative to the largest entry.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from pyxtal_ff_gb300 import engine, ops
from pyxtal_ff_gb300 import structures as S
from tests import goldens as G

pytestmark = pytest.mark.gpu
W = {"Si": 1.0, "O": 0.5}


def _batch():
    structs = [S.diamond_si(2, 1, 1, sigma=0.1, strain=0.03, rng=np.random.default_rng(31)),
               S.sio2_random(n_si=8, seed=32)]
    pos = np.concatenate([s.positions for s in structs])
    cells = np.stack([s.get_cell() for s in structs])
    pbc = np.ones((2, 3), np.int32)
    ptr = np.concatenate([[0], np.cumsum([len(s) for s in structs])])
    numbers = np.concatenate([s.numbers for s in structs])
    symbols = sum([list(s.symbols) for s in structs], [])
    return structs, pos, cells, pbc, ptr, numbers, symbols


def _ctx(lmax=3, rc=4.5):
    structs, pos, cells, pbc, ptr, numbers, symbols = _batch()
    p = torch.from_numpy(pos).cuda()
    ctx = ops.Context.build(p, cells, pbc, ptr, numbers, symbols, lmax=lmax, rcut=rc, kind="SNAP", weights=W)
    x, utot = engine.forward32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.w_site)
    ctx.utot = utot
    return structs, ptr, p, ctx, x


@pytest.mark.parametrize("lmax", [1.5, 2, 2.5, 3, 3.5, 4, 4.5, 5.5])
def test_jvp_matches_oracle_dxdr_and_rdxdr(cuda_device, lmax):
    # half-integer lmax (SNAP's odd twol) runs the same row-chain kernels at twol 3 to 11
    rc = 4.5
    structs, ptr, p, ctx, _ = _ctx(lmax, rc)
    N, S_ = ctx.nb.natoms, ctx.nb.nstruct
    rng = np.random.default_rng(int(2 * lmax))
    v = rng.normal(size=(N, 3))
    Gm = rng.normal(size=(S_, 3, 3))
    dB_v = engine.jvp32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.utot, v=torch.from_numpy(v).cuda()).cpu().numpy()
    dB_G = engine.jvp32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.utot, G=torch.from_numpy(Gm).cuda()).cpu().numpy()
    for s, st in enumerate(structs):
        a0, a1 = ptr[s], ptr[s + 1]
        ref = O.descriptor(st, kind="SNAP", lmax=lmax, rcut=rc, weights=W, rfac0=0.99363, stress=True)
        seq = ref["seq"]
        exp_v = np.zeros((a1 - a0, ref["x"].shape[1]))
        exp_G = np.zeros_like(exp_v)
        vol = st.get_volume()
        for q, (i, j) in enumerate(seq):
            exp_v[i] += ref["dxdr"][q] @ v[a0 + j]
            exp_G[i] += vol * np.einsum("kab,ab->k", ref["rdxdr"][q], Gm[s])
        assert G.rel_err(dB_v[a0:a1], exp_v) < 2e-4
        assert G.rel_err(dB_G[a0:a1], exp_G) < 2e-4


def test_autograd_positions_grad_is_minus_forces(cuda_device):
    structs, ptr, p, ctx, _ = _ctx(3, 4.5)
    p = p.clone().requires_grad_(True)
    x = ops.SO4Descriptor.apply(p, ctx)
    coef = torch.from_numpy(np.random.default_rng(3).normal(0, 0.01, size=x.shape[1])).float().cuda()
    E = (x * coef).sum()
    E.backward()
    grad = p.grad.cpu().numpy()
    for s, st in enumerate(structs):
        a0, a1 = ptr[s], ptr[s + 1]
        beta = np.broadcast_to(coef.cpu().numpy().astype(np.float64), (a1 - a0, x.shape[1]))
        ref = O.forces_virial(st, beta, kind="SNAP", lmax=3, rcut=4.5, weights=W, rfac0=0.99363)
        assert G.rel_err(-grad[a0:a1], ref["forces"]) < 2e-4


def test_force_loss_gradient_in_beta_is_exact_difference(cuda_device):
    structs, ptr, p, ctx, x = _ctx(3, 4.5)
    N, nB = x.shape
    rng = np.random.default_rng(4)
    beta = torch.from_numpy(rng.normal(0, 0.01, size=(N, nB))).float().cuda().requires_grad_(True)
    cF = torch.from_numpy(rng.normal(size=(N, 3))).cuda()
    cW = torch.from_numpy(rng.normal(size=(ctx.nb.nstruct, 3, 3))).cuda()

    def loss(b):
        F, Wv = ops.AdjointForces.apply(b, ctx)
        return (F * cF).sum() + (Wv * cW).sum()

    L = loss(beta)
    L.backward()
    g = beta.grad.cpu().numpy()
    for (i, k) in [(0, 0), (3, 7), (N - 1, nB - 1), (20, 11)]:
        eps = 0.5
        bp = beta.detach().clone()
        bm = beta.detach().clone()
        bp[i, k] += eps
        bm[i, k] -= eps
        fd = (loss(bp).item() - loss(bm).item()) / (2 * eps)
        assert abs(fd - g[i, k]) <= 2e-4 * max(1.0, np.abs(g).max()), (i, k, fd, g[i, k])


def test_neighbor_and_plain_ops_match_engine(cuda_device):
    _, _, p, ctx, _ = _ctx()
    k = ops.key(ctx)
    pos = p.detach().clone() + 0.01
    img_ptr, img_j, img_off, img_r, pair_ptr, seq = torch.ops.so4gb300.neighbors(k, pos)
    nb = engine.build_neighbors(pos, *ctx.layout[:3], ctx.layout[3])
    for a, b in ((img_ptr, nb.img_ptr), (img_j, nb.img_j), (img_off, nb.img_off), (img_r, nb.img_r),
                 (pair_ptr, nb.pair_ptr), (seq, nb.seq)):
        assert torch.equal(a, b)
    for prec in (0, 1):
        x, dxdr, rdxdr = torch.ops.so4gb300.forward_deriv(k, pos, prec)
        x2, dxdr2, rdxdr2 = engine.plain(ctx.tab, ctx.prm, nb, pos, ctx.w_nb, ctx.w_site, precision=prec)
        assert torch.equal(x, x2) and torch.equal(dxdr, dxdr2) and torch.equal(rdxdr, rdxdr2)
    ops.release(ctx)


def test_operator_set_names_and_contraction_op(cuda_device):
    # forward / adjoint / adjoint_jvp are the 32-bit operators under the operator set's
    # names; contract_dxdr contracts the plain path's outputs on the context's pair list
    _, _, p, ctx, x = _ctx()
    k = ops.key(ctx)
    xa, ua = torch.ops.so4gb300.forward(k)
    xb, ub = torch.ops.so4gb300.forward32(k)
    assert torch.equal(xa, xb) and torch.equal(ua, ub)
    beta = torch.randn_like(xa)
    fa, wa = torch.ops.so4gb300.adjoint(k, ua, beta)
    fb, wb = torch.ops.so4gb300.adjoint32(k, ua, beta)
    assert torch.equal(fa, fb) and torch.equal(wa, wb)
    v = torch.randn((xa.shape[0], 3), dtype=torch.float64, device="cuda")
    Gs = torch.randn((ctx.nb.nstruct, 3, 3), dtype=torch.float64, device="cuda")
    assert torch.equal(torch.ops.so4gb300.adjoint_jvp(k, ua, v, Gs), torch.ops.so4gb300.jvp32(k, ua, v, Gs))
    x64, dxdr, rdxdr = torch.ops.so4gb300.forward_deriv(k, p, 0)
    rda = engine.rdxdr_atom(rdxdr, ctx.nb.pair_ptr, ctx.nb.natoms)
    b64 = beta.double()
    f, st = torch.ops.so4gb300.contract_dxdr(k, b64, dxdr, rda)
    f2, st2 = engine.contract_dxdr(b64, ctx.nb.pair_ptr, ctx.nb.seq, ctx.nb.atom_struct, ctx.nb.atom_ptr_dev,
                                   dxdr=dxdr, rdxdr_atom=rda)
    assert torch.equal(f, f2) and torch.equal(st, st2)
    # the FP64 contraction and the FP32 adjoint agree on the forces
    assert (f - fa).abs().max().item() <= 2e-4 * fa.abs().max().item()
    ops.release(ctx)
