"""PyTorch operators and autograd functions over the C ABI.

Operators (``torch.ops.so4gb300.*``, registered with ``torch.library.custom_op``;
they launch the CUDA kernels on torch's current stream):

  neighbors(...)      -> (img_ptr, img_j, img_off, img_r, pair_ptr, seq)   so4_nl_*
  forward_deriv(...)  -> (B, dB/dr, rdxdr), FP64 or FP32                    so4_plain
  forward32(...)      -> (B, U_tot)                                         so4_forward32
  adjoint32(...)      -> (forces, virial)                                   so4_adjoint32
  jvp32(...)          -> dB                                                 so4_jvp32
  forward / adjoint / adjoint_jvp: the same three under the operator set's names
  contract_dxdr(...)  -> (forces, stress sums) from dxdr, rdxdr_atom         so4_contract_dxdr

Autograd:

  ``SO4Descriptor.apply(positions, ctx)`` returns B (N, nB) f32; its backward is the
  adjoint kernel, so ``E = model(B); E.backward()`` leaves dE/dr = -F in
  ``positions.grad`` without forming dB/dr.

  ``AdjointForces.apply(beta, ctx)`` returns (forces, virial) for beta = dE/dB;
  its backward is the JVP kernel, so a loss on forces or stress trains the model
  that produced beta (double backward through the model, then the JVP).

``ctx`` is a ``Context`` holding the neighbour list, tables and U_tot of one
batch (built by ``Context.build``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine

_NS = "so4gb300"


class Context:
    """Per-batch state shared by the operators: tables, parameters, neighbours, weights, U_tot."""

    def __init__(self, tab, prm, nb, w_nb, w_site):
        self.tab, self.prm, self.nb, self.w_nb, self.w_site = tab, prm, nb, w_nb, w_site
        self.utot = None

    @classmethod
    def build(cls, positions, cells, pbc, atom_ptr, numbers, symbols, *, lmax, rcut, kind="SO4", weights=None,
              rfac0=0.99363, cutoff_function="cosine", normalize_U=False, tuning=None):
        """tuning: an autotune.Choice (its kernel launch shapes) or None for the defaults."""
        twol = int(round(2 * lmax))
        tab = engine.tables(twol, normalize_U, None if tuning is None else tuning.kernel_tuning())
        prm = engine.params(twol, rcut, 1.0 if kind == "SO4" else rfac0, cutoff_function)
        nb = engine.build_neighbors(positions.detach(), cells, pbc, atom_ptr, rcut, device=positions.device)
        w_nb, w_site = engine.site_weights(kind, numbers, symbols, weights)
        dev = positions.device
        c = cls(tab, prm, nb, torch.from_numpy(w_nb).to(dev), torch.from_numpy(w_site).to(dev))
        c.layout = (np.asarray(cells), np.asarray(pbc), np.asarray(atom_ptr), float(rcut))
        return c

    def rebuild_neighbors(self, positions):
        """Neighbour list of new positions for the same cells and atom ranges."""
        cells, pbc, atom_ptr, rcut = self.layout
        self.nb = engine.build_neighbors(positions.detach(), cells, pbc, atom_ptr, rcut, device=positions.device)
        self.utot = None
        return self.nb


_CTX = {}


def _register(ctx):
    key = id(ctx)
    _CTX[key] = ctx
    return key


def key(ctx):
    """The integer handle the operators take for a context (registers it)."""
    return _register(ctx)


@torch.library.custom_op(_NS + "::neighbors", mutates_args=())
def neighbors_op(ctx_key: int, positions: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor,
                                                                 torch.Tensor, torch.Tensor, torch.Tensor]:
    """Rebuild the context's neighbour list for positions (N,3) f64; CSR arrays by centre."""
    nb = _CTX[ctx_key].rebuild_neighbors(positions)
    return (nb.img_ptr.clone(), nb.img_j.clone(), nb.img_off.clone(), nb.img_r.clone(), nb.pair_ptr.clone(),
            nb.seq.clone())


@torch.library.custom_op(_NS + "::forward_deriv", mutates_args=())
def forward_deriv_op(ctx_key: int, positions: torch.Tensor, precision: int) -> tuple[torch.Tensor, torch.Tensor,
                                                                                     torch.Tensor]:
    """The plain path: B (N,nB), dB/dr per (i, j) pair (P,nB,3) and rdxdr (P,nB,3,3),
    FP64 (precision 0) or FP32 (1), on the context's neighbour list."""
    c = _CTX[ctx_key]
    x, dxdr, rdxdr = engine.plain(c.tab, c.prm, c.nb, positions.contiguous(), c.w_nb, c.w_site,
                                  precision=int(precision))
    return x.clone(), dxdr.clone(), rdxdr.clone()


@torch.library.custom_op(_NS + "::forward32", mutates_args=())
def forward32_op(ctx_key: int) -> tuple[torch.Tensor, torch.Tensor]:
    c = _CTX[ctx_key]
    x, utot = engine.forward32(c.tab, c.prm, c.nb, c.w_nb, c.w_site)
    return x.clone(), utot.clone()


@torch.library.custom_op(_NS + "::adjoint32", mutates_args=())
def adjoint32_op(ctx_key: int, utot: torch.Tensor, beta: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    c = _CTX[ctx_key]
    f, w = engine.adjoint32(c.tab, c.prm, c.nb, c.w_nb, utot, beta)
    return f.clone(), w.clone()


@torch.library.custom_op(_NS + "::jvp32", mutates_args=())
def jvp32_op(ctx_key: int, utot: torch.Tensor, v: torch.Tensor, G: torch.Tensor) -> torch.Tensor:
    c = _CTX[ctx_key]
    return engine.jvp32(c.tab, c.prm, c.nb, c.w_nb, utot, v=v, G=G).clone()


# The same operators under the names of the path's operator set (forward / adjoint /
# adjoint_jvp), and the NN consumer's contraction of the plain path's outputs.
@torch.library.custom_op(_NS + "::forward", mutates_args=())
def forward_op(ctx_key: int) -> tuple[torch.Tensor, torch.Tensor]:
    """B (N, nB) f32 and U_tot (kept for the adjoint): forward32."""
    return forward32_op(ctx_key)


@torch.library.custom_op(_NS + "::adjoint", mutates_args=())
def adjoint_op(ctx_key: int, utot: torch.Tensor, beta: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """Forces (N, 3) and virial (S, 3, 3) f64 for beta = dE/dB: adjoint32."""
    return adjoint32_op(ctx_key, utot, beta)


@torch.library.custom_op(_NS + "::adjoint_jvp", mutates_args=())
def adjoint_jvp_op(ctx_key: int, utot: torch.Tensor, v: torch.Tensor, G: torch.Tensor) -> torch.Tensor:
    """The adjoint's backward, dB along dr_m = (v_j - v_i) + G_s^T r_m: jvp32."""
    return jvp32_op(ctx_key, utot, v, G)


@torch.library.custom_op(_NS + "::contract_dxdr", mutates_args=())
def contract_dxdr_op(ctx_key: int, beta: torch.Tensor, dxdr: torch.Tensor,
                     rdxdr_atom: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    """Forces (N, 3) and per-structure stress sums (S, 6) from the plain path's dxdr and
    per-atom rdxdr on the context's pair list (so4_contract_dxdr)."""
    nb = _CTX[ctx_key].nb
    f, st = engine.contract_dxdr(beta.contiguous(), nb.pair_ptr, nb.seq, nb.atom_struct, nb.atom_ptr_dev,
                                 dxdr=dxdr.contiguous(), rdxdr_atom=rdxdr_atom.contiguous())
    return f.clone(), st.clone()


class SO4Descriptor(torch.autograd.Function):
    """B = SO4Descriptor.apply(positions, ctx); backward: grad_positions = -F(beta = grad_B)."""

    @staticmethod
    def forward(actx, positions, ctx):
        key = _register(ctx)
        x, utot = torch.ops.so4gb300.forward32(key)
        ctx.utot = utot
        actx.key = key
        actx.save_for_backward(utot)
        return x

    @staticmethod
    def backward(actx, grad_x):
        (utot,) = actx.saved_tensors
        forces, _ = torch.ops.so4gb300.adjoint32(actx.key, utot, grad_x.contiguous().float())
        return -forces, None


class AdjointForces(torch.autograd.Function):
    """(F, W) = AdjointForces.apply(beta, ctx): F = -dE/dr, W = sum r (x) dE/dr for beta = dE/dB.
    Backward: dL/dbeta = JVP(v = -dL/dF, G = dL/dW)."""

    @staticmethod
    def forward(actx, beta, ctx):
        key = _register(ctx)
        if ctx.utot is None:
            raise RuntimeError("run SO4Descriptor (or forward32) on this context first")
        f, w = torch.ops.so4gb300.adjoint32(key, ctx.utot, beta.contiguous().float())
        actx.key = key
        actx.save_for_backward(ctx.utot)
        return f, w

    @staticmethod
    def backward(actx, gF, gW):
        (utot,) = actx.saved_tensors
        c = _CTX[actx.key]
        dev = utot.device
        v = -gF.double() if gF is not None else torch.zeros((c.nb.natoms, 3), dtype=torch.float64, device=dev)
        G = gW.double() if gW is not None else torch.zeros((c.nb.nstruct, 3, 3), dtype=torch.float64, device=dev)
        dB = torch.ops.so4gb300.jvp32(actx.key, utot, v.contiguous(), G.contiguous())
        return dB, None


def release(ctx):
    """Forget a context registered by the autograd functions."""
    _CTX.pop(id(ctx), None)
