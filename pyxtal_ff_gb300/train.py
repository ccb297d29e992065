"""Force-matching training on the adjoint path.

The reference trains its NN on stored descriptors, dxdr and rdxdr
(pyxtal_ff/models/neuralnetwork.py:466-545): forces are
-einsum(dE/dx, dxdr_dense) and the loss mixes energy and force errors.  Here the
descriptors and the adjoint state (U_tot) are computed once on the GPU and kept
there; each optimiser step runs the model on B, gets beta = dE/dB with a graph,
forms forces with the adjoint kernel (``ops.AdjointForces``), and back-propagates
the loss through the JVP kernel into the model weights.  dB/dr is never stored.

``stillinger_weber`` provides synthetic FP64 targets: the Stillinger-Weber
two- and three-body potential with the published silicon parameters
(F. H. Stillinger and T. A. Weber, Phys. Rev. B 31, 5262 (1985)), evaluated on
the GPU neighbour list in FP64 with torch autograd for the forces.
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine, ops
from .calculator import Batch

# Stillinger-Weber silicon (eV, Angstrom)
SW_SI = dict(epsilon=2.1683, sigma=2.0951, a=1.80, lam=21.0, gamma=1.20, A=7.049556277, B=0.6022245584,
             p=4.0, q=0.0, cos0=-1.0 / 3.0)


def stillinger_weber(batch: Batch, device="cuda", params=SW_SI):
    """FP64 energies (S,) and forces (N,3) of every structure of a batch."""
    prm = params
    rc = prm["a"] * prm["sigma"]
    pos = torch.from_numpy(batch.positions).to(device).requires_grad_(True)
    nb = engine.build_neighbors(pos.detach(), batch.cells, batch.pbc, batch.atom_ptr, rc, device=device)
    img_ptr = nb.img_ptr.long()
    N = batch.natoms
    centre = torch.repeat_interleave(torch.arange(N, device=device), img_ptr[1:] - img_ptr[:-1])
    j = nb.img_j.long()
    # image vectors as a differentiable function of the positions: r = pos[j] - pos[i] + o . cell
    cells = torch.from_numpy(batch.cells).to(device)
    struct = torch.repeat_interleave(torch.arange(batch.nstruct, device=device),
                                     torch.from_numpy(np.diff(batch.atom_ptr)).to(device))
    shift = torch.einsum("mk,mkc->mc", nb.img_off.double(), cells[struct[centre]])
    rv = pos[j] - pos[centre] + shift
    r = torch.linalg.norm(rv, dim=1)
    s, eps = prm["sigma"], prm["epsilon"]
    x = r / s
    inside = x < prm["a"]
    # evaluate outside entries at a harmless x so no branch of torch.where is infinite
    xs = torch.where(inside, x, torch.ones_like(x))
    den = xs - prm["a"]
    e2 = torch.where(inside, prm["A"] * eps * (prm["B"] * xs.pow(-prm["p"]) - xs.pow(-prm["q"])) * torch.exp(1.0 / den),
                     torch.zeros_like(x))
    e_atom = torch.zeros(N, dtype=torch.float64, device=device).index_add(0, centre, 0.5 * e2)
    # three-body: every ordered pair (m, n), m < n, of images of the same centre
    g = torch.where(inside, torch.exp(prm["gamma"] / den), torch.zeros_like(x))
    counts = (img_ptr[1:] - img_ptr[:-1]).cpu().numpy()
    mi, ni = [], []
    base = img_ptr.cpu().numpy()
    for a in range(N):
        c = counts[a]
        if c > 1:
            iu = np.triu_indices(c, 1)
            mi.append(base[a] + iu[0])
            ni.append(base[a] + iu[1])
    if mi:
        mi = torch.from_numpy(np.concatenate(mi)).to(device)
        ni = torch.from_numpy(np.concatenate(ni)).to(device)
        cos = (rv[mi] * rv[ni]).sum(1) / (r[mi] * r[ni])
        e3 = prm["lam"] * eps * (cos - prm["cos0"]) ** 2 * g[mi] * g[ni]
        e_atom = e_atom.index_add(0, centre[mi], e3)
    energy = torch.zeros(batch.nstruct, dtype=torch.float64, device=device).index_add(0, struct, e_atom)
    forces, = torch.autograd.grad(energy.sum(), pos)
    return energy.detach(), (-forces).detach()


class RowChunkedLinear(torch.nn.Linear):
    """nn.Linear computed over chunks of `rows` input rows with one batched matmul.

    The trainer's layers are tall and narrow (tens of thousands of atoms by 30 features), so
    the gradient of a weight is a 30 x 30 product summed over all the atoms; as one GEMM that
    reduction runs on a handful of thread blocks.  Chunked, autograd forms it as one product
    per chunk (in parallel) and a sum over the chunks, at every order of differentiation the
    force-matching loss needs.  The parameters and results are those of nn.Linear (up to the
    order of the sums)."""

    rows = 512

    def forward(self, x):
        n = x.shape[0]
        if x.dim() != 2 or n < 4 * self.rows:
            return super().forward(x)
        c = (n + self.rows - 1) // self.rows
        xp = torch.nn.functional.pad(x, (0, 0, 0, c * self.rows - n)).view(c, self.rows, self.in_features)
        y = torch.bmm(xp, self.weight.t().unsqueeze(0).expand(c, self.in_features, self.out_features))
        y = y.reshape(c * self.rows, self.out_features)[:n]
        return y + self.bias if self.bias is not None else y


class SpeciesMLP(torch.nn.Module):
    """Per-species MLP on B (nB -> hidden... -> 1, tanh), Xavier-uniform weights from a seed."""

    def __init__(self, nB, nspecies, hidden=(30, 30), seed=0, dtype=torch.float32):
        super().__init__()
        gen = torch.Generator().manual_seed(seed)
        self.nets = torch.nn.ModuleList()
        for _ in range(nspecies):
            layers, n_in = [], nB
            for h in hidden:
                layers += [RowChunkedLinear(n_in, h), torch.nn.Tanh()]
                n_in = h
            layers.append(RowChunkedLinear(n_in, 1))
            net = torch.nn.Sequential(*layers)
            for m in net:
                if isinstance(m, torch.nn.Linear):
                    torch.nn.init.xavier_uniform_(m.weight, generator=gen)
                    torch.nn.init.zeros_(m.bias)
            self.nets.append(net.to(dtype))

    def forward(self, x, species, index=None):
        """Per-atom energies; index: optional list of per-species atom index tensors (given
        once for a fixed batch, so that the forward needs no host synchronisation)."""
        if len(self.nets) == 1:
            return self.nets[0](x).squeeze(-1)
        if index is None:
            index = [(species == s).nonzero().squeeze(-1) for s in range(len(self.nets))]
        out = torch.zeros(x.shape[0], dtype=x.dtype, device=x.device)
        for idx, net in zip(index, self.nets):
            out = out.index_put((idx,), net(x.index_select(0, idx)).squeeze(-1))
        return out


class ForceMatching:
    """One-optimiser-step trainer: loss = MSE(E/atom) + w_f MSE(F), forces from the adjoint.

    ``capture()`` records one whole step (model, adjoint forces, the JVP backward, Adam)
    as a CUDA graph for the fixed batch; later ``step()`` calls replay it."""

    def __init__(self, structures, *, lmax=3, rcut=4.9, kind="SNAP", weights=None, rfac0=1.0, hidden=(30, 30),
                 seed=0, lr=1e-3, force_weight=0.1, targets=None, device="cuda", tuning=None):
        self.device = torch.device(device)
        self.batch = structures if isinstance(structures, Batch) else Batch(structures)
        b = self.batch
        pos = torch.from_numpy(b.positions).to(self.device)
        self.ctx = ops.Context.build(pos, b.cells, b.pbc, b.atom_ptr, b.numbers, b.symbols, lmax=lmax, rcut=rcut,
                                     kind=kind, weights=weights or {s: 1.0 for s in set(b.symbols)}, rfac0=rfac0,
                                     tuning=tuning)
        x, utot = engine.forward32(self.ctx.tab, self.ctx.prm, self.ctx.nb, self.ctx.w_nb, self.ctx.w_site)
        self.ctx.utot = utot
        self.x = x
        self.species = torch.from_numpy(b.species).to(self.device)
        self.struct = torch.repeat_interleave(torch.arange(b.nstruct, device=self.device),
                                              torch.from_numpy(np.diff(b.atom_ptr)).to(self.device))
        self.natoms_s = torch.from_numpy(np.diff(b.atom_ptr)).to(self.device).double()
        if targets is None:
            targets = stillinger_weber(b, device=self.device)
        self.e_ref, self.f_ref = targets
        self.model = SpeciesMLP(x.shape[1], len(b.species_order), hidden=hidden, seed=seed).to(self.device)
        # capturable: the optimiser's step counters live on the device, so a step can be graphed
        self.opt = torch.optim.Adam(self.model.parameters(), lr=lr, capturable=True)
        self.force_weight = force_weight
        self.sp_index = [torch.from_numpy(np.nonzero(b.species == s)[0]).to(self.device)
                         for s in range(len(b.species_order))]
        self.graph = None

    def loss(self):
        xg = self.x.detach().requires_grad_(True)
        e_atom = self.model(xg, self.species, self.sp_index)
        beta, = torch.autograd.grad(e_atom.sum(), xg, create_graph=True)
        forces, _ = ops.AdjointForces.apply(beta, self.ctx)
        energy = torch.zeros(self.batch.nstruct, dtype=torch.float64, device=self.device).index_add(
            0, self.struct, e_atom.double())
        le = torch.mean(((energy - self.e_ref) / self.natoms_s) ** 2)
        lf = torch.mean((forces - self.f_ref) ** 2)
        return le + self.force_weight * lf

    def _step(self):
        L = self.loss()
        L.backward()
        self.opt.step()
        return L.detach()

    def step(self):
        """One optimiser step; the loss of this step (before the update) on the device."""
        if self.graph is not None:
            self.graph.replay()
            return self._loss
        self.opt.zero_grad(set_to_none=True)
        return self._step()

    def capture(self, warmup=3):
        """Record one step as a CUDA graph (after `warmup` eager steps on a side stream, which
        train the model like any other steps); later step() calls replay it."""
        side = torch.cuda.Stream(device=self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                self.opt.zero_grad(set_to_none=True)
                self._step()
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        # gradients are created inside the capture and overwritten by every replay
        self.opt.zero_grad(set_to_none=True)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._loss = self._step()
        self.graph = g
        return self
