"""Batched energy / forces / stress on the GPU (the public API of the adjoint path).

``SO4Calculator`` evaluates many structures in one pass: the GPU neighbour list,
the FP32 forward (U_tot, B), a per-atom energy model on B, and the FP32 adjoint
that turns beta = dE/dB into forces and the virial without forming dB/dr.  It is
the batched counterpart of what the reference does per structure in
pyxtal_ff/calculator/__init__.py:22-73 (compute_descriptor, then
NeuralNetwork.calculate_properties :579-678, which contracts dxdr and rdxdr with
dE/dx).  Stress follows the reference's convention:
  stress_voigt (GPa) = -(1/V) sum_images r (x) dE/dr in (xx, yy, zz, xy, xz, yz) x 160.21766.

``LinearModel`` is E_i = B_i . c[species_i] + b[species_i] (the reference's
order-1 PolynomialRegression, pyxtal_ff/models/polynomialregression.py:374).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import engine
from .structures import as_arrays

EV_A3_TO_GPA = 160.21766208
VOIGT = [0, 4, 8, 1, 2, 5]


class LinearModel(torch.nn.Module):
    """Per-species linear energy on B: E_i = B_i . coef[s_i] + bias[s_i]."""

    def __init__(self, coef, bias=None):
        super().__init__()
        coef = torch.as_tensor(coef, dtype=torch.float32)
        if coef.dim() == 1:
            coef = coef[None]
        self.coef = torch.nn.Parameter(coef)
        b = torch.zeros(coef.shape[0]) if bias is None else torch.as_tensor(bias, dtype=torch.float32).reshape(-1)
        self.bias = torch.nn.Parameter(b)

    def forward(self, x, species):
        return (x * self.coef[species]).sum(-1) + self.bias[species]


class Batch:
    """Host description of a batch of structures (cells, pbc, atom ranges, species)."""

    def __init__(self, structures, species_order=None):
        structures = list(structures)
        self.structures = structures
        pos, cells, pbcs, nums, syms = [], [], [], [], []
        for s in structures:
            p, c, b, n, y = as_arrays(s)
            pos.append(p)
            cells.append(c)
            pbcs.append(b)
            nums.append(n)
            syms.extend(y)
        self.positions = np.ascontiguousarray(np.concatenate(pos)) if pos else np.zeros((0, 3))
        self.cells = np.stack(cells) if cells else np.zeros((0, 3, 3))
        self.pbc = np.stack(pbcs).astype(np.int32) if pbcs else np.zeros((0, 3), np.int32)
        self.numbers = np.concatenate(nums) if nums else np.zeros(0, np.int64)
        self.symbols = syms
        self.atom_ptr = np.concatenate([[0], np.cumsum([len(p) for p in pos])]).astype(np.int64)
        self.volumes = np.abs(np.linalg.det(self.cells)) if len(cells) else np.zeros(0)
        order = species_order or sorted(set(syms))
        self.species_order = list(order)
        idx = {s: i for i, s in enumerate(self.species_order)}
        self.species = np.array([idx[s] for s in syms], dtype=np.int64)

    @property
    def natoms(self):
        return int(self.atom_ptr[-1])

    @property
    def nstruct(self):
        return len(self.atom_ptr) - 1


class SO4Calculator:
    """Energy, forces and stress of many structures with the FP32 adjoint kernels.

    kind="SO4": neighbour and site weights are atomic numbers, psi = pi r / rcut
    (pyxtal_ff/descriptors/SO4.py).  kind="SNAP": weights[symbol] and 1,
    psi = rfac0 pi r / rcut (pyxtal_ff/descriptors/SNAP.py).
    """

    def __init__(self, lmax=3, rcut=3.5, kind="SO4", weights=None, rfac0=0.99363, cutoff_function="cosine",
                 normalize_U=False, device="cuda", tuning=None):
        engine.require_cuda()
        if kind not in ("SO4", "SNAP"):
            raise ValueError("kind must be 'SO4' or 'SNAP'")
        if kind == "SNAP" and not isinstance(weights, dict):
            raise TypeError("weights must be a dictionary")
        self.kind = kind
        self.weights = weights
        self.lmax = lmax
        self.twol = int(round(2 * lmax))
        self.rcut = float(rcut)
        self.rfac0 = 1.0 if kind == "SO4" else float(rfac0)
        self.cutoff_function = cutoff_function
        self.device = torch.device(device)
        self.normalize_U = bool(normalize_U)
        self.params = engine.params(self.twol, self.rcut, self.rfac0, cutoff_function)
        self._ws = None
        self._batch_key = None
        self.set_tuning(tuning)

    def set_tuning(self, tuning=None):
        """Launch shapes (an autotune.Choice, e.g. from autotune.autotune_step; None: the
        defaults): the kernels' tables and the captured step's branches and PDL."""
        self.tuning = tuning
        with torch.cuda.device(self.device):
            self.tables = engine.tables(self.twol, self.normalize_U, None if tuning is None else tuning.kernel_tuning())
        self.branches = 2 if tuning is None else int(tuning.branches)
        self.pdl = False if tuning is None else bool(tuning.pdl)
        self._ws = None

    @property
    def nB(self):
        return self.tables.nB

    def prepare(self, batch: Batch):
        """Upload the per-atom weights and species of a batch (once per batch layout)."""
        if batch is not self._batch_key:
            w_nb, w_site = engine.site_weights(self.kind, batch.numbers, batch.symbols, self.weights)
            self._w_nb = torch.from_numpy(w_nb).to(self.device)
            self._w_site = torch.from_numpy(w_site).to(self.device)
            self._species = torch.from_numpy(batch.species).to(self.device)
            self._struct = torch.from_numpy(np.repeat(np.arange(batch.nstruct), np.diff(batch.atom_ptr))).to(self.device)
            self._vol = torch.from_numpy(batch.volumes).to(self.device)
            # atoms of each species per structure: a model's per-species constant, summed exactly
            counts = np.zeros((batch.nstruct, max(len(batch.species_order), 1)))
            np.add.at(counts, (np.repeat(np.arange(batch.nstruct), np.diff(batch.atom_ptr)), batch.species), 1.0)
            self._counts = torch.from_numpy(counts).to(self.device)
            self._batch_key = batch
        return self

    def capture(self, batch: Batch, model, headroom=1.25, branches=None, pdl=None, host_io=False):
        """The whole energy / forces / stress step of this batch layout as one CUDA graph
        (see CapturedStep); call the result with new positions.  branches / pdl default to
        the calculator's tuning (2 and off untuned); host_io: the graph also copies the
        positions in from, and the results out to, pinned host buffers of the step."""
        return CapturedStep(self, batch, model, headroom=headroom, branches=self.branches if branches is None else branches,
                            pdl=self.pdl if pdl is None else pdl, host_io=host_io)

    def neighbors(self, batch: Batch, positions):
        return engine.build_neighbors(positions, batch.cells, batch.pbc, batch.atom_ptr, self.rcut, device=self.device)

    def descriptors(self, batch: Batch, positions=None, precision="fp64", derivative=True, stress=True):
        """Plain path for a batch: x, dxdr, rdxdr, seq on the device."""
        self.prepare(batch)
        pos = self._positions(batch, positions)
        nb = self.neighbors(batch, pos)
        x, dxdr, rdxdr = engine.plain(self.tables, self.params, nb, pos, self._w_nb, self._w_site,
                                      precision=0 if precision == "fp64" else 1, want_deriv=derivative,
                                      want_stress=stress)
        return dict(x=x, dxdr=dxdr, rdxdr=rdxdr, seq=nb.seq, pair_ptr=nb.pair_ptr, neighbors=nb)

    def _positions(self, batch, positions):
        if positions is None:
            positions = batch.positions
        if isinstance(positions, np.ndarray):
            positions = torch.from_numpy(np.ascontiguousarray(positions, dtype=np.float64))
        return positions.to(self.device, dtype=torch.float64, non_blocking=True).contiguous()

    def compute(self, batch: Batch, model, positions=None):
        """Energy (S,) f64, forces (N,3) f64, virial (S,3,3) f64, stress (S,6) GPa and B."""
        self.prepare(batch)
        pos = self._positions(batch, positions)
        nb = self.neighbors(batch, pos)
        if isinstance(model, LinearModel):
            # beta = dE/dB does not depend on B: forward and adjoint in one fused pass
            beta = model.coef.detach()[self._species]
            need = engine.lib().so4_linear_workspace_size(self.tables.handle, nb.natoms, nb.nimg)
            if self._ws is None or self._ws.numel() < need:
                self._ws = torch.empty(int(need * 1.25) + 4096, dtype=torch.uint8, device=self.device)
            x, forces, virial, energy = engine.adjoint_linear32(self.tables, self.params, nb, self._w_nb,
                                                                self._w_site, beta, workspace=self._ws)
            energy = energy + self._counts @ model.bias.detach().double()
            stress = -(virial.reshape(-1, 9)[:, VOIGT] / self._vol[:, None]) * EV_A3_TO_GPA
            return dict(energy=energy, forces=forces, virial=virial, stress=stress, x=x, neighbors=nb)
        x, utot = engine.forward32(self.tables, self.params, nb, self._w_nb, self._w_site)
        xg = x.detach().requires_grad_(True)
        with torch.enable_grad():
            e_atom = model(xg, self._species)
            beta, = torch.autograd.grad(e_atom.sum(), xg)
        forces, virial, energy = engine.adjoint32(self.tables, self.params, nb, self._w_nb, utot, beta,
                                                  eatom=e_atom.detach())
        stress = -(virial.reshape(-1, 9)[:, VOIGT] / self._vol[:, None]) * EV_A3_TO_GPA
        return dict(energy=energy, forces=forces, virial=virial, stress=stress, x=x, neighbors=nb,
                    energies=e_atom.detach())


def contract_plain(x, dxdr, rdxdr, seq, pair_ptr, atom_ptr, beta, volumes):
    """Forces and stress from the plain path's dxdr / rdxdr, as the reference's
    consumers contract them (neuralnetwork.py:492, 497, 677-678), in FP64:
      F_m = -sum_i beta_i . dxdr_dense[i, m],  stress = -sum_i beta_i . rdxdr_atom[i] x 160.21766."""
    dev = dxdr.device
    atom_ptr_t = torch.as_tensor(np.asarray(atom_ptr), device=dev)
    natoms = int(atom_ptr[-1])
    centre = torch.repeat_interleave(torch.arange(natoms, device=dev), (pair_ptr[1:] - pair_ptr[:-1]).long())
    struct = torch.repeat_interleave(torch.arange(len(atom_ptr) - 1, device=dev), (atom_ptr_t[1:] - atom_ptr_t[:-1]))
    base = atom_ptr_t[:-1][struct[centre]]
    j = seq[:, 1] + base
    b = beta.double()[centre]
    contrib = torch.einsum("pk,pkc->pc", b, dxdr.double())
    forces = torch.zeros((natoms, 3), dtype=torch.float64, device=dev).index_add_(0, j, -contrib)
    vir_pair = torch.einsum("pk,pkab->pab", b, rdxdr.double())
    vir = torch.zeros((len(atom_ptr) - 1, 3, 3), dtype=torch.float64, device=dev).index_add_(0, struct[centre], vir_pair)
    stress = -(vir.reshape(-1, 9)[:, VOIGT]) * EV_A3_TO_GPA
    energy = torch.zeros(len(atom_ptr) - 1, dtype=torch.float64, device=dev).index_add_(
        0, struct, (beta.double() * x.double()).sum(-1))
    return dict(forces=forces, stress=stress, energy=energy)


class CapturedStep:
    """Energy, forces and stress of one batch layout as a single CUDA graph replay.

    For fixed cells / pbc / atom ranges (an MD or relaxation loop moves only the
    positions), the whole step is captured once into a CUDA graph on static device
    buffers; a step copies the positions in and replays it, with no host
    synchronisation and no per-kernel launch cost.  For a LinearModel: the neighbour
    list, U_tot, the fused B + Y pass, the per-image dE/dr and the gather, then the
    per-structure constant and the stress, in parallel branches over ranges of atoms.
    For any other model of (B, species) whose forward can be captured (no host
    synchronisation; a species_index() method, as the NN potential's networks have,
    supplies the atoms of each species once): the list, U_tot and B, the model and its
    gradient dE/dB, Y, the per-image dE/dr and the gather, on one stream.  Either way the
    results equal those of SO4Calculator.compute bit for bit.

    The image / pair buffers have a fixed capacity (the counts of the structure at
    capture time plus `headroom`); the true counts are only known on the device.
    `check()` reads them (one small synchronising copy) and returns False when the
    neighbour list outgrew the buffers, after which the step must be captured again
    (`SO4Calculator.capture`); it raises for non-finite positions like the eager path.

    With host_io=True the step owns pinned host buffers, `host_positions` (N, 3) and
    `host_out` (energy, forces, stress), and the graph itself copies the positions in
    and the results out: a step is one graph launch and one wait, with no other call
    (an MD engine writes its positions into `host_positions` and reads `host_out`).
    """

    def __init__(self, calc: "SO4Calculator", batch: Batch, model, headroom=1.25, branches=2, pdl=False,
                 host_io=False):
        self.linear = isinstance(model, LinearModel)
        # programmatic dependent launch between U_tot, the window pass and the per-image pass
        # (so4_set_pdl): only for a linear energy, whose beta is fixed for the whole step
        self.pdl = bool(pdl) and self.linear
        calc.prepare(batch)
        # the graph reads these per-batch tensors by address: hold them, so that a later
        # prepare() of another batch cannot free them under the graph
        self._held = (calc._w_nb, calc._w_site, calc._species, calc._vol)
        dev = calc.device
        self.calc, self.batch = calc, batch
        self.layout = engine.layout(batch.cells, batch.pbc, batch.atom_ptr, calc.rcut, dev)
        lay = self.layout
        N, S = lay.natoms, lay.nstruct
        self.pos = torch.from_numpy(np.ascontiguousarray(batch.positions, dtype=np.float64)).to(dev)
        # learn the counts at capture time, then size the buffers with headroom
        nb0 = engine.build_neighbors(self.pos, batch.cells, batch.pbc, batch.atom_ptr, calc.rcut, device=dev)
        self.cap_m = int(nb0.nimg * headroom) + 64
        self.cap_p = int(nb0.npair * headroom) + 64 + N
        # one-pass neighbour list: per-atom key slots sized from the largest count seen now
        counts = torch.diff(nb0.img_ptr[: N + 1]).max().item() if N else 0
        self.slot_cap = (int(counts * headroom) + 8 + 7) // 8 * 8
        del nb0
        self.nl = engine.NeighborBuffers.allocate(lay, self.cap_m, self.cap_p, dev, slot_cap=self.slot_cap)
        L = engine.lib()
        tab = calc.tables
        if self.linear:
            self.ws = torch.empty(L.so4_linear_workspace_size(tab.handle, N, self.cap_m), dtype=torch.uint8,
                                  device=dev)
            self.beta = model.coef.detach()[calc._species].to(torch.float32).contiguous()
            self.bias_s = (calc._counts @ model.bias.detach().double()).contiguous()
        else:
            # any model of (B, species) -> per-atom energy whose forward is capturable: B, the
            # model and its gradient dE/dB, then the adjoint, as in the uncaptured compute();
            # a model with species_index() gets the atoms of each species precomputed
            self.model = model
            self.index = model.species_index(calc._species) if hasattr(model, "species_index") else None
            nh = tab.n_half
            self.fws = torch.empty(max(L.so4_forward32_workspace_size(tab.handle, N), 1), dtype=torch.uint8,
                                   device=dev)
            self.utot = torch.empty((max(N, 1), nh, 2), dtype=torch.float32, device=dev)
            self.ybuf = torch.empty((max(N, 1), nh, 2), dtype=torch.float32, device=dev)
            self.beta = torch.empty((max(N, 1), tab.nB), dtype=torch.float32, device=dev)
            self.eatom = torch.empty(max(N, 1), dtype=torch.float32, device=dev)
            self.energies = torch.empty(max(N, 1), dtype=torch.float64, device=dev)
            self.g = torch.empty((self.cap_m, 3), dtype=torch.float32, device=dev)
            self.part = torch.empty(L.so4_gather_workspace_size(N), dtype=torch.uint8, device=dev)
        self.x = torch.empty((max(N, 1), tab.nB), dtype=torch.float32, device=dev)
        self.forces = torch.empty((max(N, 1), 3), dtype=torch.float64, device=dev)
        self.virial = torch.empty((max(S, 1), 3, 3), dtype=torch.float64, device=dev)
        self.energy_sum = torch.empty(max(S, 1), dtype=torch.float64, device=dev)
        # Branches: after the neighbour list every stage up to the gather is independent per
        # centre, so consecutive ranges of atoms (cut at multiples of 32) run as parallel graph
        # branches and the tail of one branch's kernels overlaps the others' work.
        self.branches = max(1, min(int(branches), N // 128)) if self.linear else 1
        if self.branches > 1:
            cuts = [0] + [min(N, (N * k // self.branches + 31) // 32 * 32) for k in range(1, self.branches)] + [N]
            self.chunks = [(a0, a1) for a0, a1 in zip(cuts[:-1], cuts[1:]) if a1 > a0]
            self.branches = len(self.chunks)
            nh = tab.n_half
            self.utot = torch.empty((N, nh, 2), dtype=torch.float32, device=dev)
            self.ybuf = torch.empty((N, nh, 2), dtype=torch.float32, device=dev)
            self.bc = [torch.empty((max(tab.n_bsec, 1), a1 - a0), dtype=torch.float32, device=dev)
                       for a0, a1 in self.chunks]
            self.eatom = torch.empty(N, dtype=torch.float32, device=dev)
            self.g = torch.empty((self.cap_m, 3), dtype=torch.float32, device=dev)
            self.part = torch.empty(L.so4_gather_workspace_size(N), dtype=torch.uint8, device=dev)
            self.sides = [torch.cuda.Stream(device=dev) for _ in range(self.branches - 1)]
        self.energy = torch.empty(max(S, 1), dtype=torch.float64, device=dev)
        self.stress = torch.empty((max(S, 1), 6), dtype=torch.float64, device=dev)
        self._voigt = torch.tensor(VOIGT, device=dev)  # on the device before capture (no copies inside it)
        self.host_io = bool(host_io)
        if self.host_io:
            self.host_positions = torch.from_numpy(np.ascontiguousarray(batch.positions, dtype=np.float64)).pin_memory()
            self.host_out = dict(energy=torch.empty(S, dtype=torch.float64).pin_memory(),
                                 forces=torch.empty((N, 3), dtype=torch.float64).pin_memory(),
                                 stress=torch.empty((S, 6), dtype=torch.float64).pin_memory())
        self.launches = 0
        # eager warm-up on a side stream (sets kernel attributes, lets torch's allocator settle)
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            self._enqueue()
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        c0 = L.so4_launch_count()
        with torch.cuda.graph(self.graph):
            self._enqueue()
        self.launches = int(L.so4_launch_count() - c0)  # kernels of this library in one replay

    def _enqueue(self):
        if self.host_io:  # the positions from the pinned host buffer, as a node of the graph
            self.pos.copy_(self.host_positions, non_blocking=True)
        if not self.linear:
            self._enqueue_model()
        else:
            L = engine.lib()
            prev = L.so4_set_pdl(1 if self.pdl else 0)
            try:
                self._enqueue_linear()
            finally:
                L.so4_set_pdl(prev)
        if self.host_io:  # and the results back to the pinned host buffers
            N, S = self.layout.natoms, self.layout.nstruct
            self.host_out["energy"].copy_(self.energy[:S], non_blocking=True)
            self.host_out["forces"].copy_(self.forces[:N], non_blocking=True)
            self.host_out["stress"].copy_(self.stress[:S], non_blocking=True)

    def _enqueue_linear(self):
        lay, calc, tab, L = self.layout, self.calc, self.calc.tables, engine.lib()
        b = self.nl
        _p = engine._ptr
        check = engine.check
        if self.branches == 1:
            engine.enqueue_neighbors(lay, self.pos, b, lite=True)
            check(L.so4_adjoint_linear32(tab.handle, C.byref(calc.params), lay.nstruct, _p(lay.atom_struct),
                                         _p(lay.atom_ptr_dev), lay.natoms, _p(calc._w_nb), _p(calc._w_site),
                                         _p(b.img_ptr), _p(b.img_j), _p(b.img_r), _p(b.img_rev), self.cap_m,
                                         _p(self.beta), _p(self.x), _p(self.forces), _p(self.virial),
                                         _p(self.energy_sum), _p(self.ws), self.ws.numel(), engine._stream()),
                  "so4_adjoint_linear32")
        else:
            # the list itself runs per branch: bins for all atoms, then each branch counts and
            # sorts its own centres (their scans chained in branch order) and goes on to its
            # compute while the other branches' lists are still being built; the reverse images
            # (read only by the gather) and the summary follow the join
            N, S_, G = lay.natoms, lay.nstruct, lay.nbins
            check(L.so4_nl_bins(_p(lay.geom), S_, G, _p(self.pos), _p(lay.atom_struct), N, b.slot_cap, _p(b.ws),
                                b.ws.numel(), engine._stream()), "so4_nl_bins")
            main = torch.cuda.current_stream()
            for sd in self.sides:
                sd.wait_stream(main)
            scanned = None
            for (a0, a1), bc, st in zip(self.chunks, self.bc, [main] + self.sides):
                with torch.cuda.stream(st):
                    s_ = engine._stream()
                    n = a1 - a0
                    check(L.so4_nl_count_keys_range(_p(lay.geom), S_, G, _p(self.pos), _p(lay.atom_struct), N,
                                                    lay.rcut, b.slot_cap, a0, a1, _p(b.ws), b.ws.numel(), s_),
                          "so4_nl_count_keys_range")
                    if scanned is not None:
                        st.wait_event(scanned)
                    check(L.so4_nl_scan_range(N, G, b.slot_cap, a0, a1, _p(b.img_ptr), _p(b.ws), b.ws.numel(), s_),
                          "so4_nl_scan_range")
                    scanned = torch.cuda.Event()
                    scanned.record(st)
                    check(L.so4_nl_sort_range(_p(lay.geom), S_, G, _p(self.pos), _p(lay.atom_struct), N, a0, a1,
                                              _p(b.img_ptr), b.cap_m, b.slot_cap, _p(b.img_j), _p(b.img_off),
                                              _p(b.img_r), _p(b.ws), b.ws.numel(), s_), "so4_nl_sort_range")
                    check(L.so4_utot32(tab.handle, C.byref(calc.params), n, _p(calc._w_nb), _p(calc._w_site[a0:a1]),
                                       _p(b.img_ptr[a0:a1 + 1]), _p(b.img_j), _p(b.img_r), _p(self.utot[a0:a1]),
                                       s_), "so4_utot32")
                    check(L.so4_linear_by32(tab.handle, n, _p(self.utot[a0:a1]), _p(self.beta[a0:a1]),
                                            _p(self.x[a0:a1]), _p(self.ybuf[a0:a1]), _p(bc), _p(self.eatom[a0:a1]),
                                            s_), "so4_linear_by32")
                    check(L.so4_adjoint_deidrj32(tab.handle, C.byref(calc.params), n, _p(calc._w_nb),
                                                 _p(b.img_ptr[a0:a1 + 1]), _p(b.img_j), _p(b.img_r), self.cap_m,
                                                 _p(self.ybuf[a0:a1]), _p(self.g), s_), "so4_adjoint_deidrj32")
            for sd in self.sides:
                main.wait_stream(sd)
            check(L.so4_nl_pairs(_p(lay.geom), S_, _p(lay.atom_struct), N, _p(b.img_ptr), b.cap_m, _p(b.img_j),
                                 _p(b.img_off), _p(None), b.cap_p, _p(None), _p(None), _p(None), _p(None),
                                 _p(b.img_rev), _p(b.ws), b.ws.numel(), engine._stream()), "so4_nl_pairs")
            check(L.so4_nl_summary(_p(b.img_ptr), _p(None), N, _p(b.ws), b.ws.numel(), engine._stream(), None),
                  "so4_nl_summary")
            check(L.so4_adjoint_gather(lay.natoms, lay.nstruct, _p(lay.atom_ptr_dev), _p(b.img_ptr), _p(b.img_rev),
                                       _p(b.img_r), _p(self.g), _p(self.eatom), _p(self.part), _p(self.forces),
                                       _p(self.virial), _p(self.energy_sum), engine._stream()), "so4_adjoint_gather")
        S = lay.nstruct
        torch.add(self.energy_sum[:S], self.bias_s, out=self.energy[:S])
        # same operations as the uncaptured path, so the two agree bit for bit
        self.stress[:S].copy_(-(self.virial[:S].reshape(S, 9)[:, self._voigt] / self.calc._vol[:, None]) * EV_A3_TO_GPA)

    def _enqueue_model(self):
        """The general-model step: neighbour list, U_tot and B (so4_forward32), the model and
        beta = dE/dB by autograd, Y, the per-image dE/dr and the gather with the per-atom
        energies -- the kernels and order of SO4Calculator.compute, so the two agree bit for bit."""
        lay, calc, tab, L = self.layout, self.calc, self.calc.tables, engine.lib()
        b, _p, check, st = self.nl, engine._ptr, engine.check, engine._stream()
        N, S = lay.natoms, lay.nstruct
        engine.enqueue_neighbors(lay, self.pos, b, lite=True)
        check(L.so4_forward32(tab.handle, C.byref(calc.params), N, _p(calc._w_nb), _p(calc._w_site), _p(b.img_ptr),
                              _p(b.img_j), _p(b.img_r), _p(self.utot), _p(self.x), _p(self.fws), self.fws.numel(), st),
              "so4_forward32")
        xg = self.x[:N].detach().requires_grad_(True)
        with torch.enable_grad():
            if self.index is not None:
                e_atom = self.model(xg, calc._species, self.index)
            else:
                e_atom = self.model(xg, calc._species)
            beta, = torch.autograd.grad(e_atom.sum(), xg)
        self.beta[:N].copy_(beta)
        self.energies[:N].copy_(e_atom.detach())
        self.eatom[:N].copy_(e_atom.detach())
        check(L.so4_adjoint_y32(tab.handle, N, _p(self.utot), _p(self.beta), _p(self.ybuf), st), "so4_adjoint_y32")
        check(L.so4_adjoint_deidrj32(tab.handle, C.byref(calc.params), N, _p(calc._w_nb), _p(b.img_ptr),
                                     _p(b.img_j), _p(b.img_r), self.cap_m, _p(self.ybuf), _p(self.g), st),
              "so4_adjoint_deidrj32")
        check(L.so4_adjoint_gather(N, S, _p(lay.atom_ptr_dev), _p(b.img_ptr), _p(b.img_rev), _p(b.img_r), _p(self.g),
                                   _p(self.eatom), _p(self.part), _p(self.forces), _p(self.virial),
                                   _p(self.energy), st), "so4_adjoint_gather")
        self.stress[:S].copy_(-(self.virial[:S].reshape(S, 9)[:, self._voigt] / calc._vol[:, None]) * EV_A3_TO_GPA)

    def __call__(self, positions=None):
        """One step; positions (N,3) f64 from the host (pinned for an asynchronous copy)
        or the device, or None to reuse the last ones.  Returns views of the static
        outputs (valid until the next call).  With host_io: positions (if given) are first
        written into `host_positions`, and the call waits for the step and returns
        `host_out`."""
        if self.host_io:
            if positions is not None:
                if not isinstance(positions, torch.Tensor):
                    positions = torch.from_numpy(np.ascontiguousarray(positions, dtype=np.float64))
                self.host_positions.copy_(positions)
            self.graph.replay()
            torch.cuda.current_stream(self.pos.device).synchronize()
            return self.host_out
        if positions is not None:
            if isinstance(positions, np.ndarray):
                positions = torch.from_numpy(np.ascontiguousarray(positions, dtype=np.float64))
            self.pos.copy_(positions, non_blocking=True)
        self.graph.replay()
        N, S = self.layout.natoms, self.layout.nstruct
        out = dict(energy=self.energy[:S], forces=self.forces[:N], virial=self.virial[:S], stress=self.stress[:S],
                   x=self.x[:N])
        if not self.linear:
            out["energies"] = self.energies[:N]
        return out

    def check(self):
        """True if the last step's neighbour list fitted its buffers (raises on bad input)."""
        M, P, bits = [int(v) for v in self.nl.summary_dev().cpu()]
        return engine.check_summary(M, P, bits, self.cap_m, self.cap_p)
