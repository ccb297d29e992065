"""The reference NN potential's prediction side, on the GPU.

``NeuralNetworkPotential`` holds what the reference's ``NeuralNetwork`` keeps for
prediction after ``load_checkpoint`` (pyxtal_ff/models/neuralnetwork.py:838-893):
the elements (sorted), one torch network per element, the descriptor range
``drange`` per element and the energy unit.

- ``calculate_properties(descriptor, bforce, bstress)`` returns what the reference
  method of that name returns (:579-678): per-atom energies stored element after
  element (sorted), forces (N, 3) and stress (6,) in GPa.  The descriptors are
  scaled per element into [0, 1] (x' = (x - dmin) / (dmax - dmin)), so dE/dx =
  dE/dx' / (dmax - dmin); the force and stress contractions of dE/dx with the
  plain path's dxdr and per-atom rdxdr run in ``so4_contract_dxdr`` (one warp per
  target atom over the reverse pairs, fixed summation order) instead of the
  reference's dense (N_e, N, nB, 3) array (N <= 400) or one np.where over all
  pairs per atom (N > 400).
- ``energy_model(species_order)`` is the same networks as a module of
  (x, species) -> per-atom energy, for the adjoint path (``SO4Calculator.compute``),
  where dxdr is never formed.

Differences from the reference, both outside what a valid input meets: atoms of
one element need not be contiguous (the reference slices x[e[0]:e[-1]+1] and fails
on interleaved elements), and with unit 'Ha' the stress rows are scaled by
0.529177^3 (the reference adds the scaled dxdr there, a shape error).
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine

EV2GPA = 160.21766
BOHR = 0.529177


class NeuralNetworkPotential:
    def __init__(self, models, drange, elements=None, unit="eV", device="cuda", path=""):
        if unit not in ("eV", "Ha"):
            raise NotImplementedError(f"{unit} is not implemented. Please choose from ['eV', 'Ha'].")
        self.elements = sorted(elements if elements is not None else models.keys())
        self.unit = unit
        self.path = path
        self.device = torch.device(device)
        self.models = {e: models[e].to(self.device) for e in self.elements}
        self.drange = {e: np.asarray(drange[e], dtype=np.float64) for e in self.elements}
        self._dmin = {e: torch.from_numpy(self.drange[e][:, 0].copy()).to(self.device) for e in self.elements}
        self._scale = {e: torch.from_numpy(1.0 / (self.drange[e][:, 1] - self.drange[e][:, 0])).to(self.device)
                       for e in self.elements}

    @classmethod
    def from_checkpoint(cls, checkpoint, device="cuda"):
        """From the dict the reference's save_checkpoint writes (neuralnetwork.py:681-716)."""
        if checkpoint["algorithm"] != "NN":
            raise NotImplementedError("The loaded algorithm is not Neural Network.")
        return cls(checkpoint["models"], checkpoint["drange"], checkpoint["elements"], checkpoint["unit"], device)

    def _dtype(self, e):
        return next(self.models[e].parameters()).dtype

    def energies_and_dedx(self, x, symbols):
        """Per-atom energies (element-grouped order, as the reference stores them), the
        atom order of that grouping, and dE/dx (N, nB) of the raw descriptors."""
        symbols = np.asarray(symbols)
        n = x.shape[0]
        dedx = torch.zeros_like(x)
        energies, order = [], []
        for e in self.elements:
            idx_np = np.nonzero(symbols == e)[0]
            if len(idx_np) == 0:
                continue
            idx = torch.from_numpy(idx_np).to(self.device)
            dt = self._dtype(e)
            xe = ((x[idx] - self._dmin[e]) * self._scale[e]).to(dt).requires_grad_(True)
            with torch.enable_grad():
                out = self.models[e](xe)
                g, = torch.autograd.grad(out.sum(), xe)
            energies.append(out.detach().reshape(-1).to(torch.float64))
            order.append(idx_np)
            dedx[idx] = g.to(x.dtype) * self._scale[e]
        if set(symbols.tolist()) - set(self.elements):
            raise KeyError(sorted(set(symbols.tolist()) - set(self.elements))[0])
        en = torch.cat(energies) if energies else torch.zeros(0, dtype=torch.float64, device=self.device)
        return en, (np.concatenate(order) if order else np.zeros(0, np.int64)), dedx[:n]

    def calculate_properties(self, descriptor, bforce=True, bstress=False):
        """energies (N,), forces (N, 3), stress (6,) GPa, numpy FP64 (neuralnetwork.py:579-678).

        descriptor: the plain path's dict -- x (N, nB), dxdr (P, nB, 3), seq (P, 2),
        rdxdr (N, nB, 6) per-atom Voigt rows (the caller's reduction), elements --
        as numpy arrays or device tensors."""
        dev = self.device

        def dev64(a):
            return torch.as_tensor(a).to(dev, dtype=torch.float64).contiguous()

        x = dev64(descriptor["x"])
        n = x.shape[0]
        energies, _, dedx = self.energies_and_dedx(x, descriptor["elements"])
        forces = np.zeros((n, 3))
        stress = np.zeros(6)
        if (bforce or bstress) and n > 0:
            seq = torch.as_tensor(descriptor["seq"]).to(dev, dtype=torch.int64).contiguous()
            counts = torch.bincount(seq[:, 0], minlength=n)
            pair_ptr = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(counts, 0)]).int()
            atom_struct = torch.zeros(n, dtype=torch.int32, device=dev)
            atom_ptr = torch.tensor([0, n], dtype=torch.int32, device=dev)
            fscale = BOHR if self.unit == "Ha" else 1.0
            sscale = BOHR ** 3 if self.unit == "Ha" else 1.0
            dxdr = dev64(descriptor["dxdr"]) * fscale if bforce else None
            rd = dev64(descriptor["rdxdr"]) * sscale if bstress else None
            f, s = engine.contract_dxdr(dedx, pair_ptr, seq, atom_struct, atom_ptr, dxdr=dxdr, rdxdr_atom=rd)
            if f is not None:
                forces = f.cpu().numpy()
            if s is not None:
                stress = s[0].cpu().numpy() * EV2GPA
        return energies.cpu().numpy(), forces, stress

    @property
    def no_of_descriptors(self):
        first = next(m for m in self.models[self.elements[0]].modules() if isinstance(m, torch.nn.Linear))
        return first.in_features

    def save_weights_to_txt(self, des_info):
        """NN_weights.txt and DescriptorParam.txt for LAMMPS ML-IAP under the prefix self.path
        (neuralnetwork.py:719-836; the format is in lammps_export)."""
        from .lammps_export import write_nn
        write_nn(self.path, self.elements, self.models, self.drange, self.no_of_descriptors, des_info)

    def energy_model(self, species_order):
        """The networks as a module (x (N, nB), species (N,) indices into species_order)
        -> per-atom energies, with the drange scaling inside."""
        return _SpeciesNetworks(self, list(species_order))


class _SpeciesNetworks(torch.nn.Module):
    def __init__(self, pot: NeuralNetworkPotential, species_order):
        super().__init__()
        self.pot = pot
        self.species_order = species_order
        self.nets = torch.nn.ModuleList([pot.models[s] for s in species_order])

    def species_index(self, species):
        """The atoms of each species, in species_order (one synchronising nonzero each)."""
        return [torch.nonzero(species == k).reshape(-1) for k in range(len(self.species_order))]

    def forward(self, x, species, index=None):
        """index: the atoms of each species (a list of index tensors, as species_index
        returns); given, the forward has no host synchronisation and can be graph-captured."""
        out = torch.zeros(x.shape[0], dtype=torch.float64, device=x.device)
        if index is None:
            index = self.species_index(species)
        for k, name in enumerate(self.species_order):
            idx = index[k]
            if idx.numel() == 0:
                continue
            p = self.pot
            dt = p._dtype(name)
            xe = ((x[idx].to(torch.float64) - p._dmin[name]) * p._scale[name]).to(dt)
            out = out.index_put((idx,), self.nets[k](xe).reshape(-1).to(torch.float64))
        return out
