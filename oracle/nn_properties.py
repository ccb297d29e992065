"""CPU restatement of the reference NN potential's property evaluation (test
infrastructure only: the checker, never the product path).

``calculate_properties`` follows pyxtal_ff/models/neuralnetwork.py:579-678:
per element (sorted), the descriptors of its atoms are scaled into [0, 1] by
drange (scale = 1 / (dmax - dmin), x' = scale (x - dmin), dxdr' = scale dxdr,
rdxdr' = scale rdxdr; :603-633), the element's network gives per-atom energies
(stored element after element, :650-655), dE/dx' comes from autograd, and
  forces[m] -= sum over pairs p with seq[p, 1] == m of dE/dx'[seq[p, 0]] . dxdr'[p]
(the dense (N_e, N, nB, 3) form of :668-673), stress -= sum_i dE/dx'[i] . rdxdr'[i]
(:675-678), times 160.21766 for GPa.  The networks are torch modules, as in the
reference (the model, not the path); the contraction is numpy in FP64.

``voigt_atom`` is the caller's per-atom stress-row reduction
(pyxtal_ff/utilities/__init__.py:226-233).
"""
import numpy as np

EV2GPA = 160.21766


def voigt_atom(rdxdr, seq, natoms):
    """(P, nB, 3, 3) per pair -> (natoms, nB, 6): the sum over each centre's pairs, then
    the flattened entries 0, 4, 8, 1, 2, 5."""
    out = np.zeros((natoms, rdxdr.shape[1], 3, 3))
    np.add.at(out, np.asarray(seq)[:, 0], rdxdr)
    return out.reshape(natoms, rdxdr.shape[1], 9)[:, :, [0, 4, 8, 1, 2, 5]]


def calculate_properties(models, drange, elements, descriptor, bforce=True, bstress=False):
    """energies (N,) in element order, forces (N, 3), stress (6,) GPa."""
    import torch
    x = np.asarray(descriptor["x"], dtype=np.float64)
    seq = np.asarray(descriptor["seq"])
    symbols = np.asarray(descriptor["elements"])
    n = x.shape[0]
    energies, forces, stress = np.zeros(n), np.zeros((n, 3)), np.zeros(6)
    count = 0
    for e in sorted(elements):
        idx = np.nonzero(symbols == e)[0]
        if len(idx) == 0:
            continue
        scale = 1.0 / (drange[e][:, 1] - drange[e][:, 0])
        xe = torch.from_numpy(scale * (x[idx] - drange[e][:, 0])).requires_grad_(True)
        out = models[e](xe)
        energies[count:count + len(idx)] = out.detach().numpy().reshape(-1)
        count += len(idx)
        dedx = torch.autograd.grad(out.sum(), xe)[0].numpy() * scale  # dE/dx of the raw descriptors
        if bforce:
            dense = np.zeros((len(idx), n, x.shape[1], 3))
            pos = {int(a): r for r, a in enumerate(idx)}
            dxdr = np.asarray(descriptor["dxdr"])
            for p in range(len(seq)):
                i = int(seq[p, 0])
                if i in pos:
                    dense[pos[i], int(seq[p, 1])] += dxdr[p]
            forces -= np.einsum("ik,ijkl->jl", dedx, dense)
        if bstress:
            stress -= np.einsum("ik,ikl->l", dedx, np.asarray(descriptor["rdxdr"])[idx])
    return energies, forces, stress * EV2GPA
