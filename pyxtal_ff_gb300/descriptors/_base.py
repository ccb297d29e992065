"""Shared implementation of the drop-in SO4 / SNAP descriptor classes.

Mirrors pyxtal_ff/descriptors/SO4.py:10-304 (and SNAP.py:10-334): the same
constructor arguments, property validation and exception types, save_dict /
load_from_dict keys, clear_memory(), and calculate(atoms, atom_ids=None)
returning the same dict -- computed by the CUDA path in FP64.
"""
from __future__ import annotations

import numpy as np

_CUTOFFS = {"cosine": 1, "tanh": 2, "poly1": 3, "poly2": 4, "poly3": 5, "poly4": 6, "exp": 7}


class BispectrumBase:
    _kind = "SO4"
    _essential = {"_twol", "_rcut", "_derivative", "_stress", "_norm", "_cutoff_function", "_cutoff_id"}

    # -- properties (SO4.py:63-158)
    @property
    def lmax(self):
        return self._twol // 2

    @property
    def rcut(self):
        return self._rcut

    @rcut.setter
    def rcut(self, rcut):
        if isinstance(rcut, float) is True or isinstance(rcut, int) is True:
            if rcut <= 0:
                raise ValueError("rcut must be greater than zero")
            self._rcut = rcut
        else:
            raise ValueError("rcut must be a float")

    @property
    def derivative(self):
        return self._derivative

    @derivative.setter
    def derivative(self, derivative):
        if isinstance(derivative, bool) is True:
            self._derivative = derivative
        else:
            raise ValueError("derivative must be a boolean value")

    @property
    def stress(self):
        return self._stress

    @stress.setter
    def stress(self, stress):
        if isinstance(stress, bool) is True:
            self._stress = stress
        else:
            raise ValueError("stress must be a boolean value")

    @property
    def normalize_U(self):
        return self._norm

    @normalize_U.setter
    def normalize_U(self, normalize_U):
        if isinstance(normalize_U, bool) is True:
            self._norm = normalize_U
        else:
            raise ValueError("normalize_U must be a boolean value")

    @property
    def cutoff_function(self):
        return self._cutoff_function

    @cutoff_function.setter
    def cutoff_function(self, cutoff_function):
        if isinstance(cutoff_function, str) is True:
            if cutoff_function in _CUTOFFS:
                self._cutoff_id = _CUTOFFS[cutoff_function]
                self._cutoff_function = cutoff_function
            else:
                raise NotImplementedError("The requested cutoff function has not been implemented")
        else:
            raise ValueError("You must specify the cutoff function as a string")

    def clear_memory(self):
        """Drop every attribute but the parameters (SO4.py:160-169)."""
        for attr in list(vars(self).keys()):
            if attr not in self._essential:
                delattr(self, attr)

    def __repr__(self):
        return str(self)

    # -- the computation
    def _weights(self, numbers, symbols):
        raise NotImplementedError

    def _rfac0(self):
        return 1.0

    def calculate(self, atoms, atom_ids=None, *, stress_per_atom=False):
        """B, dB/dr and the per-pair virial of one structure, as the reference's
        calculate() returns them (SO4.py:171-209), from the CUDA FP64 path.

        stress_per_atom=True returns rdxdr already reduced the way the reference's
        caller reduces it after calculate() (pyxtal_ff/utilities/__init__.py:226-233):
        one (len(x), nB, 6) Voigt row block per centre, summed on the GPU, so the
        per-pair array never leaves the device."""
        import torch
        from .. import engine
        from ..structures import as_arrays

        engine.require_cuda()
        self._atoms = atoms
        vol = atoms.get_volume()
        pos, cell, pbc, numbers, symbols = as_arrays(atoms)
        n = len(pos)
        if atom_ids is None:
            k = n
        else:
            ids = [int(i) for i in atom_ids]
            k = len(ids)
            if ids != list(range(k)) or k > n:
                # the reference indexes its per-centre arrays by atom id (SO4.py:224-232),
                # so only a prefix range(k) is meaningful there
                raise IndexError("atom_ids must be range(k) with k <= len(atoms)")
        dev = torch.device("cuda", torch.cuda.current_device())
        twol = self._twol
        tab = engine.tables(twol, self._norm)
        prm = engine.params(twol, self._rcut, self._rfac0(), self._cutoff_function)
        pos_d = torch.from_numpy(pos).to(dev)
        nb = engine.build_neighbors(pos_d, cell[None], pbc[None], [0, n], self._rcut, device=dev)
        counts = np.diff(nb.img_ptr[: k + 1].cpu().numpy())
        if k and np.any(counts == 0):
            # the reference cannot pad an empty neighbour list (SO4.py:274-276 raises
            # "could not broadcast input array from shape (0,) into shape (0,3)")
            i = int(np.nonzero(counts == 0)[0][0])
            raise ValueError("atom %d has no neighbour within rcut=%g" % (i, self._rcut))
        w_nb, w_site = self._weights(numbers, symbols)
        w_nb_d = torch.from_numpy(w_nb).to(dev)
        w_site_d = torch.from_numpy(w_site).to(dev)
        x, dxdr, rdxdr = engine.plain(tab, prm, nb, pos_d, w_nb_d, w_site_d, precision=0,
                                      want_deriv=self._derivative, want_stress=self._stress)
        pk = int(nb.pair_ptr[k].item())
        out_x = x[:k].cpu().numpy()
        elements = list(atoms.symbols)
        if self._derivative:
            res = {"x": out_x, "dxdr": dxdr[:pk].cpu().numpy(), "elements": elements,
                   "seq": nb.seq[:pk].cpu().numpy()}
            if not self._stress:
                res["rdxdr"] = None
            elif stress_per_atom:
                res["rdxdr"] = engine.rdxdr_atom(rdxdr, nb.pair_ptr, k).cpu().numpy()
            else:
                res["rdxdr"] = rdxdr[:pk].cpu().numpy()
        else:
            res = {"x": out_x, "dxdr": None, "elements": elements}
            # without derivatives the reference never fills bstress (SO4.py:1671-1728),
            # so it returns -0/vol over every pair (and its caller's per-atom sum, +0)
            if not self._stress:
                res["rdxdr"] = None
            elif stress_per_atom:
                res["rdxdr"] = np.zeros((k, tab.nB, 6))
            else:
                res["rdxdr"] = -np.zeros((pk, tab.nB, 3, 3)) / vol
        self.clear_memory()
        return res
