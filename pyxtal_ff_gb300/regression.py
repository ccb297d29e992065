"""The reference's polynomial (order 1 and 2) potential, with its design matrix built
on the GPU.

``PolynomialRegressionPotential`` mirrors pyxtal_ff/models/polynomialregression.py
(class PR): ``parse_descriptors`` returns the same design matrix X (:438-682), rows
per structure -- the energy row (per element: the atom count and the summed
descriptors), three force rows per atom, six stress rows for structures in the
stress group -- or, with train=False (one structure), one energy row per atom;
``calculate_properties`` is X . coef_ (:374-411); ``LinearRegression`` the same
weighted, optionally L2/L1-regularised least squares (:240-260) on the GPU;
``save_weights_to_txt`` the LAMMPS export (:286-345).

The force and stress rows, which the reference fills with one np.where over all
pairs per atom, come from so4_design_forces (one warp per target atom over its
reverse pairs, per source element) and so4_design_struct; the per-atom energy rows
of train=False are plain copies.  Order 2 (quadratic SNAP, :488-559) uses the features
x_a, then per d1 the square 0.5 x_d1^2 and the products x_d1 x_d2 (d2 > d1) of the first
d_max descriptors, with the force and stress rows from so4_design_forces_q and
so4_design_struct_q (the derivative of a feature along a pair's dxdr uses the pair's
centre descriptors, as the reference's does).
"""
from __future__ import annotations

import numpy as np
import torch

from . import engine

EV2GPA = 160.21766


class PolynomialRegressionPotential:
    def __init__(self, elements, coef_=None, order=1, d_max=None, path="", force_coefficient=None,
                 stress_coefficient=None, stress_group=None, alpha=None, norm=2, device="cuda"):
        if order not in (1, 2):
            raise ValueError("Order must be 1 or 2")
        self.elements = sorted(elements)
        self.order = order
        self.quadratic = order == 2
        self.coef_ = None if coef_ is None else np.asarray(coef_, dtype=np.float64)
        self.d_max = d_max
        self.path = path
        self.force_coefficient = force_coefficient
        self.stress_coefficient = stress_coefficient
        self.stress_group = stress_group
        self.alpha = alpha
        self.norm = norm
        self.unit = "eV"
        self.device = torch.device(device)

    # ------------------------------------------------------------ design matrix
    @staticmethod
    def features(d, quadratic):
        """(F, 2) int32 feature table in the reference's column order: (a, -1) for x_a, then
        per d1 (d1, d1) for 0.5 x_d1^2 and (d1, d2) for x_d1 x_d2, d2 > d1."""
        f = [(a, -1) for a in range(d)]
        if quadratic:
            for d1 in range(d):
                f.append((d1, d1))
                f.extend((d1, d2) for d2 in range(d1 + 1, d))
        return np.asarray(f, dtype=np.int32)

    def _stack(self, descs, d_max):
        """Concatenate structures on the device: x (N, d), dxdr (P, d, 3), seq (P, 2) local,
        rdxdr (N, d, 6), species (N,), atom / pair pointers."""
        dev = self.device
        xs, ds, qs, rs, sp, nat, npr = [], [], [], [], [], [], []
        idx = {e: i for i, e in enumerate(self.elements)}
        for d in descs:
            x = torch.as_tensor(d["x"]).to(dev, torch.float64)[:, :d_max]
            xs.append(x)
            sp.append(torch.tensor([idx[e] for e in d["elements"]], dtype=torch.int32))
            nat.append(x.shape[0])
            if d.get("dxdr") is not None:
                ds.append(torch.as_tensor(d["dxdr"]).to(dev, torch.float64)[:, :d_max, :])
                q = torch.as_tensor(d["seq"]).to(dev, torch.int64)
                qs.append(q)
                npr.append(torch.bincount(q[:, 0], minlength=x.shape[0]))
            if d.get("rdxdr") is not None:
                rs.append(torch.as_tensor(d["rdxdr"]).to(dev, torch.float64)[:, :d_max, :])
        out = dict(x=torch.cat(xs).contiguous(), species=torch.cat(sp).to(dev).contiguous(),
                   atom_ptr=torch.tensor(np.concatenate([[0], np.cumsum(nat)]), dtype=torch.int32, device=dev))
        out["atom_struct"] = torch.repeat_interleave(torch.arange(len(descs), dtype=torch.int32, device=dev),
                                                     torch.tensor(nat, device=dev))
        if len(ds) == len(descs):
            out["dxdr"] = torch.cat(ds).contiguous()
            out["seq"] = torch.cat(qs).contiguous()
            cnt = torch.cat(npr)
            out["pair_ptr"] = torch.cat([torch.zeros(1, dtype=torch.int64, device=dev), torch.cumsum(cnt, 0)]).int()
        if len(rs) == len(descs):
            out["rdxdr"] = torch.cat(rs).contiguous()
        return out

    def design_matrix(self, descs, fc=True, sc=False, train=True, stress_rows=None):
        """X on the device for a list of descriptor dicts (x, dxdr, seq, rdxdr per atom
        in Voigt order, elements).  stress_rows[s]: whether structure s gets stress rows
        (default: all when sc)."""
        if self.d_max is None:
            self.d_max = len(np.asarray(descs[0]["x"])[0])
        d = self.d_max
        ne = len(self.elements)
        feat_np = self.features(d, self.quadratic)
        nf = len(feat_np)
        ncols = (1 + nf) * ne
        S = len(descs)
        st = self._stack(descs, d)
        nat = [int(np.asarray(dd["x"]).shape[0]) for dd in descs]
        if stress_rows is None:
            stress_rows = [bool(sc)] * S
        # row layout, structure after structure (:578-603): energy row(s), forces, stress
        energy_row, force_row, stress_row = [], [], []
        r = 0
        for s in range(S):
            energy_row.append(r if train else -1)
            r += 1 if train else nat[s]
            force_row.append(r)
            r += 3 * nat[s] if fc else 0
            stress_row.append(r if (sc and stress_rows[s]) else -1)
            r += 6 if (sc and stress_rows[s]) else 0
        dev = self.device
        X = torch.zeros((r, ncols), dtype=torch.float64, device=dev)
        t64 = lambda v: torch.tensor(v, dtype=torch.int64, device=dev)  # noqa: E731
        feat = torch.from_numpy(feat_np).to(dev)
        if not train:  # one energy row per atom: [1, features(x_i)] in the atom's element block
            if S != 1:
                raise ValueError("train=False takes one structure")
            rows = torch.arange(nat[0], device=dev)
            c0 = st["species"].long() * (1 + nf)
            X[rows, c0] = 1.0
            xv = st["x"]
            f1, f2 = feat[:, 0].long(), feat[:, 1].long()
            sq = (f2 == f1).to(xv.dtype)
            quad = xv[:, f1] * xv[:, f2.clamp(min=0)] * (1.0 - 0.5 * sq)
            vals = torch.where((f2 < 0)[None, :], xv[:, f1], quad)
            X[rows[:, None], c0[:, None] + 1 + torch.arange(nf, device=dev)] = vals
        if fc and nat and sum(nat):
            if "dxdr" not in st:
                raise ValueError("fc=True needs dxdr and seq")
            if self.quadratic:
                engine.design_forces_q(X, ncols, d, feat, ne, st["species"], st["pair_ptr"], st["seq"],
                                       st["atom_struct"], st["atom_ptr"], st["x"], st["dxdr"], t64(force_row))
            else:
                engine.design_forces(X, ncols, d, ne, st["species"], st["pair_ptr"], st["seq"], st["atom_struct"],
                                     st["atom_ptr"], st["dxdr"], t64(force_row))
        want_s = any(v >= 0 for v in stress_row)
        if train or want_s:
            if want_s and "rdxdr" not in st:
                raise ValueError("sc=True needs per-atom rdxdr")
            rd = st.get("rdxdr") if want_s else None
            srow = t64(stress_row) if want_s else None
            if self.quadratic:
                engine.design_struct_q(X, ncols, d, feat, ne, st["species"], st["atom_ptr"], st["x"], rd,
                                       t64(energy_row), srow)
            else:
                engine.design_struct(X, ncols, d, ne, st["species"], st["atom_ptr"], st["x"], rd, t64(energy_row),
                                     srow)
        return X

    def parse_descriptors(self, data, fc=True, sc=False, train=True):
        """X (numpy) as the reference's parse_descriptors returns it.  data: the mapping
        '0', '1', ... -> descriptor dict the reference reads from its database (train) or
        {'0': descriptor} (train=False); a structure gets stress rows when sc and (train)
        its 'group' is in self.stress_group."""
        n = len(data)
        descs = [data[str(i)] for i in range(n)]
        if train:
            groups = [dd.get("group") for dd in descs]
            sg = self.stress_group or []
            rows = [g in sg for g in groups]
        else:
            rows = [True] * n
        return self.design_matrix(descs, fc=fc, sc=sc, train=train, stress_rows=rows).cpu().numpy()

    # ------------------------------------------------------------ model
    def calculate_properties(self, descriptor, bforce=True, bstress=False):
        """energies (N,), forces (N, 3), stress (6,) GPa = the rows of X . coef_ (:374-411)."""
        n = len(descriptor["elements"])
        X = self.design_matrix([descriptor], fc=bforce, sc=bstress, train=False)
        y = X @ torch.from_numpy(self.coef_).to(X.device)
        y = y.cpu().numpy()
        energies = y[:n]
        force = np.zeros((n, 3))
        stress = np.zeros(6)
        if bforce:
            force += y[n:4 * n].reshape(n, 3)
        if bstress:
            stress += y[-6:] * EV2GPA
        return energies, force, stress

    def LinearRegression(self, X, y, w, alpha, norm=2):
        """Weighted least squares with optional L2 / L1 term (:240-260), FP64 on the device."""
        dev = self.device
        X = torch.as_tensor(X, dtype=torch.float64, device=dev)
        y = torch.as_tensor(y, dtype=torch.float64, device=dev)
        sw = torch.sqrt(torch.as_tensor(w, dtype=torch.float64, device=dev))
        Xw, yw = X * sw[:, None], y * sw
        if alpha:
            if norm == 1:
                A, b = Xw.T @ Xw, Xw.T @ yw - alpha
            elif norm == 2:
                A, b = Xw.T @ Xw + alpha * torch.eye(X.shape[1], dtype=torch.float64, device=dev), Xw.T @ yw
            else:
                raise NotImplementedError(f"Regularization with {norm} norm is not implemented yet.")
        else:
            A, b = Xw, yw
        # minimum-norm least squares through the SVD, as numpy's lstsq (rank-deficient X
        # is common: a column block of an element absent from every structure is zero)
        theta = torch.linalg.pinv(A) @ b
        return theta.cpu().numpy()

    def save_weights_to_txt(self, des_info):
        from .lammps_export import write_pr
        write_pr(self.path, self.elements, self.coef_, self.d_max, des_info)
