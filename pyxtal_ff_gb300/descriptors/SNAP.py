"""Drop-in for pyxtal_ff.descriptors.SNAP.SO4_Bispectrum (pyxtal_ff/descriptors/SNAP.py).

Neighbour weight weights[symbol] (SNAP.py:273), site weight 1 (SNAP.py:299-301),
psi = rfac0 pi r / rcut (SNAP.py:1473).
"""
from ._base import BispectrumBase


class SO4_Bispectrum(BispectrumBase):
    """SNAP-weighted SO(4) bispectrum B, dB/dr and per-pair virial on the GPU (CUDA, FP64)."""

    _essential = BispectrumBase._essential | {"_weights_", "_rfac0_"}

    def __init__(self, weights, lmax=3, rcut=3.5, derivative=True, stress=False, normalize_U=False,
                 cutoff_function="cosine", rfac0=0.99363):
        self.weights = weights
        self.lmax = lmax
        self.rcut = rcut
        self.derivative = derivative
        self.stress = stress
        self.normalize_U = normalize_U
        self.cutoff_function = cutoff_function
        self.rfac0 = rfac0
        self._type = "SO4"

    def __str__(self):
        s = "SO4 bispectrum descriptor with Cutoff: {:6.3f}".format(self.rcut)
        s += " lmax: {:d}\n".format(self.lmax)
        return s

    def load_from_dict(self, dict0):
        self.lmax = dict0["lmax"]
        self.rcut = dict0["rcut"]
        self.normalize_U = dict0["normalize_U"]
        self.cutoff_function = dict0["cutoff_function"]
        self.derivative = dict0["derivative"]
        self.stress = dict0["stress"]

    def save_dict(self):
        # the reference's SNAP save_dict omits weights and rfac0 (SNAP.py:50-64)
        return {"lmax": self.lmax, "rcut": self.rcut, "normalize_U": self.normalize_U,
                "cutoff_function": self.cutoff_function, "derivative": self.derivative,
                "stress": self.stress, "_type": "SO4"}

    @property
    def weights(self):
        return self._weights_

    @weights.setter
    def weights(self, w):
        if isinstance(w, dict) is True:
            self._weights_ = w
        else:
            raise TypeError("weights must be a dictionary")

    @property
    def lmax(self):
        return self._twol // 2

    @lmax.setter
    def lmax(self, lmax):
        if isinstance(lmax, int) is True or isinstance(lmax, float) is True:
            if lmax < 0:
                raise ValueError("lmax must be greater than or equal to zero")
            elif lmax > 32:
                raise NotImplementedError("Currently we only support Wigner-D matrices and spherical harmonics "
                                          "for arguments up to l=32.")
            self._twol = round(2 * lmax)
        else:
            raise ValueError("lmax must be an integer")

    @property
    def rfac0(self):
        return self._rfac0_

    @rfac0.setter
    def rfac0(self, rfac0):
        if isinstance(rfac0, float) is True or isinstance(rfac0, int) is True:
            if rfac0 <= 0:
                raise ValueError("rfac0 must be greater than zero")
            elif rfac0 > 1:
                raise ValueError("rfac0 must be less than or equal to one")
            self._rfac0_ = rfac0
        else:
            raise ValueError("rfac0 must be a float")

    def _rfac0(self):
        return float(self._rfac0_)

    def _weights(self, numbers, symbols):
        from ..engine import site_weights
        return site_weights("SNAP", numbers, symbols, self._weights_)

    def calculate(self, atoms, atom_ids=None, *, stress_per_atom=False):
        if self._twol % 2:
            # the reference sizes its blist from lmax = twol // 2 (SNAP.py:329) and then
            # overruns it for an odd twol; no valid output exists to match
            raise NotImplementedError("half-integer lmax (odd 2*lmax) is not supported")
        return super().calculate(atoms, atom_ids, stress_per_atom=stress_per_atom)
