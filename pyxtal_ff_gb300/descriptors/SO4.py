"""Drop-in for pyxtal_ff.descriptors.SO4.SO4_Bispectrum (pyxtal_ff/descriptors/SO4.py:10-304).

Neighbour weight and site weight are the atomic numbers (SO4.py:244, 271);
psi = pi r / rcut (SO4.py:1443).
"""
from ._base import BispectrumBase


class SO4_Bispectrum(BispectrumBase):
    """SO(4) bispectrum B, dB/dr and per-pair virial on the GPU (CUDA, FP64)."""

    def __init__(self, lmax=3, rcut=3.5, derivative=True, stress=False, normalize_U=False, cutoff_function="cosine"):
        self.lmax = lmax
        self.rcut = rcut
        self.derivative = derivative
        self.stress = stress
        self.normalize_U = normalize_U
        self.cutoff_function = cutoff_function
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
        return {"lmax": self.lmax, "rcut": self.rcut, "normalize_U": self.normalize_U,
                "cutoff_function": self.cutoff_function, "derivative": self.derivative,
                "stress": self.stress, "_type": "SO4"}

    @property
    def lmax(self):
        return self._twol // 2

    @lmax.setter
    def lmax(self, lmax):
        if isinstance(lmax, int) is True:
            if lmax < 0:
                raise ValueError("lmax must be greater than or equal to zero")
            elif lmax > 32:
                raise NotImplementedError("Currently we only support Wigner-D matrices and spherical harmonics "
                                          "for arguments up to l=32.")
            self._twol = 2 * lmax
        else:
            raise ValueError("lmax must be an integer")

    def _weights(self, numbers, symbols):
        from ..engine import site_weights
        return site_weights("SO4", numbers, symbols)
