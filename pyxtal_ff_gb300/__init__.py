"""pyxtal_ff_gb300 -- GB300-native SO(4)/SNAP bispectrum descriptor path.

Drop-in for PyXtal_FF's ``SO4_Bispectrum.calculate`` (pyxtal_ff/descriptors/SO4.py
and SNAP.py) with forces and stress, computed by hand-written sm_103a CUDA
kernels behind a C ABI (include/so4_gb300.h).  Importing the package creates no
CUDA context; the library is loaded on first use and the package fails loudly if
it is missing (there is no CPU fallback).
"""
__version__ = "0.1.0"
