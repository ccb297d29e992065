"""Drop-in descriptor classes: ``SO4.SO4_Bispectrum`` (pyxtal_ff/descriptors/SO4.py)
and ``SNAP.SO4_Bispectrum`` (pyxtal_ff/descriptors/SNAP.py)."""
