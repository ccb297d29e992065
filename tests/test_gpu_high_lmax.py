"""The drop-in's FP64 path at the top of the compiled range, against the oracle.

At lmax 6 (twol 12) the FP64 plain kernel's Z (12,936 entries, 207 KB) does not fit in
shared memory beside the per-warp buffers, so it lives in one global slot per CTA of a
grid of min(natoms, 2 x SMs) CTAs that take the centres in turn.  lmax 5 keeps Z in
shared memory.  Both at 1e-10 relative on x, dxdr and rdxdr, SO4 and SNAP, on a cell
with more centres than the grid has CTAs (so CTAs reuse their slot).  lmax above 6
(twol 14 up to the reference's 64) is not compiled: the constructor accepts it, as the
reference's does, and calculate() raises NotImplementedError.
"""
import numpy as np
import pytest

from oracle import oracle as O
from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.descriptors.SNAP import SO4_Bispectrum as SNAP
from pyxtal_ff_gb300.descriptors.SO4 import SO4_Bispectrum as SO4
from tests import goldens as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lmax", [5, 6])
def test_fp64_dropin_at_lmax_5_and_6_matches_the_oracle(cuda_device, lmax):
    si = S.diamond_si(1, 1, 1, sigma=0.08, rng=np.random.default_rng(51))
    out = SO4(lmax=lmax, rcut=3.2, derivative=True, stress=True).calculate(si)
    ref = O.descriptor(si, kind="SO4", lmax=lmax, rcut=3.2, derivative=True, stress=True)
    assert np.array_equal(out["seq"], ref["seq"])
    for key in ("x", "dxdr", "rdxdr"):
        assert G.rel_err(out[key], ref[key]) < 1e-10, key


def test_fp64_dropin_at_lmax_6_reuses_global_z_slots(cuda_device):
    # 7 x 7 x 7 cells: 2,744 centres, more than a GB300's 2 x 152 CTAs of the global-Z grid
    si = S.diamond_si(7, 7, 7, sigma=0.05, rng=np.random.default_rng(52))
    out = SNAP({"Si": 0.9}, lmax=6, rcut=2.6, derivative=True, stress=True, rfac0=0.99363).calculate(si)
    ref = O.descriptor(si, kind="SNAP", lmax=6, rcut=2.6, weights={"Si": 0.9}, rfac0=0.99363, derivative=True,
                       stress=True)
    assert np.array_equal(out["seq"], ref["seq"])
    for key in ("x", "dxdr", "rdxdr"):
        assert G.rel_err(out[key], ref[key]) < 1e-10, key


def test_lmax_above_the_compiled_range_raises_not_implemented(cuda_device):
    si = S.diamond_si(1, 1, 1, sigma=0.05, rng=np.random.default_rng(53))
    with pytest.raises(NotImplementedError):
        SO4(lmax=7, rcut=3.0).calculate(si)
