"""The oracle is pinned against golden vectors produced by the reference itself."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import goldens as G

CASES = G.names()


def test_factorials_match_reference_table():
    ref = G.tables()["factorial"]
    ours = np.array([O.factorial(n) for n in range(len(ref))])
    n_ok = 34  # the oracle tabulates up to 34!, beyond any supported twol (<= 20)
    assert np.array_equal(ours[:n_ok], ref[:n_ok])


@pytest.mark.parametrize("twol", range(0, 11))
def test_clebsch_gordan_matches_reference(twol):
    ref = G.tables()["cglist_%d" % twol]
    ours = O.tables(twol)["cglist"]
    assert ours.shape == ref.shape
    np.testing.assert_array_max_ulp(ours, ref, maxulp=1)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    atoms, meta, d = G.load(name)
    out = O.descriptor(atoms, **G.descriptor_kwargs(meta))
    errs = G.compare_to_golden(out, d, tol=1e-12)
    assert out["elements"] == list(atoms.symbols)
    if not meta["derivative"]:
        assert out["dxdr"] is None and "seq" not in out
    if not meta["stress"]:
        assert out["rdxdr"] is None
    print(name, errs)


def test_sizes_match_reference_loop_counts():
    # idxu / idxz / idxcg / nB for lmax 3 and 4, counted from the reference's loops
    assert O.sizes(6) == dict(idxu=140, idxz=779, idxcg=1321, nB=30, idxu_half=78)
    assert O.sizes(8) == dict(idxu=285, idxz=2386, idxcg=4098, nB=55, idxu_half=155)
