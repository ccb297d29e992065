"""Host-side behaviour of the drop-in classes that needs no GPU: parameter
validation, exception types and the save/load dict (SO4.py:40-158, SNAP.py:50-187)."""
import pytest

from pyxtal_ff_gb300.descriptors.SNAP import SO4_Bispectrum as SNAP
from pyxtal_ff_gb300.descriptors.SO4 import SO4_Bispectrum as SO4


def test_so4_validation_mirrors_reference():
    with pytest.raises(ValueError):
        SO4(lmax=-1)
    with pytest.raises(ValueError):
        SO4(lmax=2.5)
    with pytest.raises(NotImplementedError):
        SO4(lmax=33)
    with pytest.raises(ValueError):
        SO4(rcut=0)
    with pytest.raises(ValueError):
        SO4(rcut="4")
    with pytest.raises(ValueError):
        SO4(derivative=1)
    with pytest.raises(ValueError):
        SO4(stress="yes")
    with pytest.raises(ValueError):
        SO4(normalize_U=0)
    with pytest.raises(NotImplementedError):
        SO4(cutoff_function="gauss")
    with pytest.raises(ValueError):
        SO4(cutoff_function=3)


def test_snap_validation_mirrors_reference():
    with pytest.raises(TypeError):
        SNAP(["Si"])
    with pytest.raises(ValueError):
        SNAP({"Si": 1.0}, rfac0=0)
    with pytest.raises(ValueError):
        SNAP({"Si": 1.0}, rfac0=1.5)
    with pytest.raises(ValueError):
        SNAP({"Si": 1.0}, rfac0="x")
    s = SNAP({"Si": 1.0}, lmax=1.5)
    assert s._twol == 3 and s.lmax == 1


def test_save_load_roundtrip():
    a = SO4(lmax=3, rcut=4.9, derivative=True, stress=True, normalize_U=True, cutoff_function="poly2")
    d = a.save_dict()
    assert d == {"lmax": 3, "rcut": 4.9, "normalize_U": True, "cutoff_function": "poly2",
                 "derivative": True, "stress": True, "_type": "SO4"}
    b = SO4()
    b.load_from_dict(d)
    assert b.save_dict() == d
    s = SNAP({"Si": 1.0, "O": 0.5}, lmax=4, rcut=5.0, stress=True)
    assert "weights" not in s.save_dict() and s.save_dict()["_type"] == "SO4"
    assert str(a).startswith("SO4 bispectrum descriptor with Cutoff:  4.900 lmax: 3")


def test_clear_memory_keeps_parameters():
    a = SO4(lmax=2, rcut=3.0)
    a.scratch = 1
    a.clear_memory()
    assert not hasattr(a, "scratch") and a.lmax == 2 and a.rcut == 3.0
