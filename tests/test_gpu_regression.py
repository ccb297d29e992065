"""The linear potential's design matrix on the GPU against the reference's own
PR.parse_descriptors / calculate_properties (tests/golden/pr_design.npz, made by
tests/golden/make_golden_pr.py from the descriptors in tests/golden/nn_*.npz)."""
import os

import numpy as np
import pytest

from pyxtal_ff_gb300.regression import PolynomialRegressionPotential
from tests import goldens as G

pytestmark = pytest.mark.gpu

PR = dict(np.load(os.path.join(G.GOLDEN, "pr_design.npz")))


def _desc(name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    return d, dict(x=d["x"], dxdr=d["dxdr"], seq=d["seq"], rdxdr=d["rdxdr_atom"], elements=list(atoms.symbols))


@pytest.mark.parametrize("name", G.nn_names())
def test_predict_design_matrix_and_properties(cuda_device, name):
    d, desc = _desc(name)
    key = name[3:]
    pot = PolynomialRegressionPotential(sorted(set(desc["elements"])), coef_=d["pr_coef"])
    X = pot.parse_descriptors({"0": desc}, fc=True, sc=True, train=False)
    ref = PR[key + "_X"]
    assert X.shape == ref.shape
    assert G.rel_err(X, ref) < 1e-14, G.rel_err(X, ref)
    e, f, s = pot.calculate_properties(desc, bforce=True, bstress=True)
    assert G.rel_err(e, PR[key + "_energies"]) < 1e-12
    assert G.rel_err(f, PR[key + "_forces"]) < 1e-12
    assert G.rel_err(s, PR[key + "_stress"]) < 1e-12


def test_training_design_matrix_two_structures(cuda_device):
    data = {}
    for i, (name, group) in enumerate((("nn_nacl_snap", "A"), ("nn_si16_snap", "B"))):
        _, desc = _desc(name)
        desc["group"] = group
        data[str(i)] = desc
    pot = PolynomialRegressionPotential(["Cl", "Na", "Si"], stress_group=["B"])
    X = pot.parse_descriptors(data, fc=True, sc=True, train=True)
    ref = PR["train_X"]
    assert X.shape == ref.shape
    assert G.rel_err(X, ref) < 1e-14, G.rel_err(X, ref)
    # forces only / energies only layouts
    Xe = pot.parse_descriptors(data, fc=False, sc=False, train=True)
    assert Xe.shape == (2, ref.shape[1])
    assert np.array_equal(Xe[0], ref[0]) and np.array_equal(Xe[1], ref[1 + 3 * 8])


def test_linear_regression_matches_numpy(cuda_device):
    rng = np.random.default_rng(3)
    X = PR["train_X"]
    theta = rng.normal(size=X.shape[1])
    y = X @ theta + 1e-3 * rng.normal(size=X.shape[0])
    w = rng.uniform(0.5, 2.0, size=X.shape[0])
    pot = PolynomialRegressionPotential(["Cl", "Na", "Si"])
    for alpha, norm in ((None, 2), (1e-3, 2), (1e-3, 1)):
        got = pot.LinearRegression(X, y, w, alpha, norm)
        Xw, yw = X * np.sqrt(w)[:, None], y * np.sqrt(w)
        if alpha is None:
            ref = np.linalg.lstsq(Xw, yw, rcond=None)[0]
        elif norm == 2:
            ref = np.linalg.lstsq(Xw.T @ Xw + alpha * np.eye(X.shape[1]), Xw.T @ yw, rcond=None)[0]
        else:
            ref = np.linalg.lstsq(Xw.T @ Xw, Xw.T @ yw - alpha, rcond=None)[0]
        # the fitted values agree (X is rank deficient: both are minimum-norm solutions)
        assert G.rel_err(X @ got, X @ ref) < 1e-8


@pytest.mark.parametrize("name", G.nn_names())
def test_quadratic_predict_design_matrix_and_properties(cuda_device, name):
    d, desc = _desc(name)
    key = "quad_" + name[3:]
    dmax = int(PR[key + "_dmax"])
    pot = PolynomialRegressionPotential(sorted(set(desc["elements"])), coef_=PR[key + "_coef"], order=2, d_max=dmax)
    X = pot.parse_descriptors({"0": desc}, fc=True, sc=True, train=False)
    ref = PR[key + "_X"]
    assert X.shape == ref.shape
    assert G.rel_err(X, ref) < 1e-13, G.rel_err(X, ref)
    e, f, s = pot.calculate_properties(desc, bforce=True, bstress=True)
    assert G.rel_err(e, PR[key + "_energies"]) < 1e-12
    assert G.rel_err(f, PR[key + "_forces"]) < 1e-12
    assert G.rel_err(s, PR[key + "_stress"]) < 1e-12


def test_quadratic_training_design_matrix(cuda_device):
    data = {}
    for i, (name, group) in enumerate((("nn_nacl_snap", "A"), ("nn_si16_snap", "B"))):
        _, desc = _desc(name)
        desc["group"] = group
        data[str(i)] = desc
    pot = PolynomialRegressionPotential(["Cl", "Na", "Si"], order=2, d_max=6, stress_group=["B"])
    X = pot.parse_descriptors(data, fc=True, sc=True, train=True)
    ref = PR["quad_train_X"]
    assert X.shape == ref.shape
    assert G.rel_err(X, ref) < 1e-13, G.rel_err(X, ref)

