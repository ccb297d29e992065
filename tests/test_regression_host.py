"""Host-side pieces of the linear potential (no GPU)."""
from pyxtal_ff_gb300.regression import PolynomialRegressionPotential


def test_feature_table_order():
    f = PolynomialRegressionPotential.features(3, True)
    assert f.tolist() == [[0, -1], [1, -1], [2, -1], [0, 0], [0, 1], [0, 2], [1, 1], [1, 2], [2, 2]]
    assert len(PolynomialRegressionPotential.features(55, True)) == (55 * 55 + 3 * 55) // 2
