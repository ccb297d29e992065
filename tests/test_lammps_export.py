"""LAMMPS ML-IAP export files byte-for-byte against the ones the reference writes
(NeuralNetwork.save_weights_to_txt and PR.save_weights_to_txt, captured in
tests/golden/nn_*.npz by tests/golden/make_golden_nn.py)."""
import json

import numpy as np
import pytest

from pyxtal_ff_gb300 import lammps_export as LX
from pyxtal_ff_gb300.nn import NeuralNetworkPotential
from tests import goldens as G


@pytest.mark.parametrize("name", G.nn_names())
def test_nn_export_matches_reference(tmp_path, name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    des_info = json.loads(str(d["des_info"]))
    pot = NeuralNetworkPotential(nets, drange, device="cpu", path=str(tmp_path) + "/")
    pot.save_weights_to_txt(des_info)
    assert (tmp_path / "NN_weights.txt").read_text() == str(d["nn_weights_txt"])
    assert (tmp_path / "DescriptorParam.txt").read_text() == str(d["descriptor_param_txt"])


@pytest.mark.parametrize("name", G.nn_names())
def test_linear_export_matches_reference(tmp_path, name):
    atoms, meta, d, nets, drange = G.load_nn(name)
    des_info = json.loads(str(d["des_info"]))
    elements = sorted(nets)
    LX.write_pr(str(tmp_path) + "/", elements, d["pr_coef"], d["x"].shape[1], des_info)
    assert (tmp_path / "PR_weights.txt").read_text() == str(d["pr_weights_txt"])
    assert (tmp_path / "DescriptorParam.txt").read_text() == str(d["pr_descriptor_param_txt"])


def test_network_layout_reads_the_reference_layer_layout():
    atoms, meta, d, nets, drange = G.load_nn("nn_nacl_snap")
    widths, acts, params = LX.network_layout(nets["Cl"])
    assert widths == [6, 5, 1] and acts == ["Tanh", "Sigmoid", "Linear"]
    assert [w.shape for w, _ in params] == [(6, 14), (5, 6), (1, 5)]
    assert np.array_equal(params[0][0], d["w_Cl_0.weight"])
