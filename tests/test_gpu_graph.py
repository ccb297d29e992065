"""CUDA-graph captured step (SO4Calculator.capture) against the eager public API.

The graph runs the same kernels on the same data, with the image count taken on
the device instead of from a host read, so its outputs must equal the eager
path's bit for bit; replays with new positions must track the eager path; a
neighbour list that outgrows the captured capacity must be reported by check().
"""
import numpy as np
import pytest
import torch

from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.calculator import Batch, LinearModel, SO4Calculator

pytestmark = pytest.mark.gpu


def _setup(structs, lmax=3, rc=4.5):
    batch = Batch(structs)
    calc = SO4Calculator(lmax=lmax, rcut=rc, kind="SNAP", weights={"Si": 1.0, "O": 0.7}, rfac0=0.99363)
    nB = calc.nB
    rng = np.random.default_rng(3)
    model = LinearModel(rng.normal(0, 0.01, size=(len(batch.species_order), nB)),
                        bias=rng.normal(0, 1.0, size=len(batch.species_order))).cuda()
    return batch, calc, model


def _equal(res, ref):
    for k in ("energy", "forces", "virial", "stress", "x"):
        assert torch.equal(res[k], ref[k]), k


def test_graph_step_matches_eager_bitwise(cuda_device):
    structs = [S.diamond_si(2, 2, 2, sigma=0.1, rng=np.random.default_rng(1)), S.sio2_random(n_si=8, seed=2),
               S.diamond_si(1, 1, 1, sigma=0.05, rng=np.random.default_rng(4))]
    batch, calc, model = _setup(structs)
    step = calc.capture(batch, model)
    assert step.launches > 0
    res = {k: v.clone() for k, v in step().items()}
    assert step.check()
    _equal(res, calc.compute(batch, model))
    # new positions from the host (pinned) and from the device
    rng = np.random.default_rng(9)
    for it in range(3):
        pos = batch.positions + rng.normal(0, 0.02, size=batch.positions.shape)
        src = torch.from_numpy(pos).pin_memory() if it % 2 == 0 else torch.from_numpy(pos).cuda()
        res = {k: v.clone() for k, v in step(src).items()}
        torch.cuda.synchronize()
        assert step.check()
        _equal(res, calc.compute(batch, model, positions=pos))


def test_graph_step_general_model_matches_eager_bitwise(cuda_device):
    """An NN potential (two species, per-species networks) captured with its gradient dE/dB:
    every output equals the uncaptured compute(), also after the same calculator prepared
    another batch (the graph holds its per-batch tensors)."""
    from pyxtal_ff_gb300.nn import NeuralNetworkPotential
    structs = [S.diamond_si(2, 2, 2, sigma=0.1, rng=np.random.default_rng(1)), S.sio2_random(n_si=8, seed=2)]
    batch, calc, _ = _setup(structs)
    nB = calc.nB
    torch.manual_seed(5)
    nets = {e: torch.nn.Sequential(torch.nn.Linear(nB, 8), torch.nn.Tanh(), torch.nn.Linear(8, 1)).double()
            for e in batch.species_order}
    drange = {e: np.stack([np.zeros(nB), np.full(nB, 2.0)], 1) for e in nets}
    pot = NeuralNetworkPotential(nets, drange)
    model = pot.energy_model(batch.species_order)
    step = calc.capture(batch, model)
    keys = ("energy", "forces", "virial", "stress", "x", "energies")
    res = {k: v.clone() for k, v in step().items()}
    assert step.check()
    ref = calc.compute(batch, model)
    for k in keys:
        assert torch.equal(res[k], ref[k]), k
    rng = np.random.default_rng(11)
    for _ in range(2):
        pos = batch.positions + rng.normal(0, 0.02, size=batch.positions.shape)
        res = {k: v.clone() for k, v in step(pos).items()}
        assert step.check()
        ref = calc.compute(batch, model, positions=pos)
        for k in keys:
            assert torch.equal(res[k], ref[k]), k
    other = Batch([S.diamond_si(1, 1, 2, sigma=0.05, rng=np.random.default_rng(6))])
    calc.compute(other, pot.energy_model(other.species_order))
    res = {k: v.clone() for k, v in step(pos).items()}
    for k in keys:
        assert torch.equal(res[k], ref[k]), k


def test_graph_step_reports_overflow_and_bad_input(cuda_device):
    structs = [S.diamond_si(2, 2, 2, sigma=0.05, rng=np.random.default_rng(5))]
    batch, calc, model = _setup(structs)
    step = calc.capture(batch, model, headroom=1.0)
    step()
    assert step.check()
    # squeeze every atom towards one corner: many more neighbours than captured
    pos = batch.positions * 0.6
    step(pos)
    assert not step.check()
    bad = batch.positions.copy()
    bad[3, 1] = np.nan
    step(bad)
    with pytest.raises(ValueError):
        step.check()


def test_two_branch_graph_matches_eager_bitwise(cuda_device):
    # 280 atoms: the two halves split the first structure at atom 160
    structs = [S.diamond_si(3, 3, 3, sigma=0.08, rng=np.random.default_rng(11)),
               S.diamond_si(2, 2, 2, sigma=0.08, rng=np.random.default_rng(12))]
    batch, calc, model = _setup(structs)
    step = calc.capture(batch, model, branches=2)
    assert step.branches == 2
    one = calc.capture(batch, model, branches=1)
    rng = np.random.default_rng(13)
    for _ in range(2):
        pos = batch.positions + rng.normal(0, 0.02, size=batch.positions.shape)
        res = {k: v.clone() for k, v in step(pos).items()}
        res1 = {k: v.clone() for k, v in one(pos).items()}
        torch.cuda.synchronize()
        assert step.check() and one.check()
        _equal(res, calc.compute(batch, model, positions=pos))
        _equal(res, res1)


def test_host_io_graph_copies_in_and_out(cuda_device):
    # host_io: the graph copies the positions in from its pinned buffer and energy, forces,
    # stress out; the host results equal the device step's bit for bit, for the linear
    # two-branch step and for a general model on one stream
    structs = [S.diamond_si(3, 3, 3, sigma=0.08, rng=np.random.default_rng(21)),
               S.diamond_si(2, 2, 2, sigma=0.08, rng=np.random.default_rng(22))]
    batch, calc, model = _setup(structs)
    dev_step = calc.capture(batch, model, branches=2)
    io_step = calc.capture(batch, model, branches=2, host_io=True)
    assert io_step.host_positions.is_pinned() and all(v.is_pinned() for v in io_step.host_out.values())
    rng = np.random.default_rng(23)
    for _ in range(2):
        pos = batch.positions + rng.normal(0, 0.02, size=batch.positions.shape)
        io_step.host_positions.copy_(torch.from_numpy(pos))
        out = {k: v.clone() for k, v in io_step().items()}
        ref = {k: v.clone() for k, v in dev_step(pos).items()}
        torch.cuda.synchronize()
        assert io_step.check()
        for k in ("energy", "forces", "stress"):
            assert torch.equal(out[k], ref[k].cpu()), k
    mlp = torch.nn.Sequential(torch.nn.Linear(calc.nB, 8), torch.nn.Tanh(), torch.nn.Linear(8, 1)).cuda()

    class PerAtom(torch.nn.Module):
        def __init__(self, net):
            super().__init__()
            self.net = net

        def forward(self, x, species):
            return self.net(x).squeeze(-1)

    gm = PerAtom(mlp)
    g_io = calc.capture(batch, gm, host_io=True)
    g_dev = calc.capture(batch, gm)
    pos = batch.positions + rng.normal(0, 0.02, size=batch.positions.shape)
    out = {k: v.clone() for k, v in g_io(pos).items()}
    ref = g_dev(pos)
    torch.cuda.synchronize()
    for k in ("energy", "forces", "stress"):
        assert torch.equal(out[k], ref[k].cpu()), k


def test_two_branch_graph_reports_overflow(cuda_device):
    # per-branch neighbour lists: an overflow in either range empties the ranges on the
    # device, so the step reads nothing out of bounds and check() reports it
    structs = [S.diamond_si(4, 4, 2, sigma=0.05, rng=np.random.default_rng(31))]  # 256 atoms: two branches
    batch, calc, model = _setup(structs)
    step = calc.capture(batch, model, headroom=1.0, branches=2)
    assert step.branches == 2
    step()
    assert step.check()
    ref = {k: v.clone() for k, v in step().items()}
    pos = batch.positions.copy()
    pos[:100] *= 0.6  # the first range gets far more neighbours than captured
    step(pos)
    assert not step.check()
    pos = batch.positions.copy()
    pos[150:] *= 0.6  # now the second
    step(pos)
    assert not step.check()
    res = {k: v.clone() for k, v in step(batch.positions).items()}  # and back
    torch.cuda.synchronize()
    assert step.check()
    _equal(res, ref)


def test_lite_and_one_pass_neighbor_lists_match_full(cuda_device):
    from pyxtal_ff_gb300 import engine
    structs = [S.diamond_si(2, 2, 2, sigma=0.1, rng=np.random.default_rng(21)), S.sio2_random(n_si=8, seed=22)]
    batch = Batch(structs)
    pos = torch.from_numpy(batch.positions).cuda()
    full = engine.build_neighbors(pos, batch.cells, batch.pbc, batch.atom_ptr, 4.5)
    lay = engine.layout(batch.cells, batch.pbc, batch.atom_ptr, 4.5)
    counts = int(torch.diff(full.img_ptr).max())
    bufs = engine.NeighborBuffers.allocate(lay, full.nimg + 64, full.npair + 64, "cuda", slot_cap=counts + 8)
    engine.enqueue_neighbors(lay, pos, bufs, lite=True)
    M, P, bits = [int(v) for v in bufs.summary_dev().cpu()]
    assert M == full.nimg and P == full.npair and engine.check_summary(M, P, bits, bufs.cap_m, bufs.cap_p)
    for a, b in ((bufs.img_ptr, full.img_ptr), (bufs.img_j[:M], full.img_j), (bufs.img_off[:M], full.img_off),
                 (bufs.img_r[:M], full.img_r), (bufs.img_rev[:M], full.img_rev)):
        assert torch.equal(a, b)
    assert int(bufs.max_count_dev().cpu()[0]) == counts
