"""Host logic of the ASE calculator's adjoint route (pyxtal_ff_gb300/ase_calculator.py):
when it computes eagerly, when it captures the step as a CUDA graph and replays it, and
when it drops the graph.  Runs on the CPU against a stand-in for SO4Calculator that
records which of compute / capture / replay ran; the numbers themselves are checked on
the GPU (tests/test_gpu_nn.py)."""
import numpy as np
import torch

from pyxtal_ff_gb300 import structures as S
from pyxtal_ff_gb300.ase_calculator import ForceField, PyXtalFFCalculator
from pyxtal_ff_gb300.nn import NeuralNetworkPotential


def _result(n):
    return {"energies": torch.zeros(n, dtype=torch.float64), "forces": torch.zeros((n, 3), dtype=torch.float64),
            "stress": torch.zeros((1, 6), dtype=torch.float64)}


class _Step:
    def __init__(self, log, n):
        self.log, self.n, self.ok = log, n, True

    def __call__(self, positions):
        self.log.append("replay")
        return _result(self.n)

    def check(self):
        return self.ok


class _FakeCalc:
    """Records the calls the calculator makes; capture() returns a replayable step."""

    def __init__(self):
        self.log = []
        self.steps = []

    def compute(self, batch, model):
        self.log.append("compute")
        return _result(len(batch.positions))

    def capture(self, batch, model):
        self.log.append("capture")
        st = _Step(self.log, len(batch.positions))
        self.steps.append(st)
        return st


def _calculator():
    nB = 14
    nets = {"Si": torch.nn.Sequential(torch.nn.Linear(nB, 4), torch.nn.Tanh(), torch.nn.Linear(4, 1)).double()}
    pot = NeuralNetworkPotential(nets, {"Si": np.stack([np.zeros(nB), np.ones(nB)], 1)}, device="cpu")
    desc = {"type": "SNAP", "Rc": 4.0, "cutoff": "cosine", "weights": {"Si": 1.0}, "base_potential": None,
            "parameters": {"lmax": 2}}
    calc = PyXtalFFCalculator(ff=ForceField(desc, pot), route="adjoint")
    calc._calc = _FakeCalc()
    return calc


def test_md_loop_captures_on_second_step_then_replays():
    calc = _calculator()
    fake = calc._calc
    atoms = S.diamond_si(1, 1, 1, sigma=0.05, rng=np.random.default_rng(1))
    base = atoms.positions.copy()
    rng = np.random.default_rng(2)
    for _ in range(4):
        atoms.positions = base + rng.normal(0, 0.01, size=base.shape)
        calc.calculate(atoms)
    # first structure eagerly, the second captures and replays, the rest replay
    assert fake.log == ["compute", "capture", "replay", "replay", "replay"]
    assert calc.results["forces"].shape == (len(base), 3)


def test_overflow_falls_back_and_recaptures():
    calc = _calculator()
    fake = calc._calc
    atoms = S.diamond_si(1, 1, 1, sigma=0.05, rng=np.random.default_rng(3))
    calc.calculate(atoms)
    calc.calculate(atoms)
    fake.steps[-1].ok = False  # the next replay reports a neighbour list beyond the capture
    calc.calculate(atoms)
    assert calc._step is None
    calc.calculate(atoms)
    assert fake.log == ["compute", "capture", "replay", "replay", "compute", "capture", "replay"]


def test_new_layout_or_model_drops_the_graph():
    calc = _calculator()
    fake = calc._calc
    a = S.diamond_si(1, 1, 1, sigma=0.05, rng=np.random.default_rng(4))
    calc.calculate(a)
    calc.calculate(a)
    assert calc._step is not None
    # another cell: eager again, and the old graph is not replayed for it
    b = S.diamond_si(1, 1, 1, a=5.5, sigma=0.05, rng=np.random.default_rng(5))
    calc.calculate(b)
    assert fake.log[-1] == "compute" and calc._step is None
    # back on one layout: capture from its second structure on
    calc.calculate(b)
    assert fake.log[-2:] == ["capture", "replay"]
    # a network replaced in the potential: the captured graph no longer applies
    nB = 14
    calc.parameters["ff"].model.models["Si"] = torch.nn.Sequential(torch.nn.Linear(nB, 1)).double()
    calc.calculate(b)
    assert fake.log[-1] == "compute" and calc._step is None


def test_species_networks_precomputed_index_matches():
    """The NN potential's networks with their species index lists supplied (the capturable
    form) give the same per-atom energies as with the lists found by the forward itself."""
    nB = 6
    torch.manual_seed(0)
    nets = {e: torch.nn.Sequential(torch.nn.Linear(nB, 3), torch.nn.Tanh(), torch.nn.Linear(3, 1)).double()
            for e in ("O", "Si")}
    drange = {e: np.stack([np.zeros(nB), np.full(nB, 2.0)], 1) for e in nets}
    pot = NeuralNetworkPotential(nets, drange, device="cpu")
    model = pot.energy_model(["O", "Si"])
    species = torch.tensor([1, 0, 1, 1, 0, 1], dtype=torch.int64)  # interleaved elements
    x = torch.rand((6, nB), dtype=torch.float32)
    e0 = model(x, species)
    e1 = model(x, species, model.species_index(species))
    assert torch.equal(e0, e1)
    assert e0.dtype == torch.float64 and e0.shape == (6,)
