"""The reference's ASE calculator for a trained NN potential, on the GPU path.

``PyXtalFFCalculator`` mirrors pyxtal_ff/calculator/__init__.py:14-73: for a
structure it computes the descriptors (``compute_descriptor``,
pyxtal_ff/utilities/__init__.py:255-321), evaluates the potential
(``NeuralNetworkPotential.calculate_properties``) and fills ``results`` with the
same keys -- energies, energy, free_energy, forces, stress, and the *_ml / *_zbl
parts -- with the stress in ASE's order and sign (style 'ase') or the
reference's own (GPa, xx yy zz xy xz yz).

Two routes:
- route='plain' (default, the reference's arithmetic): FP64 descriptors with dxdr
  and per-atom rdxdr from the CUDA plain path, contracted by so4_contract_dxdr;
- route='adjoint': B in FP32, dE/dB from the networks, forces and virial by the
  adjoint kernels (no dxdr), the path for MD-sized structures; repeated calls on one
  layout (an MD loop) replay the step as a single CUDA graph.

ASE is not a dependency: the class keeps ASE's calculator protocol
(``calculate(atoms, properties, system_changes)``, ``results``,
``get_potential_energy / get_forces / get_stress``) without subclassing it, and
takes any object with ``positions``, ``get_cell()``, ``pbc``, ``numbers`` and
``get_chemical_symbols()`` or ``symbols``.  The ZBL base potential of the reference
is not part of this path: ``base_potential`` must be empty.
"""
from __future__ import annotations

import numpy as np

from .nn import EV2GPA, NeuralNetworkPotential

# ASE's GPa in eV/A^3 (CODATA 2014, ASE's default): 1 / 160.21766208
ASE_GPA = 1.0 / 160.21766208


class ForceField:
    """The two attributes of the reference's PyXtal_FF object the calculator reads:
    the descriptor settings dict (``_descriptors``) and the model (``model``)."""

    def __init__(self, descriptors: dict, model: NeuralNetworkPotential):
        d = dict(descriptors)
        d.setdefault("base_potential", None)
        d.setdefault("cutoff", "cosine")
        self._descriptors = d
        self.model = model


def _descriptor_object(function, derivative=True, stress=True):
    from .descriptors.SNAP import SO4_Bispectrum as SNAP
    from .descriptors.SO4 import SO4_Bispectrum as SO4
    t = function["type"]
    p = function["parameters"]
    if t in ("SO4", "Bispectrum", "bispectrum"):
        return SO4(p["lmax"], function["Rc"], derivative=derivative, stress=stress,
                   normalize_U=p.get("normalize_U", False), cutoff_function=function["cutoff"])
    if t in ("SNAP", "snap"):
        return SNAP(function["weights"], p["lmax"], function["Rc"], derivative=derivative, stress=stress,
                    normalize_U=p.get("normalize_U", False), cutoff_function=function["cutoff"],
                    rfac0=p.get("rfac", 0.99363))
    raise NotImplementedError(f"{t} is not implemented")


def compute_descriptor(function, structure):
    """x, dxdr, seq, elements and per-atom Voigt rdxdr (N, nB, 6) of one structure, as
    the reference's compute_descriptor returns them (utilities/__init__.py:255-321)."""
    return _descriptor_object(function).calculate(structure, stress_per_atom=True)


def _symbols(atoms):
    if hasattr(atoms, "get_chemical_symbols"):
        return list(atoms.get_chemical_symbols())
    return list(atoms.symbols)


class PyXtalFFCalculator:
    implemented_properties = ["energy", "forces", "stress"]
    nolabel = True

    def __init__(self, style="ase", ff: ForceField | None = None, route="plain", **kwargs):
        if route not in ("plain", "adjoint"):
            raise ValueError("route must be 'plain' or 'adjoint'")
        self.style = style
        self.route = route
        self.parameters = {"ff": ff, **kwargs}
        self.results = {}
        self.atoms = None
        self._atoms_obj = None
        self._calc = None
        self._step, self._step_key, self._last_key = None, None, None

    def _ff(self):
        ff = self.parameters["ff"]
        if ff is None:
            raise ValueError("PyXtalFFCalculator needs ff=ForceField(descriptors, model)")
        if ff._descriptors.get("base_potential"):
            raise NotImplementedError("the ZBL base potential is not part of this path")
        return ff

    def _key(self, atoms):
        return (np.array(atoms.positions, dtype=np.float64).copy(), np.array(atoms.get_cell(), dtype=np.float64).copy(),
                np.array(atoms.numbers).copy())

    def _changed(self, atoms):
        if self.atoms is None or not self.results:
            return True
        return any(a.shape != b.shape or not np.array_equal(a, b) for a, b in zip(self._key(atoms), self.atoms))

    def _adjoint(self, atoms, ff):
        from .calculator import EV_A3_TO_GPA, Batch, SO4Calculator
        if ff.model.unit == "Ha":
            raise NotImplementedError("route='adjoint' supports unit 'eV'")
        f = ff._descriptors
        p = f["parameters"]
        if self._calc is None:
            kind = "SNAP" if f["type"] in ("SNAP", "snap") else "SO4"
            if f["type"] not in ("SNAP", "snap", "SO4", "Bispectrum", "bispectrum"):
                raise NotImplementedError(f"{f['type']} is not implemented")
            self._calc = SO4Calculator(lmax=p["lmax"], rcut=f["Rc"], kind=kind, weights=f.get("weights"),
                                       rfac0=p.get("rfac", 0.99363), cutoff_function=f["cutoff"],
                                       normalize_U=p.get("normalize_U", False))
        batch = Batch([atoms])
        # an MD or relaxation loop moves only the positions: from the second structure of one
        # layout (cell, pbc, species, model) on, the step is one CUDA-graph replay
        # (SO4Calculator.capture), bit for bit the uncaptured compute()
        key = (batch.cells.tobytes(), np.asarray(batch.pbc).tobytes(), np.asarray(atoms.numbers).tobytes(),
               id(ff.model), tuple(id(ff.model.models[e]) for e in ff.model.elements))
        if self._step is not None and self._step_key != key:
            self._step = None
        if self._step is None and self._last_key == key:
            self._step = self._calc.capture(batch, ff.model.energy_model(batch.species_order))
            self._step_key = key
        self._last_key = key
        r = None
        if self._step is not None:
            r = self._step(batch.positions)
            if not self._step.check():  # the neighbour list outgrew the captured buffers
                self._step, r = None, None
        if r is None:
            r = self._calc.compute(batch, ff.model.energy_model(batch.species_order))
        e_atom = r["energies"].double()
        symbols = np.asarray(_symbols(atoms))
        order = np.concatenate([np.nonzero(symbols == e)[0] for e in ff.model.elements])
        energies = e_atom.cpu().numpy()[order]
        forces = r["forces"].cpu().numpy()
        stress = r["stress"][0].cpu().numpy() / EV_A3_TO_GPA * EV2GPA
        return energies, forces, stress

    def calculate(self, atoms=None, properties=("energy",), system_changes=None):
        if atoms is None:
            atoms = self._atoms_obj
        self._atoms_obj = atoms
        ff = self._ff()
        if self.route == "plain":
            desp = compute_descriptor(ff._descriptors, atoms)
            energies, forces, stress = ff.model.calculate_properties(desp, bforce=True, bstress=True)
            self.desp = desp
        else:
            energies, forces, stress = self._adjoint(atoms, ff)
        n = len(atoms.positions)
        base_energy, base_forces, base_stress, base_energies = 0.0, np.zeros((n, 3)), np.zeros(6), 0.0
        self.results = {}
        self.results["energies"] = energies + base_energies
        self.results["energy"] = energies.sum() + base_energy
        self.results["free_energy"] = energies.sum() + base_energy
        self.results["forces"] = forces + base_forces
        self.results["stress_zbl"] = base_stress / ASE_GPA
        self.results["energy_zbl"] = base_energy
        self.results["forces_zbl"] = base_forces
        self.results["stress_ml"] = stress
        self.results["energy_ml"] = energies.sum()
        self.results["forces_ml"] = forces
        if self.style == "ase":
            # ASE: eV/A^3, tension negative, order xx yy zz yz xz xy
            self.results["stress"] = -(stress * ASE_GPA + base_stress)[[0, 1, 2, 5, 4, 3]]
        else:
            self.results["stress"] = self.results["stress_zbl"] + self.results["stress_ml"]
        self.atoms = self._key(atoms)

    def get_property(self, name, atoms=None):
        if atoms is not None and self._changed(atoms):
            self.calculate(atoms, [name])
        elif atoms is None and not self.results:
            self.calculate(None, [name])
        return self.results[name]

    def get_potential_energy(self, atoms=None, force_consistent=False):
        return self.get_property("free_energy" if force_consistent else "energy", atoms)

    def get_forces(self, atoms=None):
        return self.get_property("forces", atoms).copy()

    def get_stress(self, atoms=None):
        return self.get_property("stress", atoms).copy()

    def __str__(self):
        return "\nASE calculator with pyxtal_ff force field\n"

    def __repr__(self):
        return str(self)
