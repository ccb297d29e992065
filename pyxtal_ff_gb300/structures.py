"""Structure container and the seeded synthetic workloads.

``Atoms`` is the subset of the ASE ``Atoms`` interface that the reference's
descriptor reads (``pyxtal_ff/descriptors/SO4.py:171-287``): ``positions``,
``numbers``, ``symbols``, ``get_cell()``, ``get_volume()``, ``pbc``,
``len()`` and ``atoms[j].number / .symbol``.  A real ``ase.Atoms`` works
everywhere an ``Atoms`` is accepted; this class exists because ASE is not a
dependency of this package.

The generators build the workloads the path is measured on, from
``numpy.random.default_rng(seed)``:

* ``diamond_si``          diamond-Si supercell of the 8-atom cubic cell, optional
                          symmetric strain and Gaussian displacement;
* ``si_batch``            many diamond-Si supercells with random n1 x n2 x n3;
* ``sio2_random``         SiO2 at a given density, uniform positions with
                          rejection to a minimum pair distance;
* ``nacl_cluster``        the 8-atom NaCl rock-salt cluster of the reference's
                          tests (``pyxtal_ff/test_all.py:23-42``) re-boxed in a
                          17.22 A periodic cube and rotated about x.
"""
from __future__ import annotations

import numpy as np

_SYMBOLS = (
    "X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn "
    "Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr "
    "Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn"
).split()
ATOMIC_NUMBERS = {s: z for z, s in enumerate(_SYMBOLS) if z > 0}
CHEMICAL_SYMBOLS = _SYMBOLS
ATOMIC_MASSES = {"H": 1.008, "O": 15.999, "Na": 22.990, "Si": 28.0855, "Cl": 35.45}

DIAMOND_BASIS = np.array([
    [0.00, 0.00, 0.00], [0.00, 0.50, 0.50], [0.50, 0.00, 0.50], [0.50, 0.50, 0.00],
    [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25],
])


class _Atom:
    __slots__ = ("number", "symbol")

    def __init__(self, number: int):
        self.number = int(number)
        self.symbol = CHEMICAL_SYMBOLS[self.number]


class Atoms:
    """Minimal periodic structure: positions (N,3) in A, cell rows a1,a2,a3 (3,3)."""

    def __init__(self, numbers, positions, cell, pbc=True):
        if isinstance(numbers, str):
            raise TypeError("numbers must be a sequence of atomic numbers or symbols")
        nums = [ATOMIC_NUMBERS[s] if isinstance(s, str) else int(s) for s in numbers]
        self.numbers = np.asarray(nums, dtype=np.int64)
        self.positions = np.array(positions, dtype=np.float64).reshape(-1, 3)
        if len(self.positions) != len(self.numbers):
            raise ValueError("numbers and positions differ in length")
        self.cell = np.array(cell, dtype=np.float64).reshape(3, 3)
        p = np.broadcast_to(np.asarray(pbc, dtype=bool), (3,))
        self.pbc = np.array(p, dtype=bool)

    def __len__(self):
        return len(self.numbers)

    def __getitem__(self, j):
        return _Atom(self.numbers[j])

    @property
    def symbols(self):
        return [CHEMICAL_SYMBOLS[z] for z in self.numbers]

    def get_chemical_symbols(self):
        return self.symbols

    def get_cell(self):
        return self.cell.copy()

    def get_volume(self):
        return abs(float(np.linalg.det(self.cell)))

    def get_positions(self):
        return self.positions.copy()

    def get_pbc(self):
        return self.pbc.copy()

    def copy(self):
        return Atoms(self.numbers.copy(), self.positions.copy(), self.cell.copy(), self.pbc.copy())


def as_arrays(atoms):
    """(positions, cell, pbc, numbers, symbols) from an Atoms or an ase.Atoms."""
    pos = np.ascontiguousarray(np.asarray(atoms.positions, dtype=np.float64))
    cell = np.ascontiguousarray(np.asarray(atoms.get_cell(), dtype=np.float64).reshape(3, 3))
    pbc = getattr(atoms, "pbc", True)
    if callable(getattr(atoms, "get_pbc", None)):
        pbc = atoms.get_pbc()
    pbc = np.array(np.broadcast_to(np.asarray(pbc, dtype=bool), (3,)), dtype=np.int32)
    numbers = np.asarray(atoms.numbers, dtype=np.int64)
    symbols = [str(s) for s in list(atoms.symbols)]
    return pos, cell, pbc, numbers, symbols


def _strain_matrix(rng, amp):
    e = rng.uniform(-amp, amp, size=(3, 3))
    e = 0.5 * (e + e.T)
    return np.eye(3) + e


def diamond_si(n1, n2, n3, a=5.43, sigma=0.0, strain=0.0, rng=None):
    """Diamond-Si supercell of n1 x n2 x n3 cubic 8-atom cells."""
    rng = np.random.default_rng(0) if rng is None else rng
    grid = np.array([[i, j, k] for i in range(n1) for j in range(n2) for k in range(n3)], dtype=np.float64)
    frac = (grid[:, None, :] + DIAMOND_BASIS[None, :, :]).reshape(-1, 3) / np.array([n1, n2, n3], dtype=np.float64)
    cell = a * np.diag([n1, n2, n3]).astype(np.float64)
    if strain:
        cell = cell @ _strain_matrix(rng, strain)
    pos = frac @ cell
    if sigma:
        pos = pos + rng.normal(0.0, sigma, size=pos.shape)
    return Atoms([14] * len(pos), pos, cell, pbc=True)


def si_batch(n_struct, seed, sizes=(1, 2, 3), max_cells=None, strain=0.03, sigma=0.08, a=5.43):
    """n_struct diamond-Si supercells, each n_i drawn uniformly from `sizes`
    (rejected while n1*n2*n3 exceeds `max_cells`), random symmetric strain
    U(-strain, strain) and Gaussian displacement sigma."""
    rng = np.random.default_rng(seed)
    out = []
    sizes = np.asarray(sizes)
    while len(out) < n_struct:
        n = rng.choice(sizes, size=3)
        if max_cells is not None and int(np.prod(n)) > max_cells:
            continue
        out.append(diamond_si(int(n[0]), int(n[1]), int(n[2]), a=a, sigma=sigma, strain=strain, rng=rng))
    return out


def sio2_random(n_si=216, density=2.2, dmin=1.4, seed=2):
    """SiO2 with n_si Si and 2 n_si O in a cubic periodic box at `density`
    g/cm^3; uniform positions with rejection to a minimum image distance dmin."""
    rng = np.random.default_rng(seed)
    mass_amu = n_si * (ATOMIC_MASSES["Si"] + 2 * ATOMIC_MASSES["O"])
    vol = mass_amu * 1.66053906660 / density  # A^3
    L = vol ** (1.0 / 3.0)
    numbers = [14] * n_si + [8] * (2 * n_si)
    pos = np.zeros((len(numbers), 3))
    n = 0
    tries = 0
    while n < len(numbers):
        p = rng.uniform(0.0, L, size=3)
        tries += 1
        if tries > 10_000_000:
            raise RuntimeError("rejection sampling did not converge")
        if n:
            d = pos[:n] - p
            d -= L * np.round(d / L)
            if np.min(np.einsum("ij,ij->i", d, d)) < dmin * dmin:
                continue
        pos[n] = p
        n += 1
    return Atoms(numbers, pos, L * np.eye(3), pbc=True)


def nacl_cluster(angle_deg=1.0, a=5.691694, box=17.22):
    """8-atom NaCl rock-salt cluster (4 Na then 4 Cl) rotated by `angle_deg`
    about x around the origin, in a periodic cube of edge `box`."""
    na = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]], dtype=np.float64)
    cl = np.array([[.5, 0, 0], [0, .5, 0], [0, 0, .5], [.5, .5, .5]], dtype=np.float64)
    pos = np.vstack([na, cl]) * a
    t = np.deg2rad(angle_deg)
    c, s = np.cos(t), np.sin(t)
    rot = np.array([[1, 0, 0], [0, c, -s], [0, s, c]])
    pos = pos @ rot.T
    return Atoms([11] * 4 + [17] * 4, pos, box * np.eye(3), pbc=True)
