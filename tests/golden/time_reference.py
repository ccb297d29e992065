"""Time the reference's own SO4/SNAP code (pure CPython: numba is unavailable) on the
64-atom and 648-atom workloads, and the C oracle on one thread of the same host.

The reference is loaded exactly as make_golden.py loads it (its unmodified
``pyxtal_ff/descriptors`` modules, numba's decorators replaced by the identity, ASE's
NeighborList by the brute-force stand-in).  It cannot run on a machine without its
source tree, so the timings are taken where it can and written to
reference_timing.json, which bench.py reports beside its live CPU baseline.

Workloads (derivative=True, stress=True, one calculate() call each, one thread):
- si64: diamond Si 2x2x2 (64 atoms, a 5.43 A, sigma 0.05 A, seed 0), SNAP weight
  Si 1.0, rfac0 1.0, lmax 3, rcut 4.9 A;
- sio2_648: SiO2 216 Si + 432 O at 2.2 g/cm^3 (seed 2, minimum distance 1.4 A),
  SNAP weights Si 1.0 / O 0.5, rfac0 0.99363, lmax 4, rcut 5.0 A.

    PYXTAL_FF_REF=<reference root> python tests/golden/time_reference.py
"""
import json
import os
import platform
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

import make_golden  # noqa: E402
from oracle import oracle as O  # noqa: E402
from pyxtal_ff_gb300 import structures as S  # noqa: E402


def _cpu_model():
    try:
        for line in subprocess.run(["lscpu"], capture_output=True, text=True).stdout.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor()


def _cases():
    si64 = S.diamond_si(2, 2, 2, sigma=0.05, rng=np.random.default_rng(0))
    sio2 = S.sio2_random(n_si=216, density=2.2, dmin=1.4, seed=2)
    return [("si64", si64, dict(lmax=3, rcut=4.9, weights={"Si": 1.0}, rfac0=1.0)),
            ("sio2_648", sio2, dict(lmax=4, rcut=5.0, weights={"Si": 1.0, "O": 0.5}, rfac0=0.99363))]


def main():
    so4, snap, _ = make_golden.load_reference()
    out = {"what": "one SO4_Bispectrum.calculate(atoms) with derivative=True, stress=True (SNAP variant), "
                   "the reference's unmodified Python on one thread; numba unavailable (its decorators are the "
                   "identity), so this is CPython + NumPy speed, not numba speed",
           "host_cpu": _cpu_model(), "python": platform.python_version(), "numpy": np.__version__, "cases": {}}
    for name, atoms, p in _cases():
        f = snap.SO4_Bispectrum(p["weights"], lmax=p["lmax"], rcut=p["rcut"], derivative=True, stress=True,
                                rfac0=p["rfac0"])
        t0 = time.perf_counter()
        ref = f.calculate(atoms)
        t_ref = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc = O.descriptor(atoms, kind="SNAP", lmax=p["lmax"], rcut=p["rcut"], weights=p["weights"],
                           rfac0=p["rfac0"], derivative=True, stress=True, nthreads=1)
        t_orc = time.perf_counter() - t0
        rel = {k: float(np.max(np.abs(orc[k] - ref[k])) / np.max(np.abs(ref[k]))) for k in ("x", "dxdr", "rdxdr")}
        n, npair = len(atoms), int(ref["seq"].shape[0])
        out["cases"][name] = {"atoms": n, "pairs": npair, "lmax": p["lmax"], "rcut": p["rcut"],
                              "reference_python_s": t_ref, "reference_python_atoms_per_s": n / t_ref,
                              "oracle_1thread_s": t_orc, "oracle_1thread_atoms_per_s": n / t_orc,
                              "oracle_vs_reference_max_rel": rel}
        print(name, json.dumps(out["cases"][name]), flush=True)
    with open(os.path.join(HERE, "reference_timing.json"), "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
