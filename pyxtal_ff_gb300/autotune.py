"""Autotuner of the FP32 path's launch shapes.

The reference has nothing to tune: its descriptor driver
(pyxtal_ff/descriptors/SO4.py:1414-1548) is one serial loop over centres.  On the
GPU the same work is spread over kernels whose best launch shapes depend on the
workload (lmax, atoms and images per centre, number of structures) and on the
device.  The knobs:

  wkmax        entries per window unit of the Z pass, 1..5 (the window work lists are
               built for it; so4_tuning.wkmax)
  rev_threads  threads per CTA of the per-image dE/dr pass, 128 or 256
  utot_warps   centres per CTA of the U_tot pass, 2, 4 or 8
  rev_pair     layout of the per-image pass: 1 two lanes per image, 2 one lane per row chain
  zw_atoms     atoms per CTA of the window Z pass: 32 (one per lane) or 64 (two per lane,
               up to twol 8)
  zw_threads   threads per CTA of the 64-atom window pass, 256 or 512
  branches     parallel graph branches of the captured linear step, 1..4
  pdl          programmatic dependent launch between that step's kernels

The search is a coordinate descent from the defaults: each knob in turn takes every
value with the others held at the best so far, and a value is kept when it is faster
by more than `min_gain`; rounds repeat until nothing changes.  Every candidate is
checked before it is timed: its forces and stress on a validation batch must match
a reference evaluation (the FP64 plain path contracted as the reference's consumers
contract dxdr / rdxdr) to the FP32 path's tolerance; a candidate that fails is never
chosen.  Choices persist per (device, lmax, workload class) in a JSON file
($SO4_TUNE_CACHE, else ~/.cache/pyxtal_ff_gb300/tuning.json).
"""
from __future__ import annotations

import dataclasses
import json
import math
import os
import tempfile
from dataclasses import dataclass

import numpy as np

SPACE_ORDER = ("branches", "wkmax", "zw_atoms", "zw_threads", "rev_pair", "rev_threads", "utot_warps", "pdl")


@dataclass(frozen=True)
class Choice:
    """One point of the search space (0 in a kernel field: the table builder's default)."""
    wkmax: int = 5
    rev_threads: int = 0
    utot_warps: int = 4
    branches: int = 2
    pdl: bool = False
    rev_pair: int = 0
    zw_atoms: int = 0
    zw_threads: int = 0

    def kernel_tuning(self):
        """(wkmax, rev_threads, utot_warps, rev_pair, zw_atoms, zw_threads) for engine.tables /
        so4_tables_create_tuned."""
        return (int(self.wkmax), int(self.rev_threads), int(self.utot_warps), int(self.rev_pair),
                int(self.zw_atoms), int(self.zw_threads))

    def as_dict(self):
        return dataclasses.asdict(self)

    @classmethod
    def from_dict(cls, d):
        return cls(**{f.name: d[f.name] for f in dataclasses.fields(cls) if f.name in d})


def search_space(twol, linear=True):
    """Values each knob may take for this twol (the kernels build every CTA shape for twol
    6 and 8 only) and step kind (branches and PDL exist only in the captured linear step)."""
    shapes = twol in (6, 8)
    return {
        "branches": (2, 1, 3, 4) if linear else (1,),
        "wkmax": (5, 4, 3),
        "rev_threads": ((256, 128) if shapes else (0,)),
        "utot_warps": ((4, 2, 8) if shapes else (4,)),
        "rev_pair": ((0, 1, 2) if shapes else (0,)),
        "zw_atoms": ((32, 64) if twol <= 8 else (0,)),
        "zw_threads": ((256, 512) if twol <= 8 else (0,)),
        "pdl": (False, True) if linear else (False,),
    }


def default_choice(twol, linear=True):
    return Choice(wkmax=5, rev_threads=0, utot_warps=4, branches=2 if linear else 1, pdl=False)


def coordinate_descent(evaluate, start, space, rounds=3, min_gain=0.01):
    """Minimise evaluate(choice) -> time (None: the choice failed its check) by one knob at a
    time.  Returns (best choice, its time, [(choice, time)] for every evaluated choice)."""
    seen = {}

    def ev(c):
        if c not in seen:
            seen[c] = evaluate(c)
        return seen[c]

    best, best_t = start, ev(start)
    if best_t is None:
        raise RuntimeError("autotune: the starting choice %r failed its check" % (start,))
    for _ in range(rounds):
        improved = False
        for knob in SPACE_ORDER:
            for v in space.get(knob, ()):
                c = dataclasses.replace(best, **{knob: v})
                if c == best:
                    continue
                t = ev(c)
                if t is not None and t < best_t * (1.0 - min_gain):
                    best, best_t, improved = c, t, True
        if not improved:
            break
    return best, best_t, [(c, t) for c, t in seen.items()]


# ----------------------------------------------------------------- cache
def cache_path():
    p = os.environ.get("SO4_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "pyxtal_ff_gb300", "tuning.json")


class TuningCache:
    """Choices keyed by workload_key(); written atomically (temporary file + rename)."""

    def __init__(self, path=None):
        self.path = path or cache_path()

    def _load(self):
        try:
            with open(self.path) as fh:
                d = json.load(fh)
            return d if isinstance(d, dict) else {}
        except (OSError, ValueError):
            return {}

    def get(self, key):
        e = self._load().get(key)
        if not e:
            return None
        return Choice.from_dict(e["choice"]), float(e["ms"])

    def put(self, key, choice, ms):
        d = self._load()
        d[key] = {"choice": choice.as_dict(), "ms": float(ms)}
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        fd, tmp = tempfile.mkstemp(dir=os.path.dirname(os.path.abspath(self.path)), suffix=".tmp")
        with os.fdopen(fd, "w") as fh:
            json.dump(d, fh, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def workload_key(device_name, twol, natoms, nimg, nstruct, kind):
    """Workloads of one class share a choice: atoms and structures by powers of two, images
    per centre rounded, the step kind ('linear', 'model' or 'train')."""
    b = lambda n: int(round(math.log2(max(int(n), 1))))  # noqa: E731
    ipa = int(round(nimg / max(natoms, 1)))
    return "%s|twol%d|%s|atoms2^%d|structs2^%d|ipa%d" % (device_name, int(twol), kind, b(natoms), b(nstruct), ipa)


# ----------------------------------------------------------------- GPU front ends
def _median_ms(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def validation_batch(batch, max_atoms=2048):
    """The leading structures of a batch, up to max_atoms atoms (at least one structure)."""
    from .calculator import Batch
    n, k = 0, 0
    sizes = np.diff(batch.atom_ptr)
    while k < batch.nstruct and (k == 0 or n + sizes[k] <= max_atoms):
        n += int(sizes[k])
        k += 1
    if k == batch.nstruct:
        return batch
    return Batch(batch.structures[:k], species_order=batch.species_order)


class Validator:
    """Forces and stress of a linear energy on a validation batch by the FP64 plain path (the
    reference arithmetic), against which each candidate's FP32 captured step is checked:
    max |dF| <= tol max|F| and max |d stress| <= tol max|stress| (tol 2e-4, the FP32 path's
    tolerance against the oracle)."""

    def __init__(self, calc, batch, tol=2e-4, seed=12345):
        import torch
        from .calculator import LinearModel, contract_plain
        self.calc, self.tol = calc, tol
        self.batch = validation_batch(batch)
        nsp = max(len(self.batch.species_order), 1)
        coef = np.random.default_rng(seed).normal(0.0, 0.01, size=(nsp, calc.nB))
        self.model = LinearModel(coef).to(calc.device)
        d = calc.descriptors(self.batch, precision="fp64")
        beta = torch.as_tensor(coef, device=calc.device)[calc._species]
        ref = contract_plain(d["x"], d["dxdr"], d["rdxdr"], d["seq"], d["pair_ptr"], self.batch.atom_ptr, beta,
                             self.batch.volumes)
        self.f_ref, self.s_ref = ref["forces"], ref["stress"]
        del d

    def check(self, branches, pdl):
        step = self.calc.capture(self.batch, self.model, branches=branches, pdl=pdl)
        res = step()
        ef = float((res["forces"] - self.f_ref).abs().max())
        es = float((res["stress"] - self.s_ref).abs().max())
        ok = (ef <= self.tol * max(float(self.f_ref.abs().max()), 1e-30)
              and es <= self.tol * max(float(self.s_ref.abs().max()), 1e-30))
        del step
        return ok, ef, es


def autotune_step(calc, batch, model, *, steps=20, warmup=5, rounds=3, use_cache=True, cache=None, log=None):
    """Tune the captured energy / forces / stress step of `model` on `batch`, apply the choice
    to `calc` (calc.set_tuning) and return a report dict.  A LinearModel gets the whole space;
    any other model the kernel knobs (its captured step is one stream)."""
    import torch
    from .calculator import LinearModel
    linear = isinstance(model, LinearModel)
    calc.prepare(batch)
    nb = calc.neighbors(batch, torch.from_numpy(batch.positions).to(calc.device))
    dev_name = torch.cuda.get_device_name(calc.device)
    key = workload_key(dev_name, calc.twol, nb.natoms, nb.nimg, nb.nstruct, "linear" if linear else "model")
    del nb
    cache = cache or TuningCache()
    if use_cache:
        hit = cache.get(key)
        if hit is not None:
            calc.set_tuning(hit[0])
            return {"key": key, "choice": hit[0].as_dict(), "ms": hit[1], "cached": True}
    val = Validator(calc, batch)

    def evaluate(c):
        calc.set_tuning(c)
        ok, ef, es = val.check(c.branches, c.pdl)
        if not ok:
            if log:
                log("autotune: %r rejected (force err %.3g, stress err %.3g)" % (c, ef, es))
            return None
        calc.prepare(batch)
        step = calc.capture(batch, model, branches=c.branches, pdl=c.pdl)
        t = _median_ms(step, steps, warmup)
        del step
        if log:
            log("autotune: %r %.4f ms" % (c, t))
        return t

    start = default_choice(calc.twol, linear)
    best, best_t, table = coordinate_descent(evaluate, start, search_space(calc.twol, linear), rounds=rounds)
    calc.set_tuning(best)
    calc.prepare(batch)
    cache.put(key, best, best_t)
    return {"key": key, "choice": best.as_dict(), "ms": best_t, "cached": False,
            "default_ms": dict(table).get(start),
            "evaluated": [{"choice": c.as_dict(), "ms": t} for c, t in table]}


def autotune_training(make_trainer, calc, batch, *, steps=10, warmup=3, rounds=3, use_cache=True, cache=None,
                      log=None):
    """Tune the kernel knobs of a captured training step: make_trainer(choice) returns a
    trainer with step() and capture(); each choice is first checked like autotune_step's
    (a linear energy's FP32 step on the leading structures of `batch` with `calc`, an
    SO4Calculator of the trainer's descriptor, against its FP64 plain path)."""
    import torch
    dev_name = torch.cuda.get_device_name(calc.device)
    calc.prepare(batch)
    nb = calc.neighbors(batch, torch.from_numpy(batch.positions).to(calc.device))
    key = workload_key(dev_name, calc.twol, nb.natoms, nb.nimg, nb.nstruct, "train")
    del nb
    cache = cache or TuningCache()
    if use_cache:
        hit = cache.get(key)
        if hit is not None:
            return {"key": key, "choice": hit[0].as_dict(), "ms": hit[1], "cached": True}
    val = Validator(calc, batch)

    def evaluate(c):
        calc.set_tuning(c)
        ok, ef, es = val.check(1, False)
        if not ok:
            if log:
                log("autotune: %r rejected (force err %.3g, stress err %.3g)" % (c, ef, es))
            return None
        tr = make_trainer(c)
        tr.capture(warmup=2)
        t = _median_ms(tr.step, steps, warmup)
        del tr
        if log:
            log("autotune: %r %.4f ms" % (c, t))
        return t

    start = default_choice(calc.twol, linear=False)
    best, best_t, table = coordinate_descent(evaluate, start, search_space(calc.twol, linear=False), rounds=rounds)
    calc.set_tuning(best)
    cache.put(key, best, best_t)
    return {"key": key, "choice": best.as_dict(), "ms": best_t, "cached": False,
            "default_ms": dict(table).get(start),
            "evaluated": [{"choice": c.as_dict(), "ms": t} for c, t in table]}
