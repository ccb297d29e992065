"""Benchmark of the SO4 energy + forces + stress path on one GB300 (or N replicas).

Workload: diamond-Si 20x20x10 supercell (32,000 atoms, a = 5.43 A, Gaussian
displacement sigma = 0.1 A, seed 5), SO4 lmax = 4, rcut = 5.0 A, cosine cutoff,
unit Si weight, psi = pi r / rcut; energy from a fixed linear model with
coefficients ~ N(0, 0.01) (seed 6).  One step = GPU neighbour list + FP32
forward (U_tot, B) + model + FP32 adjoint (forces, virial), with the positions
already in HBM.  The FP64 plain dB/dr path (NL + B, dxdr, rdxdr + the
consumers' contraction) is timed on the same structure and is the error
reference.  `e2e` is the same metric through SO4Calculator.compute() from
pinned host positions, with the H2D copy and the D2H read of energy, forces
and stress inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

LMAX, RCUT, SEED_POS, SEED_COEF = 4, 5.0, 5, 6
METRIC = "SO4 atoms/s w/ forces+stress: FP32 adjoint vs plain FP64 dB/dr, 1 GB300; err vs FP64"
CONFIG = {"workload": "diamond-Si 20x20x10 (32000 atoms), SO4 lmax=4, rcut=5.0 A, energy+forces+stress, "
                      "linear model N(0,0.01)", "structures": 1, "atoms": 32000, "lmax": LMAX, "rcut": RCUT,
          "neighbor_list": "in step", "l2": "flushed between steps (512 MiB write)",
          "path": "one CUDA graph: GPU neighbour list, FP32 U_tot, fused B + Y window pass (Z once), per-image "
                  "dE/dr, gather (compensated FP32 per atom, FP64 across atoms)"}


# DRAM bytes (read + write) per full launch of each stage's kernel: the figures of the
# one-kernel captures of a 16,384-atom case (profiles/k_zw64_k_utot_rc_k_jvp_du_rc_si16384_lmax4.md
# for the window and U_tot passes, profiles/k_utot_rc_k_zw32_k_deidrj_rev2_si16384_lmax4.md for
# the per-image pass), times 1.95 for the atoms and images of the 32,000-atom workload
NCU_TRAFFIC = {"utot32": 25.8e6, "linear_by32": 48.2e6, "adjoint_deidrj32": 68.2e6}


def workload():
    from pyxtal_ff_gb300 import structures as S
    atoms = S.diamond_si(20, 20, 10, sigma=0.1, rng=np.random.default_rng(SEED_POS))
    from pyxtal_ff_gb300.flops import sizes
    nB = sizes(2 * LMAX)["nB"]
    coef = np.random.default_rng(SEED_COEF).normal(0.0, 0.01, size=nB)
    return atoms, coef


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return None


def reference_python_record():
    """Timings of the reference's own Python code (numba unavailable: CPython + NumPy) and of
    the oracle on one thread of the same host, taken where the reference source can be
    imported (tests/golden/time_reference.py writes tests/golden/reference_timing.json); a
    side record, not measured in this run."""
    try:
        with open(os.path.join(HERE, "tests", "golden", "reference_timing.json")) as fh:
            d = json.load(fh)
    except (OSError, ValueError):
        return None
    d["note"] = ("measured by tests/golden/time_reference.py on the host named here, not in this run: the "
                 "reference's source tree is not present on the GPU host")
    return d


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ----------------------------------------------------------------- clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return out
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        load = [r for r in rows if r[2] > 250.0] or rows
        out.update(sm_mhz=float(np.median([r[0] for r in load])), sm_max_mhz=max(r[1] for r in rows),
                   reasons=reasons, samples=len(rows), power_w_max=max(r[2] for r in rows))
        return out


# ----------------------------------------------------------------- peaks
def kernels_back_to_back(calc, batch, pos_dev, beta_dev, reps=20):
    """Mean launch duration (ms) of the three adjoint kernels and of the JVP (two launches:
    the per-image tangent pass and the window pass), each called `reps` times back to back
    through its C-ABI entry and replayed as one CUDA graph, so no host launch gap enters (the
    eager stage table includes them)."""
    import ctypes as C
    import torch
    from pyxtal_ff_gb300 import _lib
    from pyxtal_ff_gb300.engine import _ptr, _stream, check

    dev = pos_dev.device
    nb = calc.neighbors(batch, pos_dev)
    tab, prm, L = calc.tables, calc.params, _lib.lib()
    N, M = nb.natoms, nb.nimg
    beta = beta_dev.to(torch.float32).contiguous()
    utot = torch.empty((N, tab.n_half, 2), dtype=torch.float32, device=dev)
    x = torch.empty((N, tab.nB), dtype=torch.float32, device=dev)
    y = torch.empty((N, tab.n_half, 2), dtype=torch.float32, device=dev)
    bc = torch.empty((tab.n_bsec, N), dtype=torch.float32, device=dev)
    eatom = torch.empty(N, dtype=torch.float32, device=dev)
    g = torch.empty((M, 3), dtype=torch.float32, device=dev)
    v = torch.from_numpy(np.random.default_rng(7).normal(size=(N, 3))).to(dev)
    dB = torch.empty((N, tab.nB), dtype=torch.float32, device=dev)
    jws = torch.empty(L.so4_jvp_workspace_size(tab.handle, N), dtype=torch.uint8, device=dev)
    w_nb, w_site = calc._w_nb, calc._w_site
    calls = {
        "utot32": lambda: check(L.so4_utot32(tab.handle, C.byref(prm), N, _ptr(w_nb), _ptr(w_site), _ptr(nb.img_ptr),
                                             _ptr(nb.img_j), _ptr(nb.img_r), _ptr(utot), _stream()), "so4_utot32"),
        "linear_by32": lambda: check(L.so4_linear_by32(tab.handle, N, _ptr(utot), _ptr(beta), _ptr(x), _ptr(y),
                                                       _ptr(bc), _ptr(eatom), _stream()), "so4_linear_by32"),
        "adjoint_deidrj32": lambda: check(L.so4_adjoint_deidrj32(tab.handle, C.byref(prm), N, _ptr(w_nb),
                                                                 _ptr(nb.img_ptr), _ptr(nb.img_j), _ptr(nb.img_r), M,
                                                                 _ptr(y), _ptr(g), _stream()), "so4_adjoint_deidrj32"),
        # the training path's backward (forces' tangent through B), on the same structure
        "jvp32": lambda: check(L.so4_jvp32(tab.handle, C.byref(prm), _ptr(nb.atom_struct), N, _ptr(w_nb),
                                           _ptr(nb.img_ptr), _ptr(nb.img_j), _ptr(nb.img_r), _ptr(utot), _ptr(v),
                                           _ptr(None), _ptr(dB), _ptr(jws), jws.numel(), _stream()), "so4_jvp32"),
    }
    out = {}
    for name, f in calls.items():
        for _ in range(3):
            f()
        torch.cuda.synchronize()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            f()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr):
            for _ in range(reps):
                f()
        gr.replay()
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        gr.replay()
        e1.record(st)
        e1.synchronize()
        out[name] = e0.elapsed_time(e1) / reps
        del gr
    return out


def run_ase_md(nstep=10):
    """One MD step of the reference's published ASE example (1000-atom diamond Si, a = 5.659 A,
    SNAP lmax 3, Rc 5.0, weight 1.0, NN 12-12 tanh, about 16 s per step on a CPU) through
    PyXtalFFCalculator: the lattice displaced by sigma 0.1 A (about 1000 K), each step moves the
    atoms by a further sigma 0.02 A, then one calculate() from host positions to host energies,
    forces and stress.  Both routes: 'plain'
    (FP64 descriptors with dxdr and per-atom rdxdr, the reference's arithmetic) and 'adjoint'
    (FP32 adjoint forces).  Random-initialised network; descriptor range from the structure
    itself; the ZBL base potential of the example is left out (not part of this path)."""
    import torch
    from pyxtal_ff_gb300 import structures as S
    from pyxtal_ff_gb300.ase_calculator import ForceField, PyXtalFFCalculator, compute_descriptor
    from pyxtal_ff_gb300.nn import NeuralNetworkPotential

    rng = np.random.default_rng(21)
    atoms = S.diamond_si(5, 5, 5, a=5.659, sigma=0.1, rng=rng)
    desc = {"type": "SNAP", "Rc": 5.0, "cutoff": "cosine", "weights": {"Si": 1.0}, "base_potential": None,
            "parameters": {"lmax": 3}}
    x = compute_descriptor(desc, atoms)["x"]
    lo, hi = x.min(0), x.max(0)
    hi = np.where(hi > lo, hi, lo + 1.0)
    torch.manual_seed(22)
    nb = x.shape[1]
    net = torch.nn.Sequential(torch.nn.Linear(nb, 12), torch.nn.Tanh(), torch.nn.Linear(12, 12), torch.nn.Tanh(),
                              torch.nn.Linear(12, 1)).double()
    base = atoms.positions.copy()
    out = {"workload": "1000-atom diamond Si (5x5x5, a 5.659 A, sigma 0.1 A, 0.02 A more per step), SNAP "
                       "lmax 3, Rc 5.0, NN 12-12 tanh (random init), energy + forces + stress per step, host "
                       "positions in, host results out; ZBL base potential left out",
           "published_cpu_s_per_step": 16.0, "published_source": "examples/Si-LAMMPS/README.md:28-40"}
    for route in ("plain", "adjoint"):
        ff = ForceField(desc, NeuralNetworkPotential({"Si": net}, {"Si": np.stack([lo, hi], 1)}))
        calc = PyXtalFFCalculator(ff=ff, route=route)
        ts = []
        for it in range(nstep + 2):
            atoms.positions = base + rng.normal(0.0, 0.02, size=base.shape)
            t0 = time.perf_counter()
            calc.calculate(atoms)
            ts.append(time.perf_counter() - t0)
        ms = 1e3 * float(np.median(ts[2:]))
        out[route] = {"ms_per_step": ms, "speedup_vs_published": 16.0 / (ms * 1e-3)}
    return out


def measured_peaks(torch):
    """Measured denominators: HBM from MEASURED_PEAKS.json; FP32 / FP64 CUDA-core rates
    measured here with cuBLAS SGEMM (TF32 off) / DGEMM, since that file has none."""
    peaks = {}
    try:
        peaks.update(json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))))
        peaks["source"] = "MEASURED_PEAKS.json"
    except Exception:
        peaks.update(hbm_gbs=6800.0, source="fallback")
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt, n in (("fp32_tflops", torch.float32, 8192), ("fp64_tflops", torch.float64, 4096)):
        a = torch.randn(n, n, device="cuda", dtype=dt)
        b = torch.randn(n, n, device="cuda", dtype=dt)
        for _ in range(2):
            a @ b
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        peaks[name] = 2.0 * n ** 3 / (best * 1e-3) / 1e12
        del a, b
    torch.backends.cuda.matmul.allow_tf32 = prev
    peaks.update(fma_peaks(torch))
    return peaks


def fma_peaks(torch):
    """The FP32 and FP64 FMA pipes measured directly (so4_peak_fma: 8 CTAs of 256 threads
    per SM, 8 independent FMA chains per thread), best of 3 launches of about 10 ms."""
    import ctypes as C
    from pyxtal_ff_gb300 import _lib
    from pyxtal_ff_gb300.engine import _stream
    L = _lib.lib()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks = 8 * sms
    out = torch.empty(blocks * 256, dtype=torch.float32, device="cuda")
    res = {}
    for name, kind, iters in (("fp32_ffma2_tflops", 0, 80000), ("fp32_ffma_tflops", 1, 80000),
                              ("fp64_dfma_tflops", 2, 2400)):
        flop = C.c_double()
        best = 1e9
        for _ in range(4):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.check(L.so4_peak_fma(kind, iters, blocks, C.c_void_p(out.data_ptr()), C.byref(flop), _stream()),
                       "so4_peak_fma")
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        res[name] = flop.value / (best * 1e-3) / 1e12
    res["fp32_fma_tflops"] = max(res["fp32_ffma2_tflops"], res["fp32_ffma_tflops"])
    return res


def nl_back_to_back(step, reps=20):
    """Mean duration (ms) of the captured step's neighbour list in its one-branch form (bins and
    per-atom keys, sort with the FP64 image vectors, reverse images, summary), `reps` times back to
    back in one CUDA graph, and its algorithmic bytes: positions read, per image j, offset (3 x i32),
    vector (3 x f64) and reverse index written, per atom the image pointer."""
    import torch
    from pyxtal_ff_gb300 import engine
    lay, b = step.layout, step.nl
    for _ in range(3):
        engine.enqueue_neighbors(lay, step.pos, b, lite=True)
    torch.cuda.synchronize()
    gr = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        engine.enqueue_neighbors(lay, step.pos, b, lite=True)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    with torch.cuda.graph(gr):
        for _ in range(reps):
            engine.enqueue_neighbors(lay, step.pos, b, lite=True)
    gr.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    gr.replay()
    e1.record()
    e1.synchronize()
    M = int(b.summary_dev().cpu()[0])
    N = lay.natoms
    nbytes = 24 * N + 4 * (N + 1) + M * (4 + 12 + 24 + 4)
    return e0.elapsed_time(e1) / reps, nbytes, M


# ----------------------------------------------------------------- CPU side
def cpu_run(atoms, coef, nthreads):
    """The oracle (C restatement of the reference path, FP64) on every centre of the
    workload: B, energy, forces and the contracted virial.  Returns (seconds, results)."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    beta = np.broadcast_to(coef, (len(atoms), len(coef)))
    ref = O.forces_virial(atoms, beta, kind="SNAP", lmax=LMAX, rcut=RCUT, weights={"Si": 1.0}, rfac0=1.0,
                          nthreads=nthreads)
    return time.perf_counter() - t0, ref


def errors_vs(got, ref):
    """Errors of one GPU path (host arrays: x, energy, forces, stress in GPa) against
    reference results of the same shapes: max abs and max-normalised relative."""
    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
    return {"force_max_abs_eV_per_A": float(np.max(np.abs(got["forces"] - ref["forces"]))),
            "force_max_rel": rel(got["forces"], ref["forces"]),
            "stress_max_abs_GPa": float(np.max(np.abs(got["stress"] - ref["stress"]))),
            "stress_max_rel": rel(got["stress"], ref["stress"]),
            "energy_rel": abs(got["energy"] - ref["energy"]) / abs(ref["energy"]),
            "B_max_rel": rel(got["x"], ref["x"])}


def oracle_results(ref):
    """The oracle's results in the GPU paths' units: stress (1, 6) GPa in the reference's
    Voigt order and sign, from its virial (which carries 1/V)."""
    from pyxtal_ff_gb300.calculator import EV_A3_TO_GPA, VOIGT
    return {"x": ref["x"], "energy": float(ref["energy"]), "forces": ref["forces"],
            "stress": -(ref["virial"].reshape(1, 9)[:, VOIGT]) * EV_A3_TO_GPA}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    atoms, coef = workload()
    nth = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_run(atoms, coef, nth)
    times = [cpu_run(atoms, coef, nth)[0] for _ in range(args.steps)]
    t = float(np.sum(times))
    value = len(atoms) * args.steps / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atoms/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": "atoms/s", "cores": nth, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "all 32000 centres of the workload per step (oracle, OpenMP)"},
            "e2e": {"value": value, "unit": "atoms/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_python": reference_python_record()}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU side
def run_contract(args):
    """The contraction alone: plain FP64 descriptors of an N x N x 10 cell, then
    args.steps back-to-back so4_contract_dxdr calls (forces and stress) timed with events."""
    import torch
    from pyxtal_ff_gb300 import engine
    from pyxtal_ff_gb300 import structures as S
    from pyxtal_ff_gb300.calculator import Batch, SO4Calculator
    n = args.contract_cells
    atoms = S.diamond_si(n, n, 10, sigma=0.1, rng=np.random.default_rng(5))
    batch = Batch([atoms])
    calc = SO4Calculator(lmax=LMAX, rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
    d = calc.descriptors(batch, precision="fp64")
    nb = d["neighbors"]
    rda = engine.rdxdr_atom(d["rdxdr"], nb.pair_ptr, nb.natoms)
    del d["rdxdr"]
    beta = torch.from_numpy(np.random.default_rng(6).normal(0, 0.01, (nb.natoms, calc.nB))).cuda()
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = (torch.empty((nb.natoms, 3), dtype=torch.float64, device="cuda"),
           torch.empty((nb.natoms, 6), dtype=torch.float64, device="cuda"),
           torch.empty((1, 6), dtype=torch.float64, device="cuda"))

    def once():
        engine.contract_dxdr(beta, nb.pair_ptr, nb.seq, nb.atom_struct, nb.atom_ptr_dev, dxdr=d["dxdr"],
                             rdxdr_atom=rda, status=st, out=out)
    for _ in range(max(args.warmup, 1)):
        once()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        once()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    if int(st.item()):
        raise RuntimeError("asymmetric pair list")
    byt = 8 * (nb.npair * calc.nB * 3 + nb.natoms * calc.nB * 7 + 2 * nb.npair)
    print(json.dumps({"contract_only": True, "atoms": nb.natoms, "pairs": nb.npair, "ms": ms,
                      "gbs": byt / (ms * 1e-3) / 1e9}), flush=True)


def run_profile_case(which):
    """Small cases of single kernels for ncu captures (summaries under profiles/)."""
    import torch
    from pyxtal_ff_gb300 import engine, ops
    from pyxtal_ff_gb300 import structures as S
    from pyxtal_ff_gb300.calculator import Batch, SO4Calculator
    if which == "plain":
        batch = Batch([S.diamond_si(8, 8, 4, sigma=0.1, rng=np.random.default_rng(5))])
        calc = SO4Calculator(lmax=LMAX, rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
        for _ in range(2):
            d = calc.descriptors(batch, precision="fp64")
            torch.cuda.synchronize()
            del d
    elif which == "train":
        from pyxtal_ff_gb300.train import ForceMatching
        batch = Batch(S.si_batch(512, seed=4, sizes=range(1, 9), max_cells=8, strain=0.04, sigma=0.1))
        fm = ForceMatching(batch, lmax=3, rcut=4.9, seed=4)
        fm.capture(warmup=2)
        for _ in range(3):
            fm.step()
        torch.cuda.synchronize()
    elif which == "nl":
        from pyxtal_ff_gb300.calculator import LinearModel
        batch = Batch([S.diamond_si(16, 16, 8, sigma=0.1, rng=np.random.default_rng(5))])
        calc = SO4Calculator(lmax=LMAX, rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
        step = calc.capture(batch, LinearModel(np.zeros(calc.nB)).cuda(), branches=1)
        for _ in range(3):
            engine.enqueue_neighbors(step.layout, step.pos, step.nl, lite=True)
        torch.cuda.synchronize()
    elif which == "linear":
        batch = Batch([S.diamond_si(16, 16, 8, sigma=0.1, rng=np.random.default_rng(5))])
        p = torch.from_numpy(batch.positions).cuda()
        ctx = ops.Context.build(p, batch.cells, batch.pbc, batch.atom_ptr, batch.numbers, batch.symbols, lmax=LMAX,
                                rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
        beta = torch.from_numpy(np.random.default_rng(6).normal(0, 0.01, (batch.natoms, ctx.tab.nB))).float().cuda()
        for _ in range(3):
            engine.adjoint_linear32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.w_site, beta)
        torch.cuda.synchronize()
    else:
        batch = Batch([S.diamond_si(16, 16, 8, sigma=0.1, rng=np.random.default_rng(5))])
        p = torch.from_numpy(batch.positions).cuda()
        ctx = ops.Context.build(p, batch.cells, batch.pbc, batch.atom_ptr, batch.numbers, batch.symbols, lmax=LMAX,
                                rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0)
        x, utot = engine.forward32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, ctx.w_site)
        v = torch.from_numpy(np.random.default_rng(1).normal(size=(batch.natoms, 3))).cuda()
        for _ in range(3):
            engine.jvp32(ctx.tab, ctx.prm, ctx.nb, ctx.w_nb, utot, v=v)
        torch.cuda.synchronize()
    print(json.dumps({"profile_case": which, "atoms": batch.natoms}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-train", action="store_true", help="skip the training-step leg")
    ap.add_argument("--no-tune", action="store_true", help="default launch shapes instead of the autotuner's choice")
    ap.add_argument("--quick", action="store_true",
                    help="device-resident steps only (no e2e, FP64, CPU or peak legs); for profiler runs")
    ap.add_argument("--profile-case", choices=["plain", "jvp", "linear", "nl", "train"], default=None,
                    help="only a small case for profiler runs: 'plain' = two FP64 plain-path evaluations of a "
                         "2,048-atom diamond-Si cell, 'jvp' = the FP32 forward and three JVPs of a 16,384-atom "
                         "cell, 'linear' = three fused linear-energy evaluations (U_tot, window B + Y, "
                         "per-image pass, gather) of the 16,384-atom cell, 'nl' = three one-branch neighbour "
                         "lists of the captured step on the 16,384-atom cell (lmax 4, rcut 5.0), 'train' = the "
                         "force-matching training step (512 Si structures, lmax 3) captured, then three replays")
    ap.add_argument("--contract-cells", type=int, default=0,
                    help="only the NN consumer's dxdr contraction (so4_contract_dxdr) on an N x N x 10 diamond-Si "
                         "cell at lmax 4 (a small case for profiler runs)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.contract_cells:
        run_contract(args)
        return
    if args.profile_case:
        run_profile_case(args.profile_case)
        return

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if ws > 1:
            dist.barrier()

    from pyxtal_ff_gb300 import replicas

    def max_over_ranks(v):
        return replicas.max_over_ranks(v, device=dev)

    from pyxtal_ff_gb300 import _lib, autotune, engine, flops
    from pyxtal_ff_gb300.calculator import EV_A3_TO_GPA, Batch, LinearModel, SO4Calculator

    atoms, coef = workload()
    batch = Batch([atoms])
    calc = SO4Calculator(lmax=LMAX, rcut=RCUT, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0, device=dev)
    model = LinearModel(coef).to(dev)
    # launch shapes: the autotuner's choice for this workload, searched afresh (outside every
    # timed region; each candidate checked against the FP64 plain path first)
    tuning = None
    if not args.no_tune:
        rep = autotune.autotune_step(calc, batch, model, use_cache=False)
        tuning = {"choice": rep["choice"], "ms": rep["ms"], "default_ms": rep["default_ms"],
                  "evaluated": len(rep["evaluated"]),
                  "rejected": sum(1 for e in rep["evaluated"] if e["ms"] is None)}
    calc.prepare(batch)
    pos_dev = torch.from_numpy(batch.positions).to(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    tab, prm = calc.tables, calc.params
    L = _lib.lib()

    stage_names = ["neighbors", "utot32", "linear_by32", "adjoint_deidrj32", "gather"]
    beta_dev = model.coef.detach()[calc._species].contiguous()
    bias0 = float(model.bias.detach()[0])

    def device_step(ev=None):
        """One step with the inputs in HBM: neighbour list, U_tot, the fused B + Y pass of the
        linear energy, per-image dE/dr, forces / virial gather and the energy; ev: events
        recorded between the stages."""
        def mark(i):
            if ev is not None:
                ev[i].record()
        mark(0)
        nb = calc.neighbors(batch, pos_dev)
        mark(1)
        x, forces, virial, energy = engine.linear_staged(tab, prm, nb, calc._w_nb, calc._w_site, beta_dev, mark=mark,
                                                         first=1)
        energy = energy + bias0
        mark(5)
        return energy, forces, virial

    # ---- warm-up
    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()

    # ---- the step as one CUDA graph (SO4Calculator.capture): the headline, positions in HBM
    step = calc.capture(batch, model)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    natoms = len(atoms)
    step_ms = []
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        step()
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    barrier()
    if not step.check():
        raise RuntimeError("neighbour list outgrew the captured capacity")
    launches = step.launches
    t_dev = max_over_ranks(float(np.sum(step_ms)))
    value = ws * natoms * args.steps / (t_dev * 1e-3)

    # ---- the same step eagerly, stage by stage (kernel table and roofline; not the headline)
    nev = len(stage_names) + 1
    stage_ms = np.zeros(len(stage_names))
    eager_ms = []
    for _ in range(args.steps):
        flush.zero_()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(nev)]
        device_step(ev)
        ev[-1].synchronize()
        eager_ms.append(ev[0].elapsed_time(ev[-1]))
        stage_ms += np.array([ev[i].elapsed_time(ev[i + 1]) for i in range(nev - 1)])
    stage_ms /= args.steps
    b2b_ms = kernels_back_to_back(calc, batch, pos_dev, beta_dev)
    nl_ms, nl_bytes, nl_images = nl_back_to_back(step)
    if args.quick:
        clocks.stop()
        if rank == 0:
            print(json.dumps({"quick": True, "value": value, "unit": "atoms/s", "ms_per_step": t_dev / args.steps,
                              "eager_ms_per_step": float(np.mean(eager_ms)),
                              "stages_ms": dict(zip(stage_names, stage_ms.tolist())),
                              "kernels_back_to_back_ms": b2b_ms,
                              "gpu_launches": int(launches)}), flush=True)
        if ws > 1:
            dist.destroy_process_group()
        return

    # ---- e2e through the public API (the captured step with host I/O: the graph copies the
    # positions in from the step's pinned host buffer and energy, forces and stress out to
    # pinned host buffers; one graph launch and one wait per step)
    step_io = calc.capture(batch, model, host_io=True)
    step_io.host_positions.copy_(torch.from_numpy(batch.positions))
    for _ in range(2):
        step_io()
    torch.cuda.synchronize()
    barrier()
    t_e2e = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res_host = step_io()
        t_e2e += time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e)
    if not step_io.check():
        raise RuntimeError("neighbour list outgrew the captured capacity")
    e2e = {"value": ws * natoms * args.steps / t_e2e, "unit": "atoms/s",
           "h2d_bytes_per_step": int(step_io.host_positions.numel() * 8),
           "d2h_bytes_per_step": int(sum(v.numel() for v in res_host.values()) * 8),
           "ms_per_step": 1e3 * t_e2e / args.steps,
           "api": "SO4Calculator.capture(batch, model, host_io=True)()"}
    del step_io
    pos_host = torch.from_numpy(batch.positions.copy()).pin_memory()
    out_f = torch.empty((natoms, 3), dtype=torch.float64).pin_memory()
    # the uncaptured public call on the same host buffers, for reference
    t_eager = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r2 = calc.compute(batch, model, positions=pos_host)
        out_f.copy_(r2["forces"], non_blocking=True)
        torch.cuda.synchronize()
        t_eager += time.perf_counter() - t0
    e2e["uncaptured_compute_ms_per_step"] = 1e3 * t_eager / args.steps

    # ---- plain FP64 dB/dr path on the same structure + errors of the FP32 path
    coef_t = torch.as_tensor(coef, dtype=torch.float64, device=dev)

    beta64 = coef_t.expand(natoms, -1).contiguous()

    def contract(d):
        # the reference NN consumer's contraction of dxdr / rdxdr with dE/dB (so4_contract_dxdr)
        nb = d["neighbors"]
        rda = engine.rdxdr_atom(d["rdxdr"], nb.pair_ptr, nb.natoms)
        f, s = engine.contract_dxdr(beta64, nb.pair_ptr, nb.seq, nb.atom_struct, nb.atom_ptr_dev, dxdr=d["dxdr"],
                                    rdxdr_atom=rda)
        return {"forces": f, "stress": s * EV_A3_TO_GPA, "rdxdr_atom": rda}

    def plain_step():
        d = calc.descriptors(batch, pos_dev, precision="fp64")
        return d, contract(d)
    plain_step()
    torch.cuda.synchronize()
    t64 = []
    for _ in range(2):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        d64, c64 = plain_step()
        e1.record()
        e1.synchronize()
        t64.append(e0.elapsed_time(e1))
    ms64 = max_over_ranks(float(np.mean(t64)))
    # the contraction alone on the FP64 dxdr (HBM-bound: each dxdr row is read once)
    nbp = d64["neighbors"]
    # (inputs of 1.3 GB, far above L2: back-to-back launches, no flush needed)
    cstat = torch.zeros(1, dtype=torch.int32, device=dev)
    cout = (torch.empty((natoms, 3), dtype=torch.float64, device=dev),
            torch.empty((natoms, 6), dtype=torch.float64, device=dev),
            torch.empty((1, 6), dtype=torch.float64, device=dev))

    def contract_once():
        engine.contract_dxdr(beta64, nbp.pair_ptr, nbp.seq, nbp.atom_struct, nbp.atom_ptr_dev, dxdr=d64["dxdr"],
                             rdxdr_atom=c64["rdxdr_atom"], status=cstat, out=cout)
    contract_once()
    torch.cuda.synchronize()
    tc = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(4):
            contract_once()
        e1.record()
        e1.synchronize()
        tc.append(e0.elapsed_time(e1) / 4)
    if int(cstat.item()):
        raise RuntimeError("so4_contract_dxdr: asymmetric pair list")
    nB = calc.nB
    cbytes = 8 * (nbp.npair * nB * 3 + natoms * nB * 6 + natoms * nB + 2 * nbp.npair + 3 * natoms + 6 * natoms)
    ms_c = float(np.min(tc))
    clk = clocks.stop()  # sampled over the device, e2e and FP64 timed legs
    clk["window"] = "device + e2e + fp64 timed legs"
    stress64 = c64["stress"]  # rdxdr already carries 1/vol
    res = {k: v.clone() for k, v in step(pos_host).items()}  # the captured (headline) step
    torch.cuda.synchronize()
    res_eager = calc.compute(batch, model)
    graph_equals_eager = all(torch.equal(res[k], res_eager[k]) for k in ("energy", "forces", "virial", "x"))
    e64 = float((d64["x"].double() @ coef_t).sum())
    # host copies of both GPU paths' results (the oracle comparison comes after the CPU leg)
    got32 = {"x": res["x"].double().cpu().numpy(), "energy": float(res["energy"].sum()) - bias0,
             "forces": res["forces"].cpu().numpy(), "stress": res["stress"].cpu().numpy()}
    got64 = {"x": d64["x"].cpu().numpy(), "energy": e64, "forces": c64["forces"].cpu().numpy(),
             "stress": stress64.cpu().numpy()}
    err = errors_vs(got32, got64)
    err["graph_bitwise_equals_uncaptured"] = bool(graph_equals_eager)
    del d64, c64
    fp64 = {"ms_per_step": ms64, "atoms_per_s": ws * natoms / (ms64 * 1e-3),
            "speedup_fp32_adjoint_over_fp64_plain": ms64 / (t_dev / args.steps)}

    # ---- roofline of the dominant kernel (live CUDA events of the timed region)
    nb = calc.neighbors(batch, pos_dev)
    kf = flops.kernel_flops(2 * LMAX, nb.natoms, nb.nimg)     # the work the kernels' own algorithm does
    ks = flops.tabulated_flops(2 * LMAX, nb.natoms, nb.nimg)     # the reference algorithm's tabulated work
    peaks = measured_peaks(torch)
    i_dom = int(np.argmax(stage_ms))
    dom = stage_names[i_dom]
    if dom in ks:
        sec = b2b_ms.get(dom, stage_ms[i_dom]) * 1e-3  # the kernel's own launch duration
        achieved = ks[dom] / sec / 1e12
        roof = {"kernel": dom, "bound": "fp32", "achieved": achieved, "peak": peaks["fp32_tflops"],
                "unit": "TFLOP/s", "frac": achieved / peaks["fp32_tflops"], "traffic": NCU_TRAFFIC.get(dom),
                "traffic_unit": "bytes per launch (ncu dram read + write)",
                "work": "tabulated per-unit work of the reference algorithm x units per launch",
                "achieved_executed": kf[dom] / sec / 1e12,
                "frac_executed": kf[dom] / sec / 1e12 / peaks["fp32_tflops"],
                "frac_vs_fma_loop": achieved / peaks["fp32_fma_tflops"],
                "frac_executed_vs_fma_loop": kf[dom] / sec / 1e12 / peaks["fp32_fma_tflops"],
                "fma_loop_tflops": peaks["fp32_fma_tflops"],
                "peak_source": "cuBLAS SGEMM (TF32 off) measured in this run; the kernel is FP32-FMA bound, "
                               "its DRAM traffic is far below the HBM roof",
                "duration": "mean of 20 back-to-back launches replayed as one CUDA graph (no host gaps)",
                "ms": sec * 1e3}
        # the same launch against the HBM roof (ncu DRAM bytes per launch / its duration, of the
        # measured copy rate): how far from memory bound the kernel is
        tr, hbm = NCU_TRAFFIC.get(dom), peaks.get("hbm_gbs")
        if tr and hbm:
            roof["hbm"] = {"achieved_gbs": tr / sec / 1e9, "peak_gbs": hbm, "frac": tr / sec / 1e9 / hbm,
                           "peak_source": peaks.get("source", "")}
    else:
        roof = {"kernel": dom, "bound": "latency", "achieved": None, "peak": None, "unit": None, "frac": None,
                "traffic": None}
    kernels = {}
    for i, nme in enumerate(stage_names):
        k = {"ms": float(stage_ms[i])}
        if nme in b2b_ms:
            k["ms_back_to_back"] = b2b_ms[nme]
        if nme in ks:
            sec = b2b_ms.get(nme, stage_ms[i]) * 1e-3
            k["tflops"] = ks[nme] / sec / 1e12
            k["frac_fp32"] = k["tflops"] / peaks["fp32_tflops"]
            k["tflops_executed"] = kf[nme] / sec / 1e12
        kernels[nme] = k
    cflop = 2.0 * (nbp.npair * nB * 3 + natoms * nB * 6)  # one FMA per dxdr / rdxdr_atom element
    kernels["contract_dxdr_fp64"] = {
        "ms": ms_c, "gbs": cbytes / (ms_c * 1e-3) / 1e9, "frac_hbm": cbytes / (ms_c * 1e-3) / 1e9 / peaks["hbm_gbs"],
        "tflops_fp64": cflop / (ms_c * 1e-3) / 1e12,
        "frac_fp64": cflop / (ms_c * 1e-3) / 1e12 / peaks["fp64_tflops"],
        "bytes": cbytes, "what": "forces and stress of the reference NN consumer from the FP64 dxdr (%.2f GB) and "
                                 "per-atom rdxdr; bytes = dxdr + rdxdr_atom + beta + seq + outputs; FP64 pipe and "
                                 "HBM bound it about equally on GB300" % (8e-9 * nbp.npair * nB * 3)}
    # the neighbour list against the HBM roof: it moves 44 B per image and runs far below that
    # roof, bound by the latency of its per-centre bin walks (profiles/k_scan_images_k_sort_*)
    kernels["neighbors_lite"] = {
        "ms_back_to_back": nl_ms, "bytes": nl_bytes, "images": nl_images,
        "gbs": nl_bytes / (nl_ms * 1e-3) / 1e9, "frac_hbm": nl_bytes / (nl_ms * 1e-3) / 1e9 / peaks["hbm_gbs"],
        "bound": "latency (per-centre bin walk), not HBM",
        "traffic": 25.9e6, "traffic_unit": "DRAM bytes per full list: scan + sort + reverse images of a 16,384-atom "
                                           "list from ncu (profiles/k_scan_images_k_sort_k_rev_si16384_dram.md) x 1.95; "
                                           "below the algorithmic bytes because the outputs stay in L2",
        "what": "one-branch form of the captured step's list: bins + per-atom keys, sort with FP64 image vectors, "
                "reverse images, summary; bytes = positions + image pointer + 44 B per image written"}
    # the JVP (training's backward) on the same structure: executed work only (the reference has
    # no such step: its trainer back-propagates through stored dxdr)
    kernels["jvp32"] = {"ms_back_to_back": b2b_ms["jvp32"],
                        "tflops_executed": kf["jvp32"] / (b2b_ms["jvp32"] * 1e-3) / 1e12,
                        "what": "so4_jvp32 with a per-atom tangent: per-image tangent pass + window pass"}
    kernels["jvp32"]["frac_executed"] = kernels["jvp32"]["tflops_executed"] / peaks["fp32_tflops"]
    for nme in ("utot32", "linear_by32", "adjoint_deidrj32", "jvp32"):
        k = kernels.get(nme, {})
        if "tflops_executed" in k:
            k["frac_executed_vs_fma_loop"] = k["tflops_executed"] / peaks["fp32_fma_tflops"]
        if "tflops" in k:
            k["frac_vs_fma_loop"] = k["tflops"] / peaks["fp32_fma_tflops"]
    # the per-kernel times are full-size launches back to back; the step runs each of them as two
    # half-size launches in parallel graph branches, plus the list and the gather
    kernels["step_reconciliation"] = {
        "sum_of_back_to_back_kernels_ms": float(sum(v for k, v in b2b_ms.items() if k != "jvp32")) + nl_ms,
        "gather_ms_eager": float(stage_ms[stage_names.index("gather")]),
        "step_ms": t_dev / args.steps,
        "note": "U_tot, window and per-image kernels back to back at full size, plus the one-branch "
                "neighbour list; the captured step runs two branches over the atom halves, so kernel tails "
                "overlap and the step is close to this sum plus the gather"}
    kernels["plain_fp64"] = {"ms": ms64, "tflops_fp64_incl_nl_contraction": ks["plain"] / (ms64 * 1e-3) / 1e12,
                             "frac_fp64": ks["plain"] / (ms64 * 1e-3) / 1e12 / peaks["fp64_tflops"],
                             "frac_fp64_vs_dfma_loop": ks["plain"] / (ms64 * 1e-3) / 1e12 / peaks["fp64_dfma_tflops"]}

    # ---- force-matching training step (512 Si structures of 8-64 atoms, lmax 3), extra line item
    train = None
    if not args.no_train:
        from pyxtal_ff_gb300 import structures as S
        from pyxtal_ff_gb300.train import ForceMatching
        tstructs = S.si_batch(512, seed=4, sizes=range(1, 9), max_cells=8, strain=0.04, sigma=0.1)
        tbatch = Batch(tstructs)
        tchoice, ttune = None, None
        if not args.no_tune:
            from pyxtal_ff_gb300.train import stillinger_weber
            targets = stillinger_weber(tbatch)
            tcalc = SO4Calculator(lmax=3, rcut=4.9, kind="SNAP", weights={"Si": 1.0}, rfac0=1.0, device=dev)
            rep = autotune.autotune_training(
                lambda c: ForceMatching(tbatch, lmax=3, rcut=4.9, seed=4, targets=targets, tuning=c), tcalc, tbatch,
                use_cache=False)
            tchoice = autotune.Choice.from_dict(rep["choice"])
            ttune = {"choice": rep["choice"], "ms": rep["ms"], "default_ms": rep["default_ms"],
                     "evaluated": len(rep["evaluated"]),
                     "rejected": sum(1 for e in rep["evaluated"] if e["ms"] is None)}
            del tcalc
        fm = ForceMatching(tbatch, lmax=3, rcut=4.9, seed=4, tuning=tchoice)

        def time_steps(nstep=10):
            for _ in range(2):
                fm.step()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(nstep):
                fm.step()
            e1.record()
            e1.synchronize()
            return e0.elapsed_time(e1) / nstep
        t_eager = time_steps()
        fm.capture(warmup=2)
        tms = time_steps()
        train = {"workload": "512 Si structures (8-64 atoms, 22256 atoms), SO4 lmax 3, rcut 4.9, MLP 30-30 tanh, "
                             "loss MSE(E/atom)+0.1 MSE(F), Adam; B and U_tot held on device; one CUDA graph per step",
                 "ms_per_step": tms, "atoms_per_s": fm.batch.natoms / (tms * 1e-3), "uncaptured_ms_per_step": t_eager,
                 "tuning": ttune}
        del fm

    # ---- the reference's published MD workload through the ASE-calculator interface, extra line item
    ase_md = None
    if not args.no_train:
        ase_md = run_ase_md()

    # ---- CPU baseline (the oracle, all host threads), rank 0 only
    # its results pin both GPU paths at the full workload: err_vs_oracle
    cpu = None
    err_oracle = None
    if rank == 0 and not args.no_cpu:
        nth = os.cpu_count() or 1
        tcpu, ref = cpu_run(atoms, coef, nth)
        cpu = {"value": natoms / tcpu, "unit": "atoms/s", "cores": nth, "kind": "port",
               "cpu_model": cpu_model(),
               "sample": "all 32000 centres of the workload, one evaluation (oracle, OpenMP, FP64)"}
        ro = oracle_results(ref)
        err_oracle = {"fp32_adjoint": errors_vs(got32, ro), "fp64_plain": errors_vs(got64, ro),
                      "oracle": "the C restatement of the reference path (FP64) on all 32000 centres",
                      "targets": {"fp32_adjoint": "force <= 1e-4 eV/A, stress <= 1e-3 GPa",
                                  "fp64_plain": "<= 1e-10 relative on every array"}}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "atoms/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_dev / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 tables and reductions)",
                "data": "synthetic (seeded diamond-Si, sigma 0.1 A)", "config": CONFIG,
                "pairs_per_s": ws * (nb.npair) * args.steps / (t_dev * 1e-3),
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
                "fp64_plain": fp64, "err_vs_oracle": err_oracle, "err_vs_fp64": err, "kernels": kernels,
                "train_step": train,
                "ase_md_step": ase_md, "tuning": tuning, "reference_python": reference_python_record(),
                "peaks": {k: peaks[k] for k in ("hbm_gbs", "fp32_tflops", "fp64_tflops", "fp32_ffma2_tflops",
                                                "fp32_ffma_tflops", "fp64_dfma_tflops") if k in peaks}}
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
