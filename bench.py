"""Benchmark: converged 1D Kohn-Sham SCF solves per second on GB300.

Workload (the batched configuration): 4096 seeded synthetic molecules, grids
of 257/385/513 points at 0.08 bohr, 1-4 nuclei of charge 1-3 in [-3, 3] bohr,
neutral; FP32 window-17 MLP exchange-correlation (17->16->16->1, SiLU,
Glorot-uniform from seed 0, local convention); FP64 SCF with the five-point
kinetic operator; 25 iterations, linear mixing alpha=0.5 decaying by 0.9,
one mixing difference; non-interacting start computed inside the solve.

A step is one batched solve of the whole batch (one kernel launch).  A solve
counts as converged under the full rule: |E_25 - E_24| < 1e-8 Ha with its
status flags clear, and its final energy within 1e-8 Ha and final density
within 1e-7 (L2) of the oracle with the same FP32 network.  The oracle runs on
the first ``--cpu-sample`` molecules (which also time the CPU baseline); the
batch's self-consistent count is scaled by the sample's pass rate, and the
line's ``parity`` object reports the error distributions against the oracle
with the FP32 and with an FP64 network.  ``value`` times the solve with inputs resident on the device; ``e2e``
times the public API with host inputs (descriptor upload and energy/density
download inside the timed region).  ``--impl reference`` times the
reference algorithm (NumPy FP64 restatement: dense eigh, materialised
Hartree kernel) on the host cores on a bounded sample.
"""

from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged SCF solves/sec at 1e-8 Ha (batched 1D, 4096 molecules)"
UNIT = "solves/s"
E_CONV = 1e-8
FP64_PEAK_FALLBACK_TFLOPS = 1.18  # FP64 FMA throughput measured on this GB300 pool


def workload(batch_size, seed):
    from qex_gb300.od import workloads

    return workloads.batched_molecules(batch_size, seed=seed)


def mlp_params(seed=0):
    from qex_gb300 import networks

    init_fn, xc_fn = networks.build_xc_functional(networks.WindowMLP().build_network(None),
                                                  np.zeros(5))
    return init_fn(seed), xc_fn


# ---------------------------------------------------------------------------
# CPU reference arm: the oracle (reference algorithm) on host cores
# ---------------------------------------------------------------------------

def _cpu_solve(args):
    """One solve of the oracle (reference algorithm: dense eigh, materialised
    Hartree kernel).  Returns (self-consistency flag, energy trajectory, final
    density); ``net_dtype`` is the arithmetic of the window MLP."""
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    from oracle import ks1d as o

    (n, r, z, ne, params, iters, net_dtype) = args
    g = (np.arange(n) - (n - 1) / 2) * 0.08
    xc = o.WindowMLP(params, dtype=net_dtype)
    ve = o.get_atomic_chain_potential(g, r, z, o.exponential_coulomb)
    n0, _, _ = o.solve_noninteracting_system(ve, ne, g, 5, "dense")
    res = o.kohn_sham(r, z, ne, iters, g, xc, o.exponential_coulomb, n0, alpha=0.5,
                      alpha_decay=0.9, num_mixing_iterations=1, convention="local", stencil=5,
                      method="dense")
    e = res["total_energy"]
    return bool(abs(e[-1] - e[-2]) < E_CONV), np.asarray(e), np.asarray(res["density"][-1])


def cpu_sample(mols, params, iters, sample, cores, net_dtype=np.float32):
    """Oracle solves of mols[:sample] on `cores` host processes (spawned, one
    molecule per task).  Returns (wall seconds, self-consistent count, count,
    per-molecule results)."""
    jobs = [(m.num_grids, m.locations, m.nuclear_charges, m.num_electrons, params, iters,
             net_dtype) for m in mols[:sample]]
    ctx = mp.get_context("spawn")
    env_old = os.environ.get("OPENBLAS_NUM_THREADS")
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    os.environ["OMP_NUM_THREADS"] = "1"
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_solve, jobs, chunksize=1)
    dt = time.perf_counter() - t0
    if env_old is not None:
        os.environ["OPENBLAS_NUM_THREADS"] = env_old
    return dt, sum(r[0] for r in res), len(jobs), res


def parity_summary(mols, energy, status, dens, ref32, ref64):
    """Oracle agreement of the GPU solves of a sample (the molecules of ref32 /
    ref64, in order).  A solve passes the full convergence rule when it is
    self-consistent (|E_25 - E_24| < 1e-8 Ha, status clear) AND its final
    energy is within 1e-8 Ha and its final density within 1e-7 (L2,
    sqrt(sum dn^2 dx)) of the oracle with the FP32 network (the network
    arithmetic of this workload).  The same statistics against the oracle
    with an FP64 network are reported beside it."""
    k = len(ref32)
    selfc = (np.abs(energy[:k, -1] - energy[:k, -2]) < E_CONV) & ((status[:k] & 0xFFFF) == 0)
    frontier = (status[:k] & 0x100) != 0
    out = {"sample": k, "self_consistent": int(selfc.sum()),
           "degenerate_frontier_flagged": int(frontier.sum())}
    full = None
    for name, ref in (("fp32_network", ref32), ("fp64_network", ref64)):
        if ref is None:
            continue
        de = np.array([abs(energy[i, -1] - ref[i][1][-1]) for i in range(k)])
        detraj = np.array([np.max(np.abs(energy[i] - ref[i][1])) for i in range(k)])
        dn = np.array([np.sqrt(np.sum((dens[i] - ref[i][2]) ** 2) * mols[i].grid_spacing)
                       for i in range(k)])
        ok = selfc & (de <= 1e-8) & (dn <= 1e-7)
        sc = selfc & ~frontier

        def stats(a, m):
            a = a[m]
            if a.size == 0:
                return None
            return {"max": float(a.max()), "p50": float(np.median(a)),
                    "p90": float(np.quantile(a, 0.9))}

        out[name] = {
            "final_energy_abs_err": {"self_consistent": stats(de, sc), "all": stats(de, ~frontier)},
            "trajectory_energy_abs_err_max": {"self_consistent": stats(detraj, sc),
                                              "all": stats(detraj, ~frontier)},
            "final_density_l2_err": {"self_consistent": stats(dn, sc), "all": stats(dn, ~frontier)},
            "full_rule_converged": int(ok.sum()),
        }
        if name == "fp32_network":
            full = ok
    return out, selfc, full


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if s[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# roofline tally
# ---------------------------------------------------------------------------

# DRAM bytes per molecule of a 25-iteration batched solve: 419.2 MB read +
# written by the 950-molecule K=4 bucket launch under ncu (FP32 solve planes
# and workspace vectors evicted from L2)
DRAM_BYTES_PER_MOLECULE = 419.2e6 / 950


def fp64_flops(mols, iterations_run, stats):
    """FP64 flops executed, tallied per code path of the kernel (an FMA is 2)."""
    total = 0.0
    for m, it, st in zip(mols, iterations_run, stats):
        n = m.num_grids
        nocc = (m.num_electrons + 1) // 2
        k = m.num_electrons // 2 + 1
        solves, rq_vec, upd = (int(x) for x in st[:3])
        # per SCF iteration: two Hartree scans (15 N each), v_KS assembly and
        # drift (4 N), energies (4 N), mixing (8 N), density (2 N nocc + 2 N),
        # XC energy sum (2 N)
        per_iter = (30 + 4 + 4 + 8 + 2 + 2) * n + 2 * n * nocc
        # per eigen-solve: FP64 diagonal (1 N), normalisations (~5 N per vector)
        per_solve = n + 5 * n * k
        # per Rayleigh-quotient pass: H x (7 N), x.x and x.Hx (4 N), residual (2 N);
        # per correction: x += w (1 N)
        total += float(it) * per_iter + solves * per_solve + 13.0 * n * rq_vec + 1.0 * n * upd
    return total


def fp32_flops_mlp(mols, iterations_run):
    # window-17 MLP: forward 2*(17*16+16*16+16) flops, backward ~ the same again
    fwd = 2 * (17 * 16 + 16 * 16 + 16)
    return float(sum(float(it) * m.num_grids * (3 * fwd) for m, it in zip(mols, iterations_run)))


# global-local conv KSR network (16 channels), FP32 flops per grid point of one
# KS iteration: the forward pass (16 two-sided exponential scans 112, two
# width-3 16->16 convolutions 2 x 1536, swish 2 x 64, output layer and
# self-interaction 39) is 3351; the backward pass 3414; an iteration runs the
# forward and backward passes at the input density (v_xc) and the forward pass
# at the output density (E_xc)
KSR_FLOPS_PER_POINT = 3351 + 3414 + 3351


def ksr_trained_params():
    """The trained H2 network shipped with the reference (data/od/h2/h2_optimal.pkl),
    stored as plain arrays in the test fixtures."""
    k = np.load(os.path.join(ROOT, "tests", "golden", "ksr_h2.npz"))
    return {"eta": k["eta"], "conv": [k["w1"], k["w2"]], "out": k["w3"],
            "width": float(k["width"])}


def run_ksr(args, peak64, peak32, flush):
    """KSR workload: 4096 H2 molecules (unit charges at +-R/2, R ~ U[0.5, 3.0]
    from the seed), 513 points at 0.08, the trained global-local conv network,
    jax_dft local convention with reflection symmetry, 15 iterations, one
    mixing step, five-point kinetic operator (the reference's KSR training SCF,
    qedft/train/od/train.py:84-125)."""
    import torch

    import qex_gb300
    from qex_gb300.od import engine as eng

    rng = np.random.default_rng(args.seed + 1)
    B, iters = args.batch, 15
    mols = [eng.Molecule1D(num_grids=513, grid_spacing=0.08, locations=np.array([-r / 2, r / 2]),
                           nuclear_charges=np.array([1.0, 1.0]), num_electrons=2)
            for r in rng.uniform(0.5, 3.0, B)]
    batch = eng.PackedBatch(mols)
    xc = qex_gb300.Partial(qex_gb300.KSRFunctional(16), params=ksr_trained_params())
    cfg = eng.SolveConfig(num_iterations=iters, alpha=0.5, alpha_decay=0.9,
                          num_mixing_iterations=1, convention="local", stencil=5,
                          enforce_reflection_symmetry=True)
    engine = eng.Ks1dEngine(autotune=True)
    out = engine.allocate_outputs(batch, cfg, ("energy", "final_density"))
    for _ in range(args.warmup):
        engine.solve(batch, xc, cfg, out=out)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        engine.solve(batch, xc, cfg, out=out)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    step_s = sum(times) / len(times)
    energy = out["energy"].cpu().numpy()
    status = out["status"].cpu().numpy()
    iters_run = out["iterations_run"].cpu().numpy()
    stats = out["stats"].cpu().numpy()
    conv = (np.abs(energy[:, -1] - energy[:, -2]) < E_CONV) & ((status & 0xFFFF) == 0)
    w64 = fp64_flops(mols, iters_run, stats)
    w32 = float(KSR_FLOPS_PER_POINT * 513 * iters_run.sum())
    bound_s = w64 / (peak64 * 1e12) + (w32 / (peak32 * 1e12) if peak32 else 0.0)
    return {
        "workload": f"{B} H2 molecules, R ~ U[0.5,3.0] bohr, 513 points, trained global-local "
                    f"conv KSR network (FP32, 16 channels), local convention, reflection "
                    f"symmetry, {iters} iterations, 5-point kinetic",
        "ms_per_step": step_s * 1e3, "solves_per_s": B / step_s,
        "converged_solves_per_s": float(conv.sum()) / step_s,
        "converged_fraction": float(conv.mean()),
        "roofline": {"bound": "fp64+fp32", "achieved_fp32_tflops": w32 / step_s / 1e12,
                     "peak_fp32_tflops": peak32, "achieved_fp64_tflops": w64 / step_s / 1e12,
                     "peak_fp64_tflops": peak64, "frac": bound_s / step_s,
                     "fp32_flops_per_step": w32, "fp64_flops_per_step": w64},
    }


def run_ksr_eval(args):
    """The KSR network alone (qex_ksr1d_eval, forward and backward, local
    convention) on args.batch copies of the eight reference H2 densities."""
    import ctypes

    import torch

    import qex_gb300
    from qex_gb300 import _native
    from qex_gb300.od import xc_eval

    lib = xc_eval._lib()
    k = np.load(os.path.join(ROOT, "tests", "golden", "ksr_h2.npz"))
    fn = qex_gb300.KSRFunctional(16)
    spec, keep = fn.spec(ksr_trained_params(), _native.QEX_XC_LOCAL)
    B = args.batch
    dens = np.tile(k["densities"], (B // len(k["densities"]) + 1, 1))[:B]
    dev = torch.device("cuda")
    d = torch.as_tensor(dens.reshape(-1), device=dev)
    ng = torch.full((B,), 513, dtype=torch.int32, device=dev)
    off = torch.arange(B, dtype=torch.int64, device=dev) * 513
    dx = torch.full((B,), 0.08, dtype=torch.float64, device=dev)
    vals, pot = torch.empty_like(d), torch.empty_like(d)
    en = torch.empty(B, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    st = ctypes.c_void_p(stream.cuda_stream)

    def run():
        _native.check(lib.qex_ksr1d_eval(B, 513, ng.data_ptr(), off.data_ptr(), dx.data_ptr(),
                                         ctypes.byref(spec), d.data_ptr(), vals.data_ptr(),
                                         pot.data_ptr(), en.data_ptr(), st), "qex_ksr1d_eval")

    for _ in range(args.warmup):
        run()
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = sorted(times)[len(times) // 2]
    flops = (3351 + 3414) * 513 * B
    _, peak32 = _native.measure_fma_peak()
    del keep
    return {"workload": f"KSR network forward+backward, {B} densities x 513 points",
            "ms": t * 1e3, "achieved_fp32_tflops": flops / t / 1e12, "peak_fp32_tflops": peak32,
            "frac": flops / t / 1e12 / peak32}


def run_fermi_eval(args):
    """Fermi-Dirac occupation search (``qex_td_fermi_occupations``, stable mode,
    100 damped Newton steps at most) on args.batch spectra of 220 orbitals,
    against the oracle's per-spectrum loop on the host."""
    import torch

    from qex_gb300.td import fermi

    rng = np.random.default_rng(args.seed)
    B, n = args.batch, 220
    e = np.sort(rng.uniform(-3.0, 3.0, (B, n)), axis=1)
    ne = 2.0 * rng.integers(1, n // 2, B)
    ed = torch.as_tensor(e, device="cuda")
    nd = torch.as_tensor(ne, device="cuda")
    for _ in range(args.warmup):
        fermi.get_fractional_occupations_jax_stable(ed, nd, 0.04, None, 0.0, 0.6, 100)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fermi.get_fractional_occupations_jax_stable(ed, nd, 0.04, None, 0.0, 0.6, 100)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = sorted(times)[len(times) // 2]
    from oracle import td as otd

    k = min(B, 64)
    t0 = time.perf_counter()
    for i in range(k):
        otd.get_fractional_occupations_jax_stable(e[i], float(ne[i]), 0.04, None, 0.0, 0.6, 100)
    cpu = (time.perf_counter() - t0) / k
    return {"workload": f"Fermi occupations, {B} spectra x {n} orbitals, theta 0.04",
            "ms": t * 1e3, "spectra_per_s": B / t,
            "cpu_baseline": {"spectra_per_s": 1.0 / cpu, "cores": 1, "kind": "port",
                             "sample": f"{k} spectra, oracle loop"}}


def run_grid_eval(args):
    """Becke/Stratmann molecular grid (level 3) for seeded synthetic molecules of
    8 and 20 atoms: GPU build time, against the oracle's NumPy partition."""
    import torch

    from oracle import td as otd
    from qex_gb300.td import grids, workloads

    out = {}
    for na in (8, 20):
        m = workloads.synthetic_molecule(na, seed=na, with_integrals=False)
        g = grids.Grids(m)
        for _ in range(args.warmup):
            g.build()
        torch.cuda.synchronize()
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            g.build()
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        t = sorted(times)[len(times) // 2]
        t0 = time.perf_counter()
        otd.becke_grid(m.charges, m.positions, 3)
        cpu = time.perf_counter() - t0
        out[f"atoms_{na}"] = {"points": int(g.weights.numel()), "ms": t * 1e3,
                              "cpu_baseline_ms": cpu * 1e3, "cpu_cores": 1}
    return {"workload": "Becke/Stratmann grid, level 3 (host tables + GPU partition), "
                        "wall time per build", **out}


def run_train_eval(args):
    """One value-and-gradient of the reference's training loss (what L-BFGS-B
    calls per step, qedft/train/od/train.py:402-466) on the GPU adjoint:
    args.batch H2 molecules (R ~ U[0.5, 3.0]), 513 points, window MLP, jax_dft
    SCF with reflection symmetry, 15 iterations, checkpoints every 5; targets
    from the exp-Coulomb LDA solve of the same molecules."""
    import torch

    from qex_gb300 import networks
    from qex_gb300.od import engine as eng
    from qex_gb300.od import train as tr

    rng = np.random.default_rng(args.seed + 2)
    B = args.batch
    R = rng.uniform(0.5, 3.0, B)
    loc = np.stack([-R / 2, R / 2], axis=1)
    z = np.ones((B, 2))
    grids = (np.arange(513) - 256) * 0.08
    mols = [eng.Molecule1D.from_grids(grids, l_, z_, 2) for l_, z_ in zip(loc, z)]
    batch = eng.PackedBatch(mols, sort=False)
    import qex_gb300

    cfg = tr.solve_config({})
    out = eng.default_engine().solve(batch, qex_gb300.LDAExpCoulomb(), cfg,
                                     records=("energy", "final_density"))
    te = out["energy"][:, -1].cpu().numpy()
    tn = out["final_density"].cpu().numpy().reshape(B, 513)
    init_fn, xc_fn = networks.build_xc_functional(networks.WindowMLP().build_network(None), grids)
    spec, flat = tr.flatten(init_fn(0))
    vg = tr.create_value_and_grad_fn(xc_fn, spec, grids, 2, {})
    for _ in range(max(1, args.warmup)):
        vg(flat, loc, z, None, te, tn)
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss, grad = vg(flat, loc, z, None, te, tn)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t = sorted(times)[len(times) // 2]
    return {"workload": f"value and gradient of the reference training loss, {B} H2 molecules, "
                        "513 points, window MLP, 15 iterations with reflection symmetry, "
                        "checkpoints every 5", "s_per_step": t,
            "molecule_gradients_per_s": B / t, "loss": float(loss),
            "grad_norm": float(np.linalg.norm(grad))}


def run_config3(args, steps=3):
    """The differentiation configuration: loss and gradient with respect to the
    FP32 window-MLP parameters of 256 H2-type molecules (unit charges,
    separation ~ U[0.5, 3.0] bohr), 513 points, 15 unrolled iterations,
    checkpoints every 5, loss sum (E - E_t)^2 + 0.1 sum |n - n_t|^2 dx with
    targets from the LDA solve; the hand-written adjoint on the GPU."""
    import torch

    import qex_gb300
    from qex_gb300.od import adjoint, engine as eng
    from qex_gb300.xc import Partial

    rng = np.random.default_rng(args.seed + 3)
    B, T = 256, 15
    mols = [eng.Molecule1D(num_grids=513, grid_spacing=0.08, locations=[-r / 2, r / 2],
                           nuclear_charges=[1.0, 1.0], num_electrons=2)
            for r in rng.uniform(0.5, 3.0, B)]
    batch = eng.PackedBatch(mols, sort=False)
    cfg = eng.SolveConfig(num_iterations=T, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                          convention="local", stencil=5)
    out = eng.default_engine().solve(batch, qex_gb300.LDAExpCoulomb(), cfg,
                                     records=("energy", "final_density"))
    te = out["energy"][:, -1].cpu().numpy()
    tn = out["final_density"].cpu().numpy()
    params, xc_fn = mlp_params(0)
    xc = Partial(xc_fn, params=params)
    adj = adjoint.Ks1dAdjoint()
    res = adj.value_and_grad(batch, xc, cfg, te, tn, density_weight=0.1, checkpoint_every=5)
    times = []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = adj.value_and_grad(batch, xc, cfg, te, tn, density_weight=0.1, checkpoint_every=5)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t = sorted(times)[len(times) // 2]
    return {"workload": f"loss and gradient, {B} H2-type molecules, 513 points, window MLP (FP32), "
                        f"{T} iterations, checkpoints every 5, loss sum (E-E_t)^2 + "
                        "0.1 sum |n-n_t|^2 dx", "s_per_step": t,
            "molecule_gradients_per_s": B / t, "loss": float(res.loss),
            "grad_norm": float(np.linalg.norm(res.grad))}


def td_flops(G, n, naux, nocc, hidden=None):
    """Algorithmic work of one 3D SCF cycle (per the 3D roofline of the
    measurement plan): FP64 GEMM-shaped work 4 G n^2 (rho and Vxc) +
    4 naux n^2 (J) + 4 n^3 (DIIS error) + 2 n^2 k (rdm1), the eigensolve
    2 n^3 + 4/3 n^3 + 4 n^2 (k + 1); FP32 network work 4 G H + 4 H^2 for a
    global [H, H, 1] network (forward and backward)."""
    w64 = 4.0 * G * n * n + 4.0 * naux * n * n + 4.0 * n ** 3 + 2.0 * n * n * nocc
    w64 += 2.0 * n ** 3 + 4.0 / 3.0 * n ** 3 + 4.0 * n * n * (nocc + 1)
    w32 = 0.0 if hidden is None else 4.0 * G * hidden + 4.0 * hidden * hidden
    return w64, w32


def run_td(args, peak64, peak32, cycles=30):
    """The 3D configuration at its shapes: synthetic molecules of 8 (s/p basis),
    14 and 20 atoms (s/p/d), Gaussian-cloud grids of 1240, ~42k and 200k points
    with positive random weights, analytic one-electron integrals and
    density-fitted Coulomb factors built on the GPU; LDA exchange and the global
    neural functional [512, 512, 1]; DIIS depth 8, 30 cycles, the reference's
    stop rule latched on the device; each SCF captured as one CUDA graph and
    replayed.  Beside it the oracle (NumPy FP64) on the host: the full SCF of the
    smallest molecule, two cycles of the others (scaled to 30)."""
    import torch

    from oracle import td as otd
    from qex_gb300.td import graph, numint, workloads

    cases = ((8, "sp", 155), (14, "spd", 3000), (20, "spd", 10000))
    if args.td_atoms:
        cases = tuple(c for c in cases if c[0] in args.td_atoms)
    out = {"workload": "3D numint SCF, synthetic H/C/N/O molecules, analytic integrals and "
                       "density-fitted J on the GPU, DIIS 8, 30 cycles (CUDA graph)"}
    cpu_total = 0.0
    for na, basis, ppa in cases:
        dev, mol = workloads.device_molecule(na, seed=100 + na, points_per_atom=ppa, basis=basis)
        G, n = dev.weights.numel(), dev.nao
        naux = int(dev.eri_factors.shape[0])
        nocc = dev.nelectron // 2
        row = {"atoms": na, "basis": basis, "nao": n, "grid_points": G, "naux": naux}
        for label, xc in (("lda", "LDA"),
                          ("global_mlp_512", numint.NeuralXC(
                              numint.NeuralXC.init(hidden=512, seed=1, inputs=G), scale=1e-2))):
            cap = graph.CapturedScf(dev, max_cycle=cycles, xc=xc)
            stream = torch.cuda.current_stream()
            times = []
            for _ in range(max(3, args.steps)):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                res = cap.replay()
                e1.record(stream)
                e1.synchronize()
                times.append(e0.elapsed_time(e1) / 1e3)
            t = sorted(times)[len(times) // 2]
            st = res.converged.cpu().numpy()
            en = res.energies.cpu().numpy()
            w64, w32 = td_flops(G, n, naux, nocc, 512 if label != "lda" else None)
            bound = cycles * (w64 / (peak64 * 1e12) + (w32 / (peak32 * 1e12) if peak32 else 0.0))
            row[label] = {"ms_per_solve": t * 1e3, "solves_per_s": 1.0 / t,
                          "converged": bool(st[0]), "converged_cycle": int(st[1]) + 1,
                          "e_tot": float(res.e_tot.cpu()[0]),
                          "last_abs_dE": float(abs(en[-1] - en[-2])),
                          "last_grad_norm": float(res.grad_norms.cpu()[-1]),
                          "eigh_path": getattr(cap, "eigh_path", None),
                          "roofline": {"bound": "fp64 (+fp32 network)", "frac": bound / t,
                                       "fp64_flops_per_cycle": w64, "fp32_flops_per_cycle": w32}}
            del cap
            torch.cuda.empty_cache()
        # oracle on the host: the LDA SCF
        hm = workloads.Molecule3D(charges=mol.charges, positions=mol.positions, shells=mol.shells,
                                  coords=mol.coords, weights=mol.weights,
                                  nelectron=mol.nelectron)
        hm.ao = dev.ao.cpu().numpy()
        hm.s1e = dev.s1e.cpu().numpy()
        hm.h1e = dev.h1e.cpu().numpy()
        hm.eri_factors = dev.eri_factors.cpu().numpy()
        hm.energy_nuc = dev.energy_nuc
        k = cycles if na == cases[0][0] else 2
        t0 = time.perf_counter()
        e_ref = otd.scf(hm, max_cycle=k)[0]
        dt = (time.perf_counter() - t0) * cycles / k
        cpu_total += dt
        row["cpu_baseline"] = {"s_per_solve": dt, "cores": host_cores(), "kind": "port",
                               "sample": f"{k} cycles of the oracle's LDA SCF"
                                         + ("" if k == cycles else f", scaled to {cycles}")}
        if k == cycles:
            row["lda"]["parity_vs_oracle_e_tot_fixed_cycles"] = float(
                abs(e_ref[-1] - float(graph_last_energy(dev, cycles))))
        out[f"atoms_{na}_{basis}"] = row
        del dev
        torch.cuda.empty_cache()
    return out


def graph_last_energy(dev, cycles):
    """Energy of the last cycle of a host-launched LDA SCF (no stop rule)."""
    from qex_gb300.td import scf

    return scf.run_scf(dev, cycles).energies[-1].cpu()


def run_eigh_eval(args):
    """Generalized eigensolves F C = S C e (batch 1) at the basis sizes of the
    3D configuration: core Hamiltonian and overlap from the analytic
    integrals of seeded molecules (s/p and spd bases).  Median wall time per
    solve over ``--steps`` repeats and the residual max|F C - S C e| / max|F|."""
    import torch

    from qex_gb300.td import eigh, integrals, workloads

    out = {}
    cases = ((8, "sp"), (20, "sp"), (20, "spd"), (21, "spd"))
    if args.eigh_atoms:
        cases = tuple(c for c in cases if c[0] in args.eigh_atoms)
    for na, basis in cases:
        m = workloads.synthetic_molecule(na, seed=na, with_integrals=False, basis=basis)
        S, T, V = integrals.int1e(m)
        F = T + V
        # the autotuner's choice of path for this size (both candidates timed)
        from qex_gb300.td.eigh import tune_path

        eigh._PATHS.pop(int(m.nao), None)
        best, path_ms = tune_path(F, S)
        for _ in range(max(args.warmup, 1)):
            w, C = eigh.generalized_eigh(F, S)
        torch.cuda.synchronize()
        times = []
        for _ in range(max(args.steps, 3)):
            t0 = time.perf_counter()
            w, C = eigh.generalized_eigh(F, S)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        res = (F @ C - S @ C * w[None, :]).abs().max().item() / F.abs().max().item()
        ev = np.linalg.eigvalsh(S.cpu().numpy())
        # the host LAPACK solve of the same problem (SciPy eigh(F, S), all host threads)
        import scipy.linalg

        Fh, Sh = F.cpu().numpy(), S.cpu().numpy()
        host = []
        for _ in range(max(args.steps, 3)):
            t0 = time.perf_counter()
            wh = scipy.linalg.eigh(Fh, Sh, eigvals_only=False)[0]
            host.append(time.perf_counter() - t0)
        out[f"atoms_{na}_{basis}"] = {"nao": int(m.nao), "ms": float(np.median(times)) * 1e3,
                                      "path_ms": {str(k): v for k, v in path_ms.items()},
                                      "tuned_path": best,
                                      "residual": res,
                                      "overlap_condition": float(ev[-1] / ev[0]),
                                      "host_scipy_ms": float(np.median(host)) * 1e3,
                                      "host_cores": host_cores(),
                                      "max_abs_eigenvalue_diff_vs_host": float(
                                          np.abs(np.sort(wh) - w.cpu().numpy()).max())}
    return {"workload": "generalized eigensolve, core Hamiltonian and overlap", **out}


# phase timers of ks1d_kernel (clock64 cycles per molecule; write_stats)
# (3 contains 8-10, 4 contains 11-13 and 15, 5 contains 14)
PHASES = {0: "Hartree on the input density", 1: "XC on the input density (network forward "
          "and backward) and v_KS", 2: "Sturm multisection", 3: "cold route: start vectors "
          "and inverse iteration", 4: "FP64 refinement, Rayleigh-Ritz, normalisation",
          5: "density, Hartree and XC energies on the output density", 6: "mixing and "
          "outputs", 7: "whole molecule", 8: "start vectors", 9: "first factorisation and "
          "solve", 10: "inverse-iteration rounds", 11: "Rayleigh quotients",
          12: "FP32 correction solves", 13: "vector updates",
          14: "XC energy on the output density (network forward)", 15: "final normalisation"}


def run_phase_eval(args):
    """The batched configuration (the headline's molecules, MLP, iterations and
    launch plan) with the kernel's per-phase clock64 timers: each phase's
    share of the summed per-molecule cycles (phase 7), and the step time."""
    import torch

    from qex_gb300 import Partial
    from qex_gb300.od import engine as eng

    mols = workload(args.batch, args.seed)
    params, xc_fn = mlp_params(0)
    xc = Partial(xc_fn, params=params)
    cfg = eng.SolveConfig(num_iterations=args.iters, alpha=0.5, alpha_decay=0.9,
                          num_mixing_iterations=1, convention="local", stencil=5)
    engine = eng.Ks1dEngine(autotune=True)
    batch = eng.PackedBatch(mols)
    out = engine.allocate_outputs(batch, cfg, ("energy",))
    for _ in range(max(args.warmup, 1)):
        engine.solve(batch, xc, cfg, out=out)
    torch.cuda.synchronize()
    ts = []
    for _ in range(max(args.steps, 1)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        engine.solve(batch, xc, cfg, out=out)
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
    pc = out["phase_cycles"].cpu().numpy().astype(np.float64)
    total = pc[:, 7].sum()
    return {"workload": f"{args.batch} molecules, window-17 MLP, {args.iters} iterations, "
                        f"5-point kinetic (the headline configuration)",
            "ms_per_step": float(np.median(ts)),
            "share_of_molecule_cycles": {f"{k} {PHASES[k]}": round(float(pc[:, k].sum() / total), 4)
                                         for k in range(16)}}


def run_ints_eval(args):
    """Analytic one-electron integrals and density-fitting factors (int3c2e,
    int2c2e, Cholesky, substitution) for seeded synthetic molecules of 8 and
    20 atoms in the s/p and the spd basis; wall time per build (the oracle's loops are too slow to time
    beside them at these sizes)."""
    import torch

    from qex_gb300.td import integrals, workloads

    out = {}
    for na, basis in ((8, "sp"), (20, "sp"), (8, "spd"), (20, "spd")):
        m = workloads.synthetic_molecule(na, seed=na, with_integrals=False, basis=basis)
        aux = integrals.even_tempered_aux(m)
        for _ in range(args.warmup):
            integrals.int1e(m)
            integrals.df_factors(m, aux)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        integrals.int1e(m)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        integrals.df_factors(m, aux)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        out[f"atoms_{na}_{basis}"] = {"nao": int(m.nao), "naux": int(sum(workloads.ncart(s.l) for s in aux)),
                              "int1e_ms": (t1 - t0) * 1e3, "df_ms": (t2 - t1) * 1e3}
    return {"workload": "analytic S, T, V and density-fitted Coulomb factors", **out}


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def combine_ranks(step_s, e2e_s, n_conv, n_mol, world, device):
    """Replicas: the job's step time is the slowest rank's (max), the work is the
    sum over ranks.  Returns (step_s, e2e_s, converged, molecules) for the job."""
    import torch

    t = torch.tensor([step_s, e2e_s], dtype=torch.float64, device=device)
    c = torch.tensor([n_conv, n_mol], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        torch.distributed.all_reduce(c, op=torch.distributed.ReduceOp.SUM)
    return float(t[0]), float(t[1]), float(c[0]), float(c[1])


def run_ours(args, rank, world):
    import torch

    from qex_gb300 import _native
    from qex_gb300.od import engine as eng
    from qex_gb300.xc import Partial

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    _native.load()
    mols = workload(args.batch, args.seed + rank)
    params, xc_fn = mlp_params(0)
    xc = Partial(xc_fn, params=params)
    cfg = eng.SolveConfig(num_iterations=args.iters, alpha=0.5, alpha_decay=0.9,
                          num_mixing_iterations=1, convention="local", stencil=5)
    # launch plan tuned on this batch during the warm-up (autotuner)
    engine = eng.Ks1dEngine(autotune=True)
    batch = eng.PackedBatch(mols)
    records = ("energy", "gap", "converged", "final_density")
    out = engine.allocate_outputs(batch, cfg, records)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        engine.solve(batch, xc, cfg, out=out)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()

    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    sampler.start()
    times = []
    launches = 0
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.fill_(1)  # evict L2 between timed solves (outside the events)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        engine.solve(batch, xc, cfg, out=out)
        e1.record(stream)
        launches += engine.last_launches
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.synchronize()
    sampler.stop()
    step_s = sum(times) / len(times)
    plan = next(iter(engine.tuner.cache.values()), None) if engine.tuner else None
    plan_desc = (None if plan is None else
                 {"bucketed": plan.bucketed, "solve_planes": plan.planes,
                  "ring_chunk": plan.chunk or 32,
                  "candidate_ms": {f"{'runs' if b else 'one'}/planes{p}/chunk{c or 32}": round(t, 3)
                                   for (b, p, c), t in
                                   next(iter(engine.tuner.timings.values())).items()}})
    energy = out["energy"].cpu().numpy()
    status = out["status"].cpu().numpy()
    iters_run = out["iterations_run"].cpu().numpy()
    stats = out["stats"].cpu().numpy()
    conv = (np.abs(energy[:, -1] - energy[:, -2]) < E_CONV) & ((status & 0xFFFF) == 0)
    n_conv = int(conv.sum())

    # ---- end-to-end through the public API with host inputs
    host = {k: getattr(batch, k).cpu().pin_memory() for k in
            ("num_grids", "offsets", "grid_start", "grid_spacing", "num_electrons",
             "num_nuclei", "locations", "nuclear_charges", "order")}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    res_host = {k: torch.empty(out[k].shape, dtype=out[k].dtype).pin_memory()
                for k in ("energy", "final_density", "status")}
    d2h = sum(t.numel() * t.element_size() for t in res_host.values())
    e2e_times = []
    for _ in range(max(2, args.steps)):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k, t in host.items():
            getattr(batch, k).copy_(t, non_blocking=True)
        engine.solve(batch, xc, cfg, out=out)
        for k, t in res_host.items():
            t.copy_(out[k], non_blocking=True)
        stream.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_times) / len(e2e_times)

    step_s, e2e_s, total_conv, total = combine_ranks(step_s, e2e_s, n_conv, args.batch, world,
                                                     "cuda")
    if rank != 0:
        return None

    try:
        peak64, peak32 = _native.measure_fma_peak()
        peak_src = "FP64 FMA throughput measured live by qex_probe_fma_peak in this run"
    except RuntimeError:
        peak64, peak32 = FP64_PEAK_FALLBACK_TFLOPS, None
        peak_src = "fallback: FP64 FMA probe measured earlier on this pool"
    w64 = fp64_flops(mols, iters_run, stats)
    w32 = fp32_flops_mlp(mols, iters_run)
    achieved = w64 / step_s / 1e12
    cpu = None
    parity = None
    value = total_conv / step_s
    if world == 1 and not args.no_cpu:
        cores = host_cores()
        sample = min(args.cpu_sample, len(mols))
        dt, cconv, cn, ref32 = cpu_sample(mols, params, args.iters, sample, cores)
        cpu = {"value": cconv / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{cn} molecules of the same workload, reference algorithm (dense "
                         f"eigh, materialised Hartree kernel), {cconv} converged, {dt:.1f} s wall",
               "total_solves_per_s": cn / dt}
        # one core (one process), a smaller sample of the same molecules
        dt1, c1, n1, _ = cpu_sample(mols, params, args.iters, min(8, sample), 1)
        cpu["single_core"] = {"value": c1 / dt1, "total_solves_per_s": n1 / dt1, "cores": 1,
                              "sample": f"first {n1} molecules, {c1} converged, {dt1:.1f} s"}
        _, _, _, ref64 = cpu_sample(mols, params, args.iters, sample, cores, np.float64)
        dens = batch.split(out["final_density"].cpu().numpy())
        parity, selfc, full = parity_summary(mols, energy, status, dens, ref32, ref64)
        # the full rule is checked on the sample; the batch's self-consistent
        # count is scaled by the sample's pass rate among its self-consistent solves
        rate = float(full.sum()) / max(1, int(selfc.sum()))
        parity["full_rule_pass_rate_of_self_consistent"] = rate
        parity["rule"] = ("converged = |E_25 - E_24| < 1e-8 Ha and status clear (whole batch) "
                          "and |E - E_oracle| <= 1e-8 Ha and density L2 <= 1e-7 against the "
                          "FP32-network oracle (checked on the first `sample` molecules; the "
                          "batch's self-consistent count is scaled by the sample's pass rate)")
        value = total_conv * rate / step_s
    ksr = None
    if world == 1 and not args.no_ksr:
        ksr = run_ksr(args, peak64, peak32, flush)
    serving = None
    if world == 1 and not args.no_serving:
        serving = run_serving(args)
    config3 = run_config3(args) if world == 1 and not args.no_ksr else None
    td = run_td(args, peak64, peak32) if world == 1 and not args.no_td else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded molecules, Glorot-init MLP from seed 0)",
        "config": {"workload": f"batched 1D KS-SCF, {args.batch} molecules x {world} ranks, "
                               f"N in {{257,385,513}}, 1-4 nuclei Z 1-3, window-17 FP32 MLP XC, "
                               f"5-point kinetic, {args.iters} iterations",
                   "global_batch": int(total), "l2": "flushed between timed steps (512 MB write)",
                   "parallelism": f"replicas x{world}",
                   "launch_plan": plan_desc},
        "total_solves_per_s": total / step_s,
        "self_consistent_fraction": total_conv / total,
        "converged_fraction": value * step_s / total,
        "e2e": {"value": value * step_s / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "s_per_step": e2e_s},
        "gpu_launches": int(launches),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64,
                     "unit": "TFLOP/s", "frac": achieved / peak64,
                     "traffic": int(DRAM_BYTES_PER_MOLECULE * args.batch),
                     "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu "
                                       "capture of the K=4 bucket launch (950 molecules, 25 "
                                       "iterations), per molecule, times the step's molecules",
                     "peak_source": peak_src, "fp32_peak_tflops": peak32,
                     "fp64_flops_per_step": w64, "fp32_mlp_flops_per_step": w32,
                     # both terms of the roofline: (W64 / P64 + W32 / P32) / t
                     "frac_fp64_plus_fp32": ((w64 / (peak64 * 1e12) + (w32 / (peak32 * 1e12)
                                                                        if peak32 else 0.0))
                                             / step_s)},
        "clocks": sampler.summary(),
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if parity is not None:
        line["parity"] = parity
    if ksr is not None:
        line["ksr"] = ksr
    if serving is not None:
        line["serving"] = serving
    if config3 is not None:
        line["differentiation"] = config3
    if td is not None:
        line["numint_3d"] = td
    return line


def run_serving(args):
    """Served (continuous batching) vs plain one-at-a-time form on a Poisson stream of
    plain-configuration 1D requests (513 points, H2-like, LDA, 3-point stencil, 20 iterations)."""
    import qex_gb300
    from qex_gb300 import serving as sv
    from qex_gb300.od import engine as eng

    cfg = eng.SolveConfig(num_iterations=20, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                          convention="local", stencil=3)
    xc = qex_gb300.LDAExpCoulomb()
    out = {"workload": "Poisson stream of 1D requests: 513 points, dx 0.08, unit charges at +-R, "
                       "R ~ U[0.5,1.5], exp-Coulomb LDA, 3-point kinetic, 20 iterations"}
    server = sv.ScfServer(xc, cfg, max_inflight=16, max_batch=1024)
    server.serve(sv.config1_requests(sv.poisson_arrivals(500, 0.05, seed=99), seed=99))  # warm-up
    for rate in args.serving_rates:
        arr = sv.poisson_arrivals(rate, args.serving_seconds, seed=int(rate))
        reqs = sv.config1_requests(arr, seed=int(rate))
        server = sv.ScfServer(xc, cfg, max_inflight=16, max_batch=1024)
        done = server.serve(reqs)
        s = sv.latency_summary(done)
        s["launches"] = server.launches
        out[f"served_rate_{int(rate)}"] = s
    arr = sv.poisson_arrivals(args.plain_rate, args.plain_seconds, seed=7)
    done = sv.serve_plain(xc, cfg, sv.config1_requests(arr, seed=7))
    out[f"plain_rate_{int(args.plain_rate)}"] = sv.latency_summary(done)
    if args.mix_rates:
        out["mix"] = run_serving_mix(args, xc, cfg)
    return out


def run_serving_mix(args, xc, cfg):
    """Config-5 mix: 80% plain-configuration 1D requests, 20% 3D SCF requests
    (numint LDA + factored Coulomb + DIIS, 30 cycles) over a pool of resident
    synthetic molecules, each replaying its captured CUDA graph; beside it the
    plain one-at-a-time form (3D through host-launched kernels)."""
    from qex_gb300 import serving as sv
    from qex_gb300.td import graph, workloads

    pool = {f"m{na}_{sd}": workloads.synthetic_molecule(na, seed=sd)
            for na, sd in ((1, 11), (2, 12), (3, 13), (4, 14))}
    graphs = {k: graph.CapturedScf(m, max_cycle=30) for k, m in pool.items()}
    out = {"workload": "Poisson stream, 80% 1D requests as above, 20% 3D SCF requests over "
                       "4 resident synthetic molecules (nao " +
                       ",".join(str(m.nao) for m in pool.values()) + "), LDA exchange, "
                       "factored Coulomb, DIIS, 30 cycles",
           "resident_3d_bytes": int(sum(g.nbytes for g in graphs.values()))}
    keys = list(pool)
    for rate in args.mix_rates:
        arr = sv.poisson_arrivals(rate, args.serving_seconds, seed=int(rate) + 1)
        reqs = sv.mixed_requests(arr, keys, frac3d=0.2, seed=int(rate) + 1)
        server = sv.ScfServer(xc, cfg, max_inflight=16, max_batch=1024, graphs3d=graphs)
        done = server.serve(reqs)
        s = sv.latency_summary(done)
        s["launches"] = server.launches
        out[f"served_rate_{int(rate)}"] = s
    rate = min(args.mix_rates)
    arr = sv.poisson_arrivals(rate, args.plain_seconds, seed=17)
    done = sv.serve_plain(xc, cfg, sv.mixed_requests(arr, keys, frac3d=0.2, seed=17),
                          molecules3d=pool, max_cycle=30)
    out[f"plain_rate_{int(rate)}"] = sv.latency_summary(done)
    return out


def run_serve_eval(args):
    """The serving configuration as specified: Poisson streams of
    ``--serve-seconds`` (default 60 s) at each rate of ``--serve-rates``
    (default 100 ... 5000 req/s) mixing 80% plain-configuration 1D solves and
    20% 3D solves over a population of 64 synthetic molecules of nao 4-117
    (s/p basis), each arriving as a new molecule the first time (grid, AO
    values, analytic integrals and density fitting on the GPU, then the
    captured SCF graph: inside that request's latency); admission by free HBM;
    a stream is cut 10 s after its last arrival (requests still waiting are
    reported as unserved).
    Then the saturated capacity of the served and the plain forms for 1D
    requests (all arrivals at t = 0)."""
    import qex_gb300
    from qex_gb300 import serving as sv
    from qex_gb300.od import engine as eng
    from qex_gb300.td import workloads

    cfg = eng.SolveConfig(num_iterations=20, alpha=0.5, alpha_decay=0.9, num_mixing_iterations=1,
                          convention="local", stencil=3)
    xc = qex_gb300.LDAExpCoulomb()
    rng = np.random.default_rng(5)
    keys = [(int(rng.integers(2, 14)), 1000 + i) for i in range(64)]

    def build(key):
        return workloads.device_molecule(key[0], seed=key[1], points_per_atom=620)[0]

    out = {"workload": "Poisson mix, 80% 1D (513 points, H2-like, exp-Coulomb LDA, 3-point "
                       "kinetic, 20 iterations), 20% 3D SCF (LDA, DIIS 8, 30 cycles, stop rule) "
                       "over 64 molecules of 2-13 atoms, new molecules built inside the "
                       "request's latency; admission by free HBM",
           "seconds": args.serve_seconds}
    server = sv.ScfServer(xc, cfg, max_inflight=16, max_batch=1024, builder3d=build)
    server.serve(sv.mixed_requests(sv.poisson_arrivals(200, 0.2, seed=1), keys[:2], 0.5, seed=1))
    for rate in args.serve_rates:
        arr = sv.poisson_arrivals(rate, args.serve_seconds, seed=int(rate) + 11)
        reqs = sv.mixed_requests(arr, keys, frac3d=0.2, seed=int(rate) + 11)
        server = sv.ScfServer(xc, cfg, max_inflight=32, max_batch=1024, builder3d=build)
        # an overloaded stream is cut 10 s after its last arrival: what waits
        # then is reported as unserved
        done = server.serve(reqs, deadline=args.serve_seconds + 10.0)
        s = sv.latency_summary(done)
        s["launches"] = server.launches
        s["molecules_built"] = server.built3d
        out[f"served_rate_{int(rate)}"] = s
        del server
    # saturated capacity, 1D
    n_cap = 20000
    reqs = sv.config1_requests(np.zeros(n_cap), seed=3)
    server = sv.ScfServer(xc, cfg, max_inflight=16, max_batch=1024)
    t0 = time.perf_counter()
    server.serve(reqs)
    dt = time.perf_counter() - t0
    out["served_capacity_1d"] = {"requests": n_cap, "s": dt, "solves_per_s": n_cap / dt}
    n_plain = 300
    reqs = sv.config1_requests(np.zeros(n_plain), seed=4)
    t0 = time.perf_counter()
    sv.serve_plain(xc, cfg, reqs)
    dt = time.perf_counter() - t0
    out["plain_capacity_1d"] = {"requests": n_plain, "s": dt, "solves_per_s": n_plain / dt}
    out["capacity_ratio_1d"] = out["served_capacity_1d"]["solves_per_s"] / (n_plain / dt)
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return None
    mols = workload(args.batch, args.seed)
    params, _ = mlp_params(0)
    cores = host_cores()
    sample = min(args.cpu_sample, len(mols))
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_sample(mols, params, args.iters, min(cores, sample), cores)
    times, convs = [], []
    for s in range(args.steps):
        dt, cconv, cn, _ = cpu_sample(mols[s * 7 % max(1, len(mols) - sample):], params, args.iters,
                                   sample, cores)
        times.append(dt)
        convs.append(cconv)
    step_s = sum(times) / len(times)
    value = (sum(convs) / len(convs)) / step_s
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": "synthetic (seeded molecules, Glorot-init MLP from seed 0)",
        "config": {"workload": f"batched 1D KS-SCF sample of {sample} molecules per step "
                               f"(same generator as the GPU arm), {args.iters} iterations",
                   "parallelism": f"{cores} host processes"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{sample} molecules per step, reference algorithm restated "
                                   f"in NumPy FP64 (dense eigh)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--iters", type=int, default=25)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-ksr", action="store_true")
    ap.add_argument("--no-td", action="store_true", help="skip the 3D configuration")
    ap.add_argument("--td-only", action="store_true", help="time only the 3D configuration")
    ap.add_argument("--td-atoms", type=int, nargs="*", default=None,
                    help="restrict the 3D configuration to the molecules of these atom counts")
    ap.add_argument("--ksr-only", action="store_true",
                    help="time only the KSR SCF workload (profiling)")
    ap.add_argument("--ksr-eval", action="store_true",
                    help="time only the standalone KSR network evaluation (profiling)")
    ap.add_argument("--fermi-eval", action="store_true",
                    help="time only the Fermi-Dirac occupation search")
    ap.add_argument("--grid-eval", action="store_true",
                    help="time only the molecular grid build")
    ap.add_argument("--train-eval", action="store_true",
                    help="time only one training-loss value and gradient")
    ap.add_argument("--eigh-atoms", type=int, nargs="*", default=None,
                    help="restrict --eigh-eval to the molecules of these atom counts")
    ap.add_argument("--eigh-eval", action="store_true",
                    help="time the 3D generalized eigensolver at the configuration's basis sizes")
    ap.add_argument("--phase-eval", action="store_true",
                    help="the batched 1D step's time by phase (the kernel's clock64 timers)")
    ap.add_argument("--probe", action="store_true",
                    help="measure the FP64/FP32 FMA and FP64 tensor-core (DMMA) throughput")
    ap.add_argument("--ints-eval", action="store_true",
                    help="time only the analytic integrals and density fitting")
    ap.add_argument("--serve-eval", action="store_true",
                    help="the serving configuration as specified (60 s streams per rate)")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serve-rates", type=float, nargs="*",
                    default=[100.0, 200.0, 500.0, 1000.0, 2000.0, 5000.0])
    ap.add_argument("--serving-rates", type=float, nargs="*", default=[1000.0, 5000.0])
    ap.add_argument("--serving-seconds", type=float, default=1.0)
    ap.add_argument("--mix-rates", type=float, nargs="*", default=[100.0, 200.0])
    ap.add_argument("--plain-rate", type=float, default=50.0)
    ap.add_argument("--plain-seconds", type=float, default=1.0)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "ours" and world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    if args.probe:
        from qex_gb300 import _native

        _native.load()
        f64, f32 = _native.measure_fma_peak()
        d1, d2 = _native.measure_dmma_peak()
        print(json.dumps({"probe": {"fp64_fma_tflops": f64, "fp32_fma_tflops": f32,
                                    "dmma_m8n8k4_tflops": d1, "dmma_m16n8k16_tflops": d2}}),
              flush=True)
        return
    if args.serve_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"serve_eval": run_serve_eval(args)}), flush=True)
        return
    if args.td_only:
        from qex_gb300 import _native

        _native.load()
        peak64, peak32 = _native.measure_fma_peak()
        print(json.dumps({"numint_3d": run_td(args, peak64, peak32)}), flush=True)
        return
    if args.eigh_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"eigh_eval": run_eigh_eval(args)}), flush=True)
        return
    if args.phase_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"phase_eval": run_phase_eval(args)}), flush=True)
        return
    if args.ints_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"ints_eval": run_ints_eval(args)}), flush=True)
        return
    if args.train_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"train_eval": run_train_eval(args)}), flush=True)
        return
    if args.grid_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"grid_eval": run_grid_eval(args)}), flush=True)
        return
    if args.fermi_eval:
        from qex_gb300 import _native

        _native.load()
        print(json.dumps({"fermi_eval": run_fermi_eval(args)}), flush=True)
        return
    if args.ksr_only or args.ksr_eval:
        import torch

        from qex_gb300 import _native

        _native.load()
        if args.ksr_eval:
            print(json.dumps({"ksr_eval": run_ksr_eval(args)}), flush=True)
        else:
            peak64, peak32 = _native.measure_fma_peak()
            flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
            print(json.dumps({"ksr": run_ksr(args, peak64, peak32, flush)}), flush=True)
        return
    line = run_ours(args, rank, world) if args.impl == "ours" else run_reference(args, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)
    if args.impl == "ours" and world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
