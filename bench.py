"""Benchmark: Krylov steps/s of pyprop's PamPropagator step on GB300.

Workload (default): hydrogen in a velocity-gauge sin^2 pulse at scale,
l = 0..63 x 1000 B-splines (order 7, exponential-linear breakpoints to 400 a.u.),
complex128, pAMP m = 30, dt = 0.005 -- pyprop_gb300/configs/hydrogen_velocity_large.ini.
Inputs are synthetic (seeded complex Gaussian coefficients, random-free operator).

One bench "step" = one PamPropagator.AdvanceStep (psi <- U^-1 pAMP(U psi)).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|fp32-mixed]
    python bench.py --impl reference ...     # CPU restatement of the reference, host cores

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "large": os.path.join(ROOT, "pyprop_gb300", "configs", "hydrogen_velocity_large.ini"),
    "small": os.path.join(ROOT, "pyprop_gb300", "configs", "hydrogen_velocity_small.ini"),
}
METRIC = "Krylov steps/s (pAMP x TensorPotential step, 1 GB300)"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# FMA issue rates measured on GB300 with dependency-free FMA loops over all SMs
FP64_PEAK_TFLOPS = 1.195
FP32_PEAK_TFLOPS = 69.9
# DRAM bytes (read + write) per launch of each step phase's kernel on the large workload,
# from one ncu capture of that kernel (capture constants, not measured by this run; the
# capture each comes from is named in PHASE_TRAFFIC_SOURCE)
PHASE_TRAFFIC = {
    ("fp64", "band"): 20802560, ("fp32-mixed", "band"): 20300288,
    ("fp64", "solve"): 1408256, ("fp32-mixed", "solve"): 826000,
    ("fp64", "gram_schmidt"): 16416768, ("fp32-mixed", "gram_schmidt"): 8750336,
}
PHASE_TRAFFIC_SOURCE = {
    "band": "profiles/band_kernel_hydrogen_large.md (ncu, dram__bytes_read/write.sum, one launch)",
    "solve": "profiles/k_solve_inv_fp64_hydrogen_large.md, profiles/k_solve_mixed_hydrogen_large.md "
             "(ncu --set full, one launch; the inverse band and the factor stay in L2)",
    "gram_schmidt": "profiles/k_arnoldi_cgs_hydrogen_large.md, profiles/k_arnoldi_cgs32_hydrogen_large.md "
                    "(ncu --set full, Arnoldi step J = 14)",
}
GOLD_LARGE = os.path.join(ROOT, "tests", "golden", "oracle_large.npz")


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._proc = None
        self._thr = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                           "--format=csv,noheader,nounits", "-lms", "200"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return

        def reader():
            for line in self._proc.stdout:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 8:
                    self.samples.append(parts)

        self._thr = threading.Thread(target=reader, daemon=True)
        self._thr.start()

    def stop(self):
        if self._proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self._proc.terminate()
        try:
            self._proc.wait(timeout=2)
        except Exception:
            self._proc.kill()
        if self._thr:
            self._thr.join(timeout=1)
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[4 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def load_peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def algorithmic_bytes(N, m, s, coef_bytes):
    """Per matvec: 2*N*s + B_coef; per Krylov step: s*N*(m^2 + 7m + 3) + m*B_coef."""
    return 2 * N * s + coef_bytes, s * N * (m * m + 7 * m + 3) + m * coef_bytes


def fp64_ops_per_step(N, nr, m, kd, nterms, kb):
    """Algorithmic FP64 FMA-pipe operations (thread instructions) of one FP64 Krylov step: band
    matvec (2 per real coefficient and complex element, 4 per term factor and element), classical
    Gram-Schmidt (4 per complex product in the dots and in the update, 2 per element of each norm),
    the last refinement residual of the 2m overlap-factor solves (2 per band entry and 2 adds per
    element), and the combination (4 per basis vector and element).  The exponential (m^3 per
    product) is below 1%."""
    W = 2 * kb + 1
    band = m * nterms * nr * (2 * W + 4)
    gs = N * (4 * m * (m + 1) + 2 * m)
    solves = 2 * m * N * (2 * (kd + 1) + 2)
    combine = 4 * m * N
    return band + gs + solves + combine


def operator_slots(prob):
    """(band slots, terms) of the device operator: one real band per stored angular
    slot and non-zero part (real / imaginary) of each consolidated TensorPotential."""
    nslots = 0
    nterms = 0
    nl = prob.psi.GetRepresentation().angular.count
    for p in prob.Propagator.BasePropagator.PotentialList:
        parts = int(np.any(p.PotentialData.real != 0)) + int(np.any(p.PotentialData.imag != 0))
        nslots += parts * p.PotentialData.shape[0]
        nterms += parts * (nl if p.GetStorageIds()[0] == "Ident" else p.PotentialData.shape[0])
    return nslots, nterms


def inverse_band_width(prob):
    """Band width w of the approximate inverse of the overlap factor the solves apply
    (same rule as the runtime: the dropped tail of every row below 2^-26 of the row)."""
    rad = prob.psi.GetRepresentation().radial
    n, kd = rad.count, rad.kd
    Ub = rad.cholesky_band()
    U = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - kd), j + 1):
            U[i, j] = Ub[j * (kd + 1) + kd + i - j]
    Ui = np.abs(np.linalg.inv(U))
    W = min(n - 1, 160)
    diag = np.stack([np.concatenate([np.diag(Ui, j), np.zeros(j)]) for j in range(W + 1)])
    tot = diag.sum(0)
    tail = np.cumsum(diag[::-1], axis=0)[::-1]           # tail[j] = sum_{j' >= j}
    w = W
    for j in range(W, 0, -1):
        if (tail[j] / np.where(tot > 0, tot, 1)).max() > 2.0 ** -26:
            break
        w = j - 1
    return w


def coef_bytes_of(prob, precision):
    """Operator bytes one balanced matvec reads once: the real band slots (FP64, or FP32
    hi + lo for the mixed path: 8 bytes per coefficient either way) and, per solve, the
    approximate-inverse band (FP32) and the factor's diagonals (FP64, or FP32 hi + lo)."""
    rad = prob.psi.GetRepresentation().radial
    nr, kd = rad.count, rad.kd
    nslots, _ = operator_slots(prob)
    band = nslots * (2 * kd + 1) * nr * 8
    w = inverse_band_width(prob)
    solve = 2 * ((w + 1) * nr * 4 + (kd + 1) * nr * 8)
    return band, solve, w


def phase_bytes(N, nr, m, s, band_coef, solve_tab, state_elem):
    """Algorithmic bytes of one step per phase (each array read or written once per launch):
      solve         m U^-1 launches: read r, write U^-1 r and the basis row v_J (3 N s) + tables;
                    m U^-T launches: read, write (2 N s) + tables; the state transform U^-1 x:
                    read x (16 N), write psi (N state_elem) + tables
      band          m launches: read the source, write the result (2 N s) + the band slots
      gram_schmidt  launch J reads v_0..v_J and w, writes w: (J + 3) N s; plus ||x|| (16 N)
      combine       read the m basis rows, read and write x (FP64): m N s + 32 N
      other         x = U psi: read psi, write x (FP64)
    solve_tab = bytes of one solve's tables (approximate-inverse band FP32 + factor diagonals)."""
    return {
        "solve": m * (3 * N * s + solve_tab) + m * (2 * N * s + solve_tab) + (16 * N + N * state_elem + solve_tab),
        "band": m * (2 * N * s + band_coef),
        "gram_schmidt": sum((J + 3) * N * s for J in range(m)) + 16 * N,
        "exponential": 0,
        "combine": m * N * s + 32 * N,
        "other": N * state_elem + 16 * N,
    }


def phase_roofline(h, psi_dev, scaling, dt, N, nr, m, elem, band_coef, solve_coef, precision, peak, peak_kind,
                   reps=5):
    """Per-phase times of the step (gbprop_time_step: one step outside its graph, an event after
    every launch, averaged over `reps` steps after one warm-up) against each phase's algorithmic
    bytes; the roofline entry of the line is the phase with the largest share of the step."""
    h.time_step(psi_dev, scaling, dt)
    acc = None
    for _ in range(reps):
        t = h.time_step(psi_dev, scaling, dt)
        if acc is None:
            acc = {k: [v[0], v[1]] for k, v in t.items() if isinstance(v, tuple)}
            acc["total_ms"] = t["total_ms"]
        else:
            for k, v in t.items():
                if isinstance(v, tuple):
                    acc[k][0] += v[0]
            acc["total_ms"] += t["total_ms"]
    total = acc.pop("total_ms") / reps
    pb = phase_bytes(N, nr, m, elem, band_coef, solve_coef // 2, elem)
    per = {}
    for name, (ms, cnt) in acc.items():
        ms /= reps
        b = pb[name]
        ent = {"ms_per_step": ms, "share": ms / total if total else 0.0, "launches_per_step": cnt,
               "algorithmic_bytes_per_step": b}
        if b and ms > 0:
            ach = b / (ms * 1e-3) / 1e9
            ent.update({"achieved": ach, "frac": ach / peak})
        tr = PHASE_TRAFFIC.get((precision, name))
        if tr is not None and cnt:
            ent["traffic_per_launch_capture"] = tr
        per[name] = ent
    top = max(per, key=lambda k: per[k]["ms_per_step"])
    return top, per, total


def build_problem(workload, precision, device):
    import pyprop_gb300 as pp
    conf = pp.Load(CONFIGS[workload])
    conf.Propagation.Set("krylov_precision", precision)
    prob = pp.Problem(conf, device=device)
    prob.SetupStep()
    return prob


def cost_stratified_sample(probs, k):
    """k problems spread over the batch's range of per-step work (evenly spaced in the order of
    N*(m^2+7m+3)), so that the sample's mean work per unit cost represents the whole batch."""
    order = sorted(range(len(probs)), key=lambda i: probs[i].N * (probs[i].m ** 2 + 7 * probs[i].m + 3))
    k = min(k, len(probs))
    return [probs[order[int(round(j * (len(order) - 1) / max(1, k - 1)))]] for j in range(k)]


def oracle_batch_rate(probs, budget_s, max_steps=3):
    """Oracle (CPU restatement, all host threads) batch steps/s of the whole batch: a
    cost-stratified sample of its problems is timed step by step (about budget_s in total), the
    time per unit of work N*(m^2+7m+3) is taken over the sample, and the rate is that time times
    the whole batch's work.  Returns (batch steps/s, description of the sample)."""
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    work = lambda p: p.N * (p.m * p.m + 7 * p.m + 3)
    sample = cost_stratified_sample(probs, 8)
    t_tot, w_tot, nsteps = 0.0, 0, 0
    t_start = time.perf_counter()
    for p in sample:
        pots = [dict(kind=orc.ORC_DIAG_BANDNH, data=p.static, pairs=None, timedep=False),
                dict(kind=orc.ORC_SIMP_BANDNH, data=p.dipole, pairs=p.pairs, timedep=True)]
        op = orc.Operator(p.nl, p.nr, p.kd, p.kb, p.cholesky_band().astype(np.complex128), pots)
        psi = p.initial_state()
        psi, _ = op.advance(psi, p.m, p.dt, [p.field(0.5)])             # warm
        for _ in range(max_steps):
            t0 = time.perf_counter()
            psi, _ = op.advance(psi, p.m, p.dt, [p.field(0.5)])
            t_tot += time.perf_counter() - t0
            w_tot += work(p)
            nsteps += 1
            if time.perf_counter() - t_start > budget_s:
                break
        if time.perf_counter() - t_start > budget_s:
            break
    batch_work = sum(work(p) for p in probs)
    rate = w_tot / t_tot / batch_work
    desc = ("%d Krylov steps of %d problems spread over the batch's range of per-step work (N*(m^2+7m+3)), "
            "time per unit work times the batch's work (oracle/oracle.c, OpenMP, %d threads)"
            % (nsteps, len(sample), threads))
    return rate, desc, threads


def run_reference_batch(args):
    """The batch workload on the CPU restatement: the same seeded problems, each advanced by the
    oracle on all host threads; a cost-stratified sample is timed and scaled to the batch's work."""
    from pyprop_gb300.batch import random_batch
    probs = random_batch(args.batch_size, seed=20261204)
    v, desc, threads = oracle_batch_rate(probs, budget_s=30.0, max_steps=max(1, min(args.steps, 3)))
    line = {
        "impl": "reference", "metric": METRIC + ", batch", "value": v, "unit": "batch steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": "hydrogen_velocity_batch", "problems": len(probs), "precision": "fp64"},
        "cpu_baseline": {"value": v, "unit": "batch steps/s", "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": v, "unit": "batch steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference(args, rank, world):
    """CPU restatement of the reference step (oracle/), all host threads."""
    if rank != 0:
        return
    if args.workload == "batch":
        run_reference_batch(args)
        return
    if args.workload == "adjoint":
        print(json.dumps({"impl": "reference", "unavailable": "the reference computes no gradients (no adjoint "
                                                             "or derivative of the propagation)"}), flush=True)
        return
    import pyprop_gb300 as pp
    from oracle import oracle as orc
    conf = pp.Load(CONFIGS[args.workload])
    prob = pp.Problem(conf, device="cpu")
    prob.SetupWavefunction()
    op = orc.Operator.from_problem(prob)
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    psi = prob.psi.GetDataNumpy().astype(np.complex128)
    m = prob.Propagator.BasisSize
    dt = prob.TimeStep
    bp = prob.Propagator.BasePropagator
    t = prob.PropagatedTime
    for _ in range(args.warmup):
        psi, _ = op.advance(psi, m, dt, [bp._scaling(t)])
        t = prob._next_time(t)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        psi, _ = op.advance(psi, m, dt, [bp._scaling(t)])
        t = prob._next_time(t)
    el = time.perf_counter() - t0
    v = args.steps / el
    nl, nr = prob.psi.GetRepresentation().GetFullShape()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": {"workload": "hydrogen_velocity_%s" % args.workload, "nl": nl, "nr": nr, "order": 7, "m": m,
                   "dt": dt.real, "precision": "fp64"},
        "cpu_baseline": {"value": v, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": "%d full Krylov steps of the workload (oracle/oracle.c, OpenMP)" % args.steps},
        "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(workload, budget_s=12.0):
    """Oracle steps/s on the host cores, on a bounded sample of the same workload."""
    import pyprop_gb300 as pp
    from oracle import oracle as orc
    conf = pp.Load(CONFIGS[workload])
    prob = pp.Problem(conf, device="cpu")
    prob.SetupWavefunction()
    op = orc.Operator.from_problem(prob)
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    psi = prob.psi.GetDataNumpy().astype(np.complex128)
    m, dt = prob.Propagator.BasisSize, prob.TimeStep
    psi, _ = op.advance(psi, m, dt, [0.0])          # warm
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s and n < 2000:
        psi, _ = op.advance(psi, m, dt, [0.0])
        n += 1
    el = time.perf_counter() - t0
    # the same restatement on one thread (a few steps of the workload, bounded)
    orc.set_threads(1)
    n1, t1 = 0, time.perf_counter()
    while time.perf_counter() - t1 < budget_s / 3 and n1 < 200:
        psi, _ = op.advance(psi, m, dt, [0.0])
        n1 += 1
    el1 = time.perf_counter() - t1
    orc.set_threads(threads)
    return {"value": n / el, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": "%d Krylov steps of the workload in %.1f s (oracle/oracle.c, OpenMP)" % (n, el),
            "single_thread": {"value": n1 / el1, "unit": "steps/s", "cores": 1,
                              "sample": "%d Krylov steps in %.1f s" % (n1, el1)},
            "host": host_cpu()}


def host_cpu():
    """The host's CPU model and core count (as the OS reports them)."""
    import platform
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":", 1)[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return {"model": model or platform.processor() or platform.machine(), "machine": platform.machine(),
            "nproc": os.cpu_count()}


def run_batch(args, rank, world, local, emit=True):
    """256 seeded uneven hydrogen-like problems advanced together (one graph launch per batch step).
    Prints the line (rank 0) when `emit`, and returns it."""
    import torch
    from pyprop_gb300 import _native
    from pyprop_gb300.batch import BatchPropagator, gather_states, random_batch, shard
    device = "cuda:%d" % local
    torch.cuda.set_device(local)
    prec = _native.FP64 if args.precision == "fp64" else _native.FP32_MIXED
    t0 = time.perf_counter()
    # one seeded batch; rank r advances its share of it (greedy bin-packing by per-step work)
    full = random_batch(args.batch_size, seed=20261204, setup="gpu")   # radial matrices formed on the GPU
    mine = shard(full, world)[rank]
    probs = [full[i] for i in mine]
    bp = BatchPropagator(probs, precision=prec, autotune=True, device=device)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    flush = torch.empty(args.flush_mb * (1 << 20) // 4, dtype=torch.float32, device=device)
    for _ in range(args.warmup):
        bp.advance(1)
    torch.cuda.synchronize()
    _barrier(world)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = _native.launch_count()
    for k in range(args.steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        bp.advance(1)
        ends[k].record(stream)
    torch.cuda.synchronize()
    _barrier(world)
    launches = _native.launch_count() - launches0
    ms = _max_over_ranks(sum(s_.elapsed_time(e) for s_, e in zip(starts, ends)), world)
    clk = clocks.stop()
    P = len(full)
    value = args.steps / (ms / 1e3)              # whole-batch steps per second (all ranks together)
    # e2e: every problem's state from pinned host memory, one batch step, back to the host
    elem = 16 if prec == _native.FP64 else 8
    hosts = [x.detach().cpu().pin_memory() for x in bp.psi]
    _barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for h, d in zip(hosts, bp.psi):
            d.copy_(h, non_blocking=True)
        bp.advance(1)
        for h, d in zip(hosts, bp.psi):
            h.copy_(d, non_blocking=True)
        torch.cuda.synchronize()
    e2e_s = _max_over_ranks(time.perf_counter() - t0, world)
    nbytes = sum(x.numel() for x in bp.psi) * elem
    N_tot = sum(p.N for p in full)
    B_step = sum(elem * p.N * (p.m * p.m + 7 * p.m + 3) for p in full)
    # the final states back in batch order on rank 0 (after the timed region)
    got = gather_states([x.detach().cpu().numpy() for x in bp.psi], mine, world, P)
    gathered = None if got is None else sum(1 for x in got if x is not None)
    line = {
        "metric": METRIC + ", batch", "value": value, "unit": "batch steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "c128" if prec == _native.FP64 else "c64+f64", "data": "synthetic",
        "config": {"workload": "hydrogen_velocity_batch", "problems": P, "elements": N_tot,
                   "precision": args.precision, "l2": "flushed between steps (%d MB write)" % args.flush_mb,
                   "setup_s": setup_s, "parallelism": "batch sharded over %d GPU(s) by per-step work, no "
                                                      "collective during propagation" % world,
                   "problems_on_rank0": len(mine), "states_gathered": gathered},
        "problem_steps_per_s": P * value,
        "e2e": {"value": args.steps / e2e_s, "unit": "batch steps/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "step_bytes": {"algorithmic_per_step": B_step, "achieved_GBps": B_step * value / world / 1e9},
        "clocks": clk, "gpu_launches": launches,
    }
    if rank == 0 and not args.no_cpu_baseline:
        v, desc, threads = oracle_batch_rate(full, budget_s=12.0)
        line["cpu_baseline"] = {"value": v, "unit": "batch steps/s", "cores": threads, "kind": "port",
                                "sample": desc}
    if rank == 0 and emit:
        print(json.dumps(line), flush=True)
    del bp
    torch.cuda.synchronize()
    return line


def batch_summary(args, rank, world, local):
    """The 256-problem batch in both precisions, a few timed steps each, for the default line
    (the full measurement is --workload batch)."""
    import copy
    out = {}
    for prec in ("fp64", "fp32-mixed"):
        a = copy.copy(args)
        a.precision, a.steps, a.warmup, a.no_cpu_baseline = prec, 5, 3, True
        b = run_batch(a, rank, world, local, emit=False)
        out[prec] = {k: b[k] for k in ("value", "unit", "ms_per_step", "problem_steps_per_s", "e2e", "gpu_launches")}
        out[prec]["setup_s"] = b["config"]["setup_s"]
    out["fp32_mixed_speedup_vs_fp64"] = out["fp32-mixed"]["value"] / out["fp64"]["value"]
    out["config"] = {"workload": "hydrogen_velocity_batch", "problems": args.batch_size, "steps": 5, "warmup": 3,
                     "l2": "flushed between steps (%d MB write)" % args.flush_mb}
    return out


def run_adjoint(args, rank, world, local):
    """Gradient of the final ground-state survival probability and of the total ionisation
    probability with respect to 64 piecewise-linear field samples (seeded ~N(0.05, 0.01)):
    l = 0..31 x 400 B-splines (linear breakpoints to 200 a.u.), m = 20, 1000 steps, forward
    checkpoints every 50 steps.

    timing (dt = 0.01): gradients/s in complex128 and complex64.  At this step the pAMP map
    is numerically chaotic on this basis (||dt H_m|| reaches ~2^11; a 1e-16 relative change
    of the initial state moves the survival probability by ~1e-5), which the line reports as
    `forward_map_sensitivity`; finite differences cannot check a gradient there.
    fd_check (dt = 0.0002, same sizes, where the discrete map is smooth): central
    differences (h = 1e-6, 1e-5, 1e-4) against the adjoint, each beside the rounding noise of
    the forward map at that h (the spread of two quotients at h and 1.001 h); the Taylor
    remainder O(c + h d) - O(c) - h g.d, whose order 2 checks the gradient below that noise;
    and the complex64 gradient against complex128."""
    if rank != 0:
        return
    import torch
    from pyprop_gb300 import _native
    from pyprop_gb300.adjoint import AdjointPropagator, bound_states
    from pyprop_gb300.batch import HydrogenProblem
    device = "cuda:%d" % local
    torch.cuda.set_device(local)
    nsteps, nsamples = 1000, 64
    rng = np.random.default_rng(20261205)
    c = rng.normal(0.05, 0.01, nsamples)

    def setup(dt):
        prob = HydrogenProblem(lmax=31, nr=400, rmax=200.0, m=20, dt=dt, seed=20261205)
        states, _, _ = bound_states(prob)
        return prob, states, states[0].reshape(prob.nl, prob.nr)

    prob, states, psi0 = setup(0.01)
    ground = states[:1]
    out = {"metric": "adjoint gradients/s (64 field samples, 1000 Krylov steps, 1 GB300)", "unit": "gradients/s",
           "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
           "config": {"workload": "hydrogen_adjoint", "nl": prob.nl, "nr": prob.nr, "rmax": 200.0, "m": prob.m,
                      "dt": 0.01, "steps": nsteps, "samples": nsamples, "checkpoint": 50,
                      "bound_states": int(len(states))}}
    for prec, name in ((_native.FP64, "c128"), (_native.FP32_MIXED, "c64")):
        ap = AdjointPropagator(prob, nsteps, nsamples, checkpoint=50, precision=prec, device=device)
        psi_T = ap.forward(psi0, c)                       # warm-up (graphs)
        ap.gradient(psi_T, ground)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        psi_T = ap.forward(psi0, c)
        ap.gradient(psi_T, ground)
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        t0 = time.perf_counter()
        psi_T = ap.forward(psi0, c, keep=False)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        out[name] = {"forward_s": t_fwd, "forward_plus_gradient_s": t_grad, "gradients_per_s": 1.0 / t_grad,
                     "gradient_over_forward": t_grad / t_fwd}
        if name == "c128":
            surv = ap.observable(psi_T, ground)
            pert = ap.observable(ap.forward(psi0 * (1 + 1e-16 * np.random.default_rng(1).standard_normal(psi0.shape)),
                                            c, keep=False), ground)
            out["forward_map_sensitivity"] = {"survival": surv, "d_survival_for_1e-16_relative_input_change":
                                              pert - surv}
    out["value"] = out["c128"]["gradients_per_s"]

    # --- finite-difference and precision check where the discrete map is smooth -------------
    dt_fd = 0.0002
    prob, states, psi0 = setup(dt_fd)
    ground = states[:1]
    res = {"dt": dt_fd}
    grads = {}
    for prec, name in ((_native.FP64, "c128"), (_native.FP32_MIXED, "c64")):
        ap = AdjointPropagator(prob, nsteps, nsamples, checkpoint=50, precision=prec, device=device)
        psi_T = ap.forward(psi0, c)
        g_s, _ = ap.gradient(psi_T, ground)
        g_b, _ = ap.gradient(ap.forward(psi0, c), states)
        grads[name] = (g_s, -g_b)
        if name == "c128":
            scale = float(np.abs(g_s).max())

            def O(x):
                return ap.observable(ap.forward(psi0, x, keep=False), ground)

            o0 = O(c)

            def fd_at(k, h):
                cp, cm = c.copy(), c.copy()
                cp[k] += h
                cm[k] -= h
                return (O(cp) - O(cm)) / (2 * h)

            # each difference quotient beside a second one at 1.001 h: their truncation errors
            # agree (h^2 times the third derivative, ~1e-15 relative here), so their spread is the
            # rounding noise of the 1000-step forward map at that h, the floor of any quotient
            for h in (1e-6, 1e-5, 1e-4):
                fd, spread = [], []
                for k in (5, 31, 58):
                    f1, f2 = fd_at(k, h), fd_at(k, 1.001 * h)
                    fd.append((f1, float(g_s[k])))
                    spread.append(abs(f1 - f2))
                res["survival_fd_h%.0e" % h] = {"samples": [5, 31, 58], "fd": [f for f, _ in fd],
                                                "adjoint": [a_ for _, a_ in fd],
                                                "max_rel_err": max(abs(f - a_) for f, a_ in fd) / scale,
                                                "noise_rel_from_spread": max(spread) / scale}
            # Taylor remainder along a seeded direction: second order in h with the adjoint gradient
            d = np.random.default_rng(3).standard_normal(nsamples)
            gd = float(g_s @ d)
            hs = (1e-2, 5e-3, 2.5e-3)
            rem = [abs(O(c + hh * d) - o0 - hh * gd) for hh in hs]
            res["taylor"] = {"h": list(hs), "remainder": rem,
                             "orders": [float(np.log2(a_ / b_)) for a_, b_ in zip(rem, rem[1:])]}
    a_, b_ = grads["c128"], grads["c64"]
    res["c64_vs_c128"] = {"survival_grad_rel_l2": float(np.linalg.norm(b_[0] - a_[0]) / np.linalg.norm(a_[0])),
                          "ionisation_grad_rel_l2": float(np.linalg.norm(b_[1] - a_[1]) / np.linalg.norm(a_[1]))}
    out["fd_check"] = res
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: 200 for a single problem, 20 for the 256-problem batch)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbprop", choices=["gbprop", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32-mixed"])
    ap.add_argument("--workload", default="large", choices=list(CONFIGS) + ["batch", "adjoint"])
    ap.add_argument("--batch-size", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--flush-mb", type=int, default=512)
    ap.add_argument("--no-mixed", action="store_true", help="skip the FP32-mixed arm of the default run")
    ap.add_argument("--no-precision-report", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batch summary of the default run")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 20 if args.workload == "batch" else 200
    args.warmup = max(args.warmup, 3)

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if args.impl == "gbprop" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "batch":
        run_batch(args, rank, world, local)
        return
    if args.workload == "adjoint":
        run_adjoint(args, rank, world, local)
        return

    import torch
    device = "cuda:%d" % local
    torch.cuda.set_device(local)
    main_arm = measure_single(args, args.precision, device, world, with_e2e=True)
    line = main_arm.pop("line")
    if args.precision == "fp64" and not args.no_mixed:
        mixed = measure_single(args, "fp32-mixed", device, world, with_e2e=True)["line"]
        line["fp32_mixed"] = {k: mixed[k] for k in ("value", "unit", "ms_per_step", "e2e", "roofline", "matvec_ms",
                                                    "gpu_launches", "parity_vs_oracle") if k in mixed}
        line["fp32_mixed"]["speedup_vs_fp64"] = mixed["value"] / line["value"]
        line["fp32_mixed"]["dtype"] = mixed["dtype"]
    if not args.no_precision_report:
        line["precision_report"] = precision_report(device)
    if world == 1 and not args.no_batch:
        line["batch"] = batch_summary(args, rank, world, local)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(args.workload)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def measure_single(args, precision, device, world, with_e2e=True):
    """One precision on the single-problem workload: device-resident steps/s (L2 flushed
    between steps), e2e through the C ABI with host buffers, the band kernel alone and the
    balanced matvec."""
    import torch
    from pyprop_gb300 import _native
    prob = build_problem(args.workload, precision, device)
    h = prob.Propagator.Handle()
    nl, nr = prob.psi.GetRepresentation().GetFullShape()
    N = nl * nr
    m = prob.Propagator.BasisSize
    elem = 16 if precision == "fp64" else 8
    dt = prob.TimeStep
    bp = prob.Propagator.BasePropagator
    psi0 = prob.psi.GetData().clone()
    local = torch.cuda.current_device()

    # --- device-resident timing: K steps, L2 flushed between steps ---------------------------
    flush = torch.empty(args.flush_mb * (1 << 20) // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        prob.AdvanceStep()
    torch.cuda.synchronize()
    _barrier(world)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = _native.launch_count()
    torch.cuda.synchronize()
    _barrier(world)
    for k in range(args.steps):
        flush.fill_(float(k))
        starts[k].record(stream)
        prob.AdvanceStep()
        ends[k].record(stream)
    torch.cuda.synchronize()
    _barrier(world)
    launches = _native.launch_count() - launches0
    sorder = int(h.stats().last_scaling_order)
    ms = sum(s_.elapsed_time(e) for s_, e in zip(starts, ends))
    clk = clocks.stop()
    ms = _max_over_ranks(ms, world)
    value = world * args.steps / (ms / 1e3)

    # --- e2e through the C ABI with host buffers (H2D psi, step, D2H psi per step) -----------
    e2e = None
    if with_e2e:
        psi_host = np.ascontiguousarray(prob.psi.GetDataNumpy())
        scal = np.array([bp._scaling(prob.PropagatedTime)])
        for _ in range(2):
            h.advance_host(psi_host, scal, dt)
        _barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            h.advance_host(psi_host, scal, dt)
        e2e_s = _max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": world * args.steps / e2e_s, "unit": "steps/s",
               "h2d_bytes_per_step": psi_host.nbytes, "d2h_bytes_per_step": psi_host.nbytes}

    # --- matvec alone: the tensor-potential kernel and the balanced matvec -------------------
    band_coef, solve_coef, w = coef_bytes_of(prob, precision)
    B_mv, B_step = algorithmic_bytes(N, m, elem, band_coef + solve_coef)
    src = psi0.clone()
    dst = torch.empty_like(src)
    # average launch duration over 100 back-to-back launches, CUDA events on the launching stream
    # (events around each launch would add their own gaps to a ~20 us kernel)
    reps = 100
    for balanced in (0, 1):
        for _ in range(5):
            h.matvec(src, dst, 0.1, balanced=bool(balanced))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            h.matvec(src, dst, 0.1, balanced=bool(balanced))
        e1.record(stream)
        torch.cuda.synchronize()
        if balanced:
            t_bal = e0.elapsed_time(e1) / reps
        else:
            t_band = e0.elapsed_time(e1) / reps
    peak, peak_kind = load_peaks()
    # per-phase roofline of the step (events between launches, outside the graph)
    scal0 = bp._scaling(prob.PropagatedTime)
    top, per_phase, phase_total = phase_roofline(h, src.clone(), scal0, dt, N, nr, m, elem, band_coef, solve_coef,
                                                 precision, peak, peak_kind)
    band_bytes = 2 * N * elem + band_coef
    achieved = band_bytes / (t_band * 1e-3) / 1e9
    _, nterms = operator_slots(prob)
    kd = prob.psi.GetRepresentation().radial.kd
    if precision == "fp64":
        # 2 FMA (4 flops) per real band entry per complex element
        band_flops = nterms * nr * (2 * kd + 1) * 4
        compute = {"unit": "TFLOP/s", "achieved": band_flops / (t_band * 1e-3) / 1e12, "peak": FP64_PEAK_TFLOPS,
                   "peak_source": "measured FP64 FMA issue rate on GB300", "what": "FP64 FMA"}
    else:
        # error-free products + compensated sums: ~22 FP32 ops per (hi, lo) band entry and component
        band_flops = nterms * nr * (2 * kd + 1) * 2 * 22
        compute = {"unit": "TFLOP/s", "achieved": band_flops / (t_band * 1e-3) / 1e12, "peak": FP32_PEAK_TFLOPS,
                   "peak_source": "measured FP32 FMA issue rate on GB300", "what": "FP32 ops of the compensated sums"}
    compute["frac"] = compute["achieved"] / compute["peak"]
    kernels = {"solve": "k_solve_inv (overlap-factor solves U^-1, U^-T)" if precision == "fp64" else
               "k_solve_mixed / k_solve_inv (complex64 basis solves, FP64 state solve)",
               "band": "k_band_apply (TensorPotentialMultiply, all terms)",
               "gram_schmidt": "k_arnoldi_cgs (cooperative Gram-Schmidt) + k_norm",
               "exponential": "k_expm_cluster (Pade scaling-and-squaring)",
               "combine": "k_combine", "other": "k_tbmv + step bookkeeping"}
    tp = per_phase[top]
    launches_top = max(1, tp["launches_per_step"])
    roofline = {
        "bound": "hbm", "kernel": kernels[top], "phase": top,
        "achieved": tp.get("achieved"), "peak": peak, "unit": "GB/s", "frac": tp.get("frac"),
        "peak_source": peak_kind,
        "traffic": PHASE_TRAFFIC.get((precision, top)),
        "traffic_source": PHASE_TRAFFIC_SOURCE.get(top) if (precision, top) in PHASE_TRAFFIC else None,
        "launch_ms": tp["ms_per_step"] / launches_top,
        "algorithmic_bytes_per_launch": tp["algorithmic_bytes_per_step"] / launches_top,
        "how": "gbprop_time_step: one step outside its CUDA graph with an event after every launch (5 steps "
               "averaged); achieved = the phase's algorithmic bytes per step / its time per step",
        "step_ms_events": phase_total,
        "per_phase": per_phase,
        "band_kernel_alone": {"achieved": achieved, "frac": achieved / peak, "launch_ms": t_band,
                              "algorithmic_bytes_per_launch": band_bytes,
                              "traffic": PHASE_TRAFFIC.get((precision, "band")), "compute": compute},
    }
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128" if precision == "fp64" else "c64+f64",
        "data": "synthetic",
        "config": {"workload": "hydrogen_velocity_%s" % args.workload, "nl": nl, "nr": nr, "order": 7, "m": m,
                   "dt": dt.real, "precision": precision, "l2": "flushed between steps (%d MB write)" % args.flush_mb,
                   "parallelism": "replicas" if world > 1 else "single", "inverse_band": w,
                   "band_variant": prob.Propagator.BandVariant, "expm_scaling_order": sorder,
                   "solve_chunks": list(h.tuning()[1])},
        "e2e": e2e,
        "roofline": roofline,
        "step_bytes": {"algorithmic_per_step": B_step, "achieved_GBps": B_step * value / world / 1e9,
                       "per_matvec": B_mv},
        "matvec_ms": {"band_apply": t_band, "balanced": t_bal},
        "clocks": clk,
        "gpu_launches": launches,
    }
    if precision == "fp64":
        # the FP64 step's own bound: FP64 FMA-pipe operations per step against the measured issue rate
        ops = fp64_ops_per_step(N, nr, m, kd, nterms, kd)
        line["step_fp64_roofline"] = {
            "fp64_ops_per_step": ops, "unit": "TFLOP/s (2 per FMA-pipe operation)",
            "achieved": 2 * ops * value / world / 1e12, "peak": FP64_PEAK_TFLOPS,
            "peak_source": "measured FP64 FMA issue rate on GB300",
            "frac": 2 * ops * value / world / 1e12 / FP64_PEAK_TFLOPS}
    par = parity_vs_fixture(args.workload, h, precision)
    if par is not None:
        line["parity_vs_oracle"] = par
        if precision == "fp64":
            line["exponential_precision"] = exponential_precision(h, dt)
    del h, prob
    torch.cuda.synchronize()
    return {"line": line}


def parity_vs_fixture(workload, h, precision):
    """The workload against the oracle's states (tests/golden/oracle_large.npz, same coefficients
    and field values), after the timed region.  From the hydrogen ground state: 20 steps (the
    field still weak, a smooth map: bar 1e-11 for FP64) and on to 200 steps, where the pulse has
    filled the stiff modes of the basis and the reference's algorithm itself amplifies rounding
    (the oracle's response to a seeded 1e-16 relative change of the start is reported beside
    each state; bar 30x that).  From the configured random start one step, whose stiff modes
    amplify rounding ~1e4-fold at once (same bar)."""
    if workload != "large" or not os.path.exists(GOLD_LARGE):
        return None
    import torch
    g = np.load(GOLD_LARGE)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    dt = complex(g["dt"])
    out = {"against": "oracle states (tests/golden/oracle_large.npz)"}
    d = torch.as_tensor(g["gs0"]).to("cuda", cdt)
    done = 0
    for n in (20, 200):
        h.advance(d, g["scalings"][done:n], dt)
        h.synchronize()
        done = n
        got = d.cpu().numpy().astype(np.complex128)
        want = g["gs%d" % n]
        sens = float(g["gs_sens%d" % n])
        out["ground_state_%d" % n] = {
            "steps": n, "rel_l2": float(np.linalg.norm(got - want) / np.linalg.norm(want)),
            "oracle_sensitivity_1e-16": sens,
            "bar": (1e-11 if n == 20 else 30.0 * sens) if precision == "fp64" else None}
    d = torch.as_tensor(g["psi0"]).to("cuda", cdt)
    h.advance(d, g["scalings"][:1], dt)
    h.synchronize()
    got = d.cpu().numpy().astype(np.complex128)
    sens = float(g["sens1"])
    out["random_start_1"] = {"steps": 1, "rel_l2": float(np.linalg.norm(got - g["rand1"]) / np.linalg.norm(g["rand1"])),
                             "oracle_sensitivity_1e-16": sens, "bar": 30.0 * sens if precision == "fp64" else None}
    return out


def exponential_precision(h, dt):
    """The three Hessenberg exponentials of the handle on the Hessenberg matrix of its last step:
    FP64 Pade, the double-float Pade of the FP32-mixed path and the eigenvector form, each against
    scipy's expm of the same -i dt H (pamp.h:634), column 0."""
    import scipy.linalg as sla
    dt = float(np.real(dt))
    H = 1j * h.hessenberg() / dt              # the step stores -i dt H; the kernels take H and dt
    want = sla.expm((-1j * dt) * H)[:, 0]
    out = {"m": int(H.shape[0]), "dt": dt, "norm_inf_dtH": float(dt * np.abs(H).sum(axis=1).max()),
           "against": "scipy.linalg.expm of the same -i dt H (column 0)"}
    ys = {}
    for form, name in ((0, "pade_fp64"), (1, "pade_double_float"), (2, "eigenvector_fp64")):
        y, so = h.debug_expm(H, dt, form)
        ys[form] = y
        out[name] = {"rel_l2": float(np.linalg.norm(y - want) / np.linalg.norm(want))}
        if form < 2:
            out[name]["scaling_order"] = so
    out["double_float_vs_fp64_rel_l2"] = float(np.linalg.norm(ys[1] - ys[0]) / np.linalg.norm(ys[0]))
    return out


def precision_report(device, nsteps=500):
    """FP32-mixed against FP64 on the hydrogen workload of the small configuration
    (l = 0..9 x 106 B-splines, m = 20, dt = 0.01, 500 steps): relative L2 of the final
    state, bound-state populations and ionisation, for the seeded random initial state
    of the workload and for the hydrogen ground state; beside each, two floors of FP64
    arithmetic with complex64 storage: the FP64 path with its band matvec outputs rounded to
    complex64, and with every Arnoldi vector rounded where the mixed path stores complex64
    (solve, band and Gram-Schmidt outputs)."""
    import torch
    import pyprop_gb300 as pp
    from pyprop_gb300 import observables as ob
    out = {"workload": "hydrogen_velocity_small", "steps": nsteps}
    probs = {}
    for prec in ("fp64", "fp32-mixed"):
        conf = pp.Load(CONFIGS["small"])
        conf.Propagation.Set("krylov_precision", prec)
        pr = pp.Problem(conf, device=device)
        pr.SetupStep()
        probs[prec] = pr
    p64 = probs["fp64"]
    states, _, _ = ob.problem_bound_states(p64)     # banded GPU eigensolver
    S = ob.radial_overlap(p64)
    bp = p64.Propagator.BasePropagator
    times, t = [], p64.PropagatedTime
    for _ in range(nsteps):
        times.append(t)
        t = p64._next_time(t)
    scal = np.array([bp._scaling(x) for x in times])
    from pyprop_gb300 import _native
    starts = {"random": p64.psi.GetDataNumpy().copy(), "ground": states[0].reshape(p64.psi.GetData().shape)}
    for name, psi0 in starts.items():
        res = {}
        for prec, rnd in (("fp64", 0), ("fp32-mixed", 0), ("floor_matvec", 1), ("floor_storage", 3)):
            pr = probs["fp64" if prec.startswith("floor") else prec]
            hd = pr.Propagator.Handle()
            dtp = torch.complex64 if prec == "fp32-mixed" else torch.complex128
            d = torch.as_tensor(np.ascontiguousarray(psi0)).to(device, dtp)
            hd.debug_set(_native.DEBUG_ROUND_MATVEC, rnd)
            hd.advance(d, scal, pr.TimeStep)
            hd.synchronize()
            hd.debug_set(_native.DEBUG_ROUND_MATVEC, 0)
            res[prec] = d.cpu().numpy().astype(np.complex128)
        a, b = res["fp64"], res["fp32-mixed"]
        r64, r32 = ob.report(a, states, S), ob.report(b, states, S)
        out[name] = {"rel_l2": float(np.linalg.norm(b - a) / np.linalg.norm(a)),
                     "complex64_matvec_floor_rel_l2": float(np.linalg.norm(res["floor_matvec"] - a) / np.linalg.norm(a)),
                     "complex64_storage_floor_rel_l2": float(np.linalg.norm(res["floor_storage"] - a) / np.linalg.norm(a)),
                     "max_abs_d_population": float(np.abs(r64["populations"] - r32["populations"]).max()),
                     "ionisation_fp64": r64["ionisation"], "ionisation_fp32_mixed": r32["ionisation"],
                     "bound_fp64": r64["bound"], "bound_fp32_mixed": r32["bound"]}
    return out


if __name__ == "__main__":
    main()
