#!/usr/bin/env python
"""Benchmark: Metropolis proposals/s of the fk_mc exact-diagonalisation path on GB300.

Workload (one line per run): cubic2d L=24 (N=576 sites), t=1, U=2,
mu_c=mu_f=1, beta=4, B independent chains with Bernoulli(0.5) f drawn from
per-chain seeds 34788+c. One step = one move_addremove proposal on every chain:
build H, full eigen-solve, logZ (compensated FP64), Metropolis decision.

  value : proposals/s of the headline path (mixed precision when built, else
          plain FP64), device-resident inputs (site indices and uniforms
          already in HBM), CUDA events on the library's stream, K timed steps.
  e2e   : the same through fkg_propose_accept with host buffers, one call per
          step, host->device and device->host copies inside the timed region.

Other fields: the plain-FP64 path's proposals/s and the ratio; F = -logZ/beta
relative error of the chains' final states against the CPU oracle; the FLOP
roofline of the dominant kernel (the Householder reduction: W_fwd = 4/3 N^3
flops per proposal times the chains of one launch, over the launch's
CUDA-event duration, against the measured dense bf16 tensor peak of
MEASURED_PEAKS.json; DRAM traffic per launch from the committed ncu capture),
with the other views of the same kernels (nominal FP32 / FP64 pipe rates, the
one-stage algorithm's matrix re-reads against HBM) as labelled context; the CPU
baseline (the oracle restatement of the reference path on all host cores);
`chebyshev`: the same chains and proposals with logZ from the reference's
Chebyshev expansion (cheb_moves; int(log N * 2.2) moments) instead of the
eigen-solve, with its logZ against the oracle's expansion; `rank1`: the
proposals' logZ by the rank-one update of the current FP64 eigen-decomposition
(O(N^2) per proposal, no counterpart in the reference), against the oracle's
re-solve; `measures`: measure_stiffness (with the conductivity on 64
frequencies) and measure_ipr for the B configurations, each including the
solve with eigenvectors, with the oracle's CPU stiffness of one configuration.

--impl reference times the reference path's CPU restatement (the reference
itself does not compile here: Eigen3, Boost.MPI, ALPSCore, ARPACK, FFTW,
gftools and HDF5 are absent) on all host cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

KIND, L, T_HOP, U, MU, BETA, SEED = "cubic2d", 24, 1.0, 2.0, 1.0, 4.0, 34788
N = L * L
# The headline metric: both arms (--impl ours / reference) print this string, unit and direction.
METRIC = "MC proposals/s at N=576: mixed+batched vs plain FP64 on GB300; dF error"
# Nominal GB300 pipe rates (context for the FLOP roofline; the roofline denominators are the measured peaks):
# FP32 FMA 152 SMs x 128 lanes x 2 flops x 2.07 GHz; FP64 and dense TF32 from NVIDIA's GB300 figures.
NOMINAL_TFLOPS = {"fp32_fma": 152 * 128 * 2 * 2.07e9 / 1e12, "fp64": 1.25, "tf32_dense": 1100.0}
W_FWD = 4.0 / 3.0 * N ** 3      # Householder tridiagonalisation flops per proposal
W_BT = 2.0 * N ** 3              # back-transformation X = Q Z flops per proposal
NB32 = 8                         # panel width of the FP32 reduction at N = 576 (tuning table)
# Compulsory matrix bytes of one FP32 reduction: the lower triangle of the
# m x m trailing matrix read by the matrix-vector product of every column, and
# read + written by the rank-2k update after every panel of NB32 columns.
A_BYTES = 4.0 * (sum(m * (m + 1) / 2 for m in range(2, N))
                 + sum(2 * m * (m + 1) / 2 for m in range(N - NB32, 2, -NB32)))


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--batch", type=int, default=256)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-uneven", action="store_true")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples taken during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def chain_seeds(B, rank=0):
    """Seeds of the B chains of one replica: rank r holds chains r*B .. r*B + B - 1 of the whole job, each
    seeded SEED + its global index (one reference MPI rank per chain, src/mc_metropolis.cpp:25)."""
    return [SEED + rank * B + c for c in range(B)]


def make_chains(B, rank=0):
    rng_f = [np.random.default_rng(s) for s in chain_seeds(B, rank)]
    f = np.stack([r.integers(0, 2, N) for r in rng_f]).astype(np.int32)
    return f


def reduce_replicas(dist, device, ms, e2e):
    """Whole-job figures of N replicas: the slowest rank's time (max over ranks) and the summed
    end-to-end throughput. No collective touches the data path; this runs once after the timed region."""
    if dist is None:
        return ms, e2e
    import torch
    t = torch.tensor([ms, e2e], dtype=torch.float64, device=device)
    m = t[:1].clone()
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    e = t[1:].clone()
    dist.all_reduce(e, op=dist.ReduceOp.SUM)
    return float(m.item()), float(e.item())


def cpu_baseline(threads, seconds):
    from oracle import oracle as O
    n, el = O.bench_proposals(KIND, L, BETA, U, MU, MU, SEED, threads, seconds)
    return n / el, n, el


def measured_peaks():
    """HBM copy bandwidth and dense bf16 tensor throughput of the GB300s (MEASURED_PEAKS.json),
    else the fallback figures of one earlier GB300 measurement."""
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "bf16_tflops_sustained": float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "of": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "of": "fallback"}


def traffic_per_launch(tag):
    """DRAM bytes per launch of a kernel as read from a committed ncu capture (profiles/traffic.txt holds
    dram__bytes_read.sum + dram__bytes_write.sum per launch of the capture named there); not measured by
    this run."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == tag:
            return float(parts[1])
    return None


def roofline(res, head, B):
    """FLOP roofline of the dominant kernel, the Householder reduction of the headline path: the
    algorithmic work of one launch (W_fwd = 4/3 N^3 flops per chain, B chains) over its mean CUDA-event
    duration (stage timers on the library's stream), against the dense bf16 tensor peak of
    MEASURED_PEAKS.json (the sustained figure: the kernel is timed inside a run of many steps). The
    other views are context: the same kernels against the nominal FP32 / FP64 pipe rates, the one-stage
    reduction's matrix re-reads against HBM, the back-transformation's FP32-equivalent rate."""
    pk = measured_peaks()
    peak = pk["bf16_tflops_sustained"]
    hr = res[head]
    red_ms, red_n = hr["stages"]["reduce"]
    red_s = red_ms / red_n * 1e-3 if red_n else None
    achieved = W_FWD * B / red_s / 1e12 if red_s else None
    f32 = head == "mixed"
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if achieved else None,
            "traffic": traffic_per_launch(f"sytrd_{'f32' if f32 else 'f64'}_B{B}"),
            "traffic_source": "ncu capture committed under profiles/ (dram__bytes_read.sum + dram__bytes_write.sum "
                              "per launch), not measured by this run",
            "kernel": "sytrd_v3<%s> (Householder reduction, one CTA per chain)" % ("float,8" if f32 else "double,4"),
            "flops_per_unit": W_FWD, "units_per_launch": B, "launch_ms": red_s * 1e3 if red_s else None,
            "peak_source": f"MEASURED_PEAKS.json bf16_tflops_sustained (of {pk['of']})"}
    other = []
    if achieved:
        pipe = "fp32_fma" if f32 else "fp64"
        other.append({"kernel": roof["kernel"], "view": f"against the nominal {pipe} pipe rate (not measured)",
                      "achieved": achieved, "peak": NOMINAL_TFLOPS[pipe], "unit": "TFLOP/s",
                      "frac": achieved / NOMINAL_TFLOPS[pipe]})
        if f32:
            other.append({"kernel": roof["kernel"], "view": "one-stage reduction's own matrix re-reads (every "
                          "column's matrix-vector product plus the rank-2k update per panel) against HBM; not "
                          "compulsory traffic", "achieved": A_BYTES * B / red_s / 1e9, "peak": pk["hbm_gbs"],
                          "unit": "GB/s", "frac": A_BYTES * B / red_s / 1e9 / pk["hbm_gbs"]})
    if "f64" in res and head != "f64":
        m, n = res["f64"]["stages"]["reduce"]
        if n:
            a64 = W_FWD * B / (m / n * 1e-3) / 1e12
            other.append({"kernel": "sytrd_v3<double,4> (plain FP64 path)", "view": "against the nominal FP64 "
                          "pipe rate (not measured)", "achieved": a64, "peak": NOMINAL_TFLOPS["fp64"],
                          "unit": "TFLOP/s", "frac": a64 / NOMINAL_TFLOPS["fp64"], "launch_ms": m / n})
    bt_ms, bt_n = hr["stages"].get("back", (0.0, 0))
    if bt_n:
        bt = W_BT * B / (bt_ms / bt_n * 1e-3) / 1e12
        other.append({"kernel": "back-transformation X = Q Z (3xTF32 on the tensor cores)",
                      "view": "FP32-equivalent work 2 N^3 per chain against the measured bf16 peak and the nominal "
                              "dense TF32 rate", "achieved": bt, "unit": "TFLOP/s", "peak": peak, "frac": bt / peak,
                      "frac_of_nominal_tf32_dense": bt / NOMINAL_TFLOPS["tf32_dense"]})
    roof["other_kernels"] = other
    return roof


def run_reference(args, rank):
    # rank 0 alone runs the CPU restatement; the other ranks exit without work
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    per_step = threads  # one proposal per running chain (one chain per host thread) per step
    done, el = O.bench_steps(KIND, L, BETA, U, MU, MU, SEED, threads, args.warmup, args.steps)
    v = done / el
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": "proposals/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"cubic2d L={L} N={N} t=1 U={U} mu=1 beta={BETA}, one proposal per host thread "
                               f"per step (running chains, warm-up proposals untimed)", "threads": threads},
        "cpu_baseline": {"value": v, "unit": "proposals/s", "cores": threads, "kind": "port",
                         "sample": f"{done} proposals ({per_step} per step) of cubic2d L=24 single-site flips"},
        "e2e": {"value": v, "unit": "proposals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def time_device_path(solver, torch, stream, f0, B, steps, warmup, dist, precision):
    """K timed proposal steps on device-resident inputs (one CUDA graph replay per step, as a user runs
    them), then K more steps with the per-stage event timers on (direct launches) for the stage split;
    those are not part of the timed figure."""
    solver.set_precision(precision)
    solver.chains_init(np.zeros(B, np.int32), f0.ravel(), U, MU, MU, BETA)
    g = torch.Generator(device="cuda").manual_seed(SEED)
    tot = 2 * steps + warmup
    with torch.cuda.stream(stream):
        site = torch.randint(0, N, (tot, B), dtype=torch.int32, device="cuda", generator=g)
        u = torch.rand((tot, B), dtype=torch.float64, device="cuda", generator=g)
        acc = torch.zeros((tot, B), dtype=torch.int32, device="cuda")
        dl = torch.zeros((tot, B), dtype=torch.float64, device="cuda")
    stream.synchronize()
    solver.propose_accept_device(warmup, site.data_ptr(), u.data_ptr(), acc.data_ptr(), dl.data_ptr())
    n0 = solver.launch_count()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    off = warmup * B
    solver.propose_accept_device(steps, site.data_ptr() + 4 * off, u.data_ptr() + 8 * off, acc.data_ptr() + 4 * off,
                                 dl.data_ptr() + 8 * off)
    e1.record(stream)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = solver.launch_count() - n0
    acc_rate = float(acc[warmup:warmup + steps].float().mean().item())
    # the stage split: the same number of steps again with the event timers on
    solver.profile(True)
    off = (warmup + steps) * B
    solver.propose_accept_device(steps, site.data_ptr() + 4 * off, u.data_ptr() + 8 * off, acc.data_ptr() + 4 * off,
                                 dl.data_ptr() + 8 * off)
    torch.cuda.synchronize()
    stages = {k: solver.stage_time(k) for k in ("reduce", "trieig", "back", "refine", "logz")}
    solver.profile(False)
    return ms, launches, stages, acc_rate


def time_e2e(solver, f0, B, steps, warmup, precision):
    """The headline path through the public host-buffer call fkg_propose_accept, one call per step: the
    step's site indices and uniforms go host -> device and its decisions and dlogZ come back inside the
    timed region. The same warm-up count as the device-resident leg."""
    solver.set_precision(precision)
    solver.chains_init(np.zeros(B, np.int32), f0.ravel(), U, MU, MU, BETA)
    rng = np.random.default_rng(SEED + 1)
    site = rng.integers(0, N, (steps + warmup, B)).astype(np.int32)
    u = rng.uniform(0, 1, (steps + warmup, B))
    for s in range(warmup):
        solver.propose_accept(site[s], u[s])
    t0 = time.perf_counter()
    for s in range(warmup, warmup + steps):
        acc, dl = solver.propose_accept(site[s], u[s])
    el = time.perf_counter() - t0
    return steps * B / el, (4 + 8) * B, (4 + 8) * B


C4 = [("cubic2d", 12), ("cubic2d", 16), ("cubic2d", 20), ("cubic2d", 24), ("cubic2d", 32), ("triangular", 12),
      ("triangular", 18), ("triangular", 24)]


def time_uneven(torch, stream, steps, warmup, B=1024):
    """Uneven batch: 1024 chains on cubic2d L in {12,16,20,24,32} and triangular L in {12,18,24}
    (N = 144..1024), U ~ U[0.5, 4], beta ~ U[1, 10], mu = U/2, mixed precision, persistent
    longest-first reduction, one CUDA graph per step."""
    import fk_mc_gb300
    s = fk_mc_gb300.Solver(max_n=1024, max_batch=B, precision="mixed")
    s.set_stream(stream.cuda_stream)
    rng = np.random.default_rng(SEED)
    ns = [s.set_lattice(i, k, Lk) for i, (k, Lk) in enumerate(C4)]
    ids = np.array([c % 8 for c in range(B)], np.int32)
    Uc, bc = rng.uniform(0.5, 4.0, B), rng.uniform(1.0, 10.0, B)
    f = np.concatenate([rng.integers(0, 2, ns[i]) for i in ids]).astype(np.int32)
    s.chains_init(ids, f, Uc, Uc / 2, Uc / 2, bc)
    tot = steps + warmup
    with torch.cuda.stream(stream):
        nmax = torch.tensor([ns[i] for i in ids], dtype=torch.int64, device="cuda")
        site = (torch.rand((tot, B), dtype=torch.float64, device="cuda") * nmax).to(torch.int32)
        u = torch.rand((tot, B), dtype=torch.float64, device="cuda")
        acc = torch.zeros((tot, B), dtype=torch.int32, device="cuda")
        dl = torch.zeros((tot, B), dtype=torch.float64, device="cuda")
    stream.synchronize()
    s.propose_accept_device(warmup, site.data_ptr(), u.data_ptr(), acc.data_ptr(), dl.data_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    off = warmup * B
    e0.record(stream)
    s.propose_accept_device(steps, site.data_ptr() + 4 * off, u.data_ptr() + 8 * off, acc.data_ptr() + 4 * off,
                            dl.data_ptr() + 8 * off)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    s.close()
    return {"proposals_per_s": steps * B / (ms * 1e-3), "ms_per_step": ms / steps, "chains": B,
            "n_range": [min(ns), max(ns)], "path": "mixed, persistent reduction, CUDA graph per step"}


def time_chebyshev(solver, torch, stream, f0, B, steps, warmup):
    """The same chains and proposals with logZ from the Chebyshev expansion (the reference's
    cheb_moves path): cheb_size = int(log(N) * 2.2) (even) moments on max(2 cheb_size, 10) points."""
    from oracle import chebyshev as C
    from oracle import oracle as O
    cs = int(math.log(N) * 2.2)
    cs += cs % 2
    G = max(2 * cs, 10)
    solver.set_chebyshev(cs, G)
    solver.set_method("chebyshev")
    try:
        ms, launches, _, acc_rate = time_device_path(solver, torch, stream, f0, B, steps, warmup, None, "f64")
        f, logz, _ = solver.chains_get()
        csr = O.lattice_csr(KIND, L, T_HOP)
        c = 0  # oracle's expansion of one chain's current configuration
        ref = C.calc_chebyshev(C.dense_h(csr, f[c * N:(c + 1) * N], U, MU), BETA, cs, G)["logZ"]
        err = abs(logz[c] - ref) / abs(ref)
    finally:
        solver.set_method("ed")
    return {"proposals_per_s": steps * B / (ms * 1e-3), "ms_per_step": ms / steps, "cheb_size": cs, "grid": G,
            "acceptance": acc_rate, "gpu_launches_per_step": launches / steps, "logZ_rel_err_vs_oracle": err,
            "path": "Lanczos bounds + ball-restricted exact moments (double-float) + coefficients (chebyshev.cu)"}


def time_rank1(solver, torch, stream, f0, B, steps, warmup):
    """Proposal evaluation by the rank-one update (fkg_rank1_logz_device): the same chains'
    single-site flips with the proposal spectrum from the current FP64 eigen-decomposition instead of
    a re-solve (no counterpart in the reference; the accept path re-solves). Times `steps` batches of
    B proposals with the eigenpairs resident in HBM."""
    from oracle import oracle as O
    solver.set_precision("f64")
    out = solver.eigh_logz(np.zeros(B, np.int32), (-MU + U * f0).ravel().astype(float), BETA, vectors=True)
    rng = np.random.default_rng(SEED + 2)
    sites = rng.integers(0, N, (steps + warmup, B))
    ev = out["evals"].reshape(B, N)
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a), device="cuda")
    d_ev = dev(ev)
    zs = [dev(np.stack([out["evecs"][c][sites[k, c]] for c in range(B)])) for k in range(steps + warmup)]
    rhos = [dev(np.where(f0[np.arange(B), sites[k]] == 0, U, -U).astype(float)) for k in range(steps + warmup)]
    d_beta = dev(np.full(B, BETA))
    d_lz = torch.zeros(B, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for k in range(warmup):
        solver.rank1_logz_device(B, N, d_ev.data_ptr(), zs[k].data_ptr(), rhos[k].data_ptr(), d_beta.data_ptr(),
                                 d_lz.data_ptr())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(warmup, warmup + steps):
        solver.rank1_logz_device(B, N, d_ev.data_ptr(), zs[k].data_ptr(), rhos[k].data_ptr(), d_beta.data_ptr(),
                                 d_lz.data_ptr())
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    lz = d_lz.cpu().numpy()
    errs = []
    for c in (0, B - 1):   # the last timed batch against the oracle's re-solve of the flipped configuration
        g = f0[c].copy()
        g[sites[-1, c]] ^= 1
        ref = O.calc_ed(KIND, L, g, BETA, U, MU)["logZ"]
        errs.append(abs(lz[c] - ref) / abs(ref))
    return {"proposals_per_s": steps * B / (ms * 1e-3), "ms_per_batch": ms / steps, "logZ_rel_err_vs_oracle": max(errs),
            "path": "secular-equation roots after deflation (rank1.cu): FP32 pole-model iteration + "
                    "double-float finish; "
                    "eigenpairs from the FP64 path; an accepted proposal needs a re-solve with vectors"}


def time_measures(solver, f0, B, reps=2):
    """measure_stiffness (with a 64-point conductivity grid) and measure_ipr on the B chains'
    configurations through the host-buffer API (each call includes the eigen-solve with eigenvectors,
    calc_ed(true)) on the mixed path, timed on the host clock; accuracy against the oracle's stiffness of
    one configuration for both paths (the stiffness is a near-cancellation of two O(1) sums, so the mixed
    path's FP32 eigenvectors leave an absolute error near 1e-7 of those sums); CPU time of the oracle's
    stiffness for that configuration beside it."""
    from oracle import oracle as O
    solver.set_stiffness_ops(0, KIND, L, T_HOP)
    ids = np.zeros(B, np.int32)
    diag = (-MU + U * f0).ravel().astype(float)
    wgrid = np.linspace(-4.0, 4.0, 64)
    solver.set_precision("f64")
    st64 = solver.measure_stiffness(ids[:1], diag[:N], BETA)
    solver.set_precision("mixed")
    solver.measure_stiffness(ids, diag, BETA, wgrid, 0.05)  # warm
    t0 = time.perf_counter()
    for _ in range(reps):
        st, _ = solver.measure_stiffness(ids, diag, BETA, wgrid, 0.05)
    t_st = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        solver.measure_ipr(ids, diag, BETA)
    t_ipr = (time.perf_counter() - t0) / reps
    c0 = time.perf_counter()
    ref = O.stiffness(L, T_HOP, U, BETA, f0[0])
    cpu_s = time.perf_counter() - c0
    return {"stiffness_per_s": B / t_st, "ipr_per_s": B / t_ipr,
            "ms_per_batch": {"stiffness": t_st * 1e3, "ipr": t_ipr * 1e3},
            "stiffness": {"oracle": ref, "f64_rel_err": abs(st64[0] - ref) / abs(ref),
                          "mixed_abs_err": abs(st[0] - ref)},
            "cpu_oracle_stiffness_s": cpu_s,
            "path": "calc_ed(true) + measures.cu, host buffers, mixed path timed on the host clock"}


def free_energy_error(solver, B, sample=3):
    from oracle import oracle as O
    f, logz, _ = solver.chains_get()
    errs = []
    for c in np.linspace(0, B - 1, sample).astype(int):
        ref = O.calc_ed(KIND, L, f[c * N:(c + 1) * N], BETA, U, MU)
        F_ref, F = -ref["logZ"] / BETA, -logz[c] / BETA
        errs.append(abs(F - F_ref) / abs(F_ref))
    return max(errs)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import fk_mc_gb300
    from fk_mc_gb300 import _lib
    B = args.batch
    solver = fk_mc_gb300.Solver(max_n=N, max_batch=B)
    solver.set_lattice(0, KIND, L, T_HOP)
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    f0 = make_chains(B, rank)

    precisions = ["f64", "mixed"]
    head = "mixed"

    clocks = ClockSampler(local)
    clocks.start()
    res = {}
    for prec in precisions:
        ms, launches, stages, acc_rate = time_device_path(solver, torch, stream, f0, B, args.steps, args.warmup,
                                                          dist, prec)
        ms, _ = reduce_replicas(dist, "cuda", ms, 0.0)
        res[prec] = {"ms": ms, "launches": launches, "stages": stages, "acc": acc_rate,
                     "pps": args.steps * B * world / (ms * 1e-3)}
        res[prec]["dF_rel_err"] = free_energy_error(solver, B)
    cheb = time_chebyshev(solver, torch, stream, f0, B, args.steps, args.warmup) if world == 1 else None
    rank1 = time_rank1(solver, torch, stream, f0, B, args.steps, args.warmup) if world == 1 else None
    measures = time_measures(solver, f0, B) if world == 1 else None
    clk = clocks.stop()
    uneven = time_uneven(torch, stream, max(2, args.steps // 3), 2) if not args.no_uneven else None
    e2e, h2d, d2h = time_e2e(solver, f0, B, args.steps, args.warmup, head)
    _, e2e = reduce_replicas(dist, "cuda", 0.0, e2e)

    hr = res[head]
    roof = roofline(res, head, B)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, n, el = cpu_baseline(threads, args.cpu_seconds)
        cpu = {"value": v, "unit": "proposals/s", "cores": threads, "kind": "port",
               "sample": f"{n} single-site-flip proposals of cubic2d L=24 in {el:.1f} s, one chain per thread"}
    if rank == 0:
        stage_ms = {p: {k: round(v[0] / args.steps, 3) for k, v in res[p]["stages"].items() if v[1]} for p in res}
        out = {
            "metric": METRIC,
            "value": hr["pps"], "unit": "proposals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": hr["ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if head == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": f"cubic2d L={L} (N={N}) t=1 U={U} mu_c=mu_f={MU} beta={BETA}, {B} chains, "
                                   f"one single-site-flip proposal per chain per step", "chains_per_gpu": B,
                       "path": head, "parallelism": f"replicas x{world}",
                       "l2": "per-step working set (dense workspace of all chains) larger than L2"},
            "f64_value": res["f64"]["pps"],
            "mixed_over_f64": (res["mixed"]["pps"] / res["f64"]["pps"]) if "mixed" in res else None,
            "dF_rel_err": {p: res[p]["dF_rel_err"] for p in res},
            "acceptance": {p: res[p]["acc"] for p in res},
            "stage_ms_per_step": stage_ms,
            "uneven_batch": uneven,
            "chebyshev": cheb,
            "rank1": rank1,
            "measures": measures,
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "proposals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": hr["launches"],
            "clocks": clk,
        }
        print(json.dumps(out), flush=True)
    solver.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
