#!/usr/bin/env python3
"""Benchmark of the Spectral2D time step on GB300.

Workload (one "step" = one TVD-RK3 step of the hot path): decaying 2-D
turbulence, N = 2048 (3072^2 collocation grid, 3/2 rule), FP64, nu = 1e-4,
dt from CFL 0.5 of the seeded initial condition (E(k) ~ k^4 exp(-2(k/10)^2),
total energy 0.5).  Metric: Mpt*steps/s = N^2 * steps/s / 1e6.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* ``value``: device-resident state, K steps replayed from a CUDA graph, timed
  with CUDA events on the solver's stream between two synchronisations.
* ``e2e``: the same metric through the C-ABI drop-in for the reference's
  IntegrateOneStep with host arrays (s2d_integrate_one_step_host): every step
  moves wC's retained modes in from page-locked host memory and wC, psiC out
  over the host link (the kernels read and write the host arrays in place).
* ``roofline``: the dominant kernel against the roof that binds it, from its
  CUDA-event launch time.  FP64: benchFFT flops per launch against the FP64
  FMA rate measured on this GPU (``bound: "fp64"``), with the HBM view
  (algorithmic bytes per launch over the measured copy bandwidth) nested as
  ``hbm``; FP32: the HBM view (``bound: "hbm"``).
* ``cpu_baseline``: the FP64 CPU restatement of the reference (scipy/pocketfft
  on all host cores, and on one core) timed on a bounded sample of the same
  workload.
* ``--impl reference``: that CPU restatement as the reference arm (the
  reference itself, Fortran + FFTW-MPI, cannot be built on these machines).

Multi-GPU: one process per GPU.  Under torchrun (or any launcher that sets
RANK / LOCAL_RANK / WORLD_SIZE / MASTER_ADDR / MASTER_PORT) each process is one
rank; ``python bench.py --gpus N`` without a launcher starts the N local ranks
itself with those variables set.  The headline DNS workload runs one
independent replica per rank (a single run does not shard): ``value`` is the
sum over ranks of the points x steps advanced over the slowest rank's time.
``--workload ensemble`` and ``les-batch`` split their runs over the ranks by
cost (replicas.shard_runs); ``value`` is all runs' work over the slowest
rank's time.  ``--dry-cpu`` runs only this rank logic over gloo on CPU, with
stand-in step times (tests/test_bench_cpu.py).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 2048
NU = 1e-4
CFL = 0.5
SEED = 0
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
# byte and flop model of one step (shared with the design notes)
# ---------------------------------------------------------------------------
def byte_model(n: int, wbytes: int, form: str = "basdevant") -> dict:
    """Compulsory HBM bytes of the fused two-pass step.
    I = (N/2+1)*M*w (half-spectral intermediate), S = (N/2+1)*(N+1)*w
    (compact state).
    Conservative form (the reference's): K1 reads S, writes 3I (u, v, w);
    K2 reads 3I, writes 2I; K3 reads 2I and 2S (stage input, w^n), writes S:
    B_rhs = 10I + 4S.
    Basdevant form: K1 writes 2I (u, v); K2 reads 2I, writes 2I:
    B_rhs = 8I + 4S."""
    m = 3 * n // 2
    I = (n // 2 + 1) * m * wbytes
    S = (n // 2 + 1) * (n + 1) * wbytes
    nf = 2 if form == "basdevant" else 3
    per = {"yinv": S + nf * I, "xpass": (nf + 2) * I, "yfwd": 2 * I + 3 * S}
    rhs = sum(per.values())
    return {"I": I, "S": S, "per_kernel": per, "rhs": rhs, "step": 3 * rhs,
            "step_reference_form": 3 * (10 * I + 4 * S)}


def flop_model(n: int, form: str = "basdevant") -> dict:
    """benchFFT convention: 2.5*M*log2(M) flops per real 1-D transform of
    length M, i.e. 2.5*M^2*log2(M) per field per direction of an M x M real
    2-D FFT.  Basdevant: K1 2 fields (y), K2 4 (x), K3 2 (y); conservative:
    3, 5, 2."""
    m = 3 * n // 2
    f = 2.5 * m * m * math.log2(m)
    a, b = (2, 4) if form == "basdevant" else (3, 5)
    return {"yinv": a * f, "xpass": b * f, "yfwd": 2 * f, "rhs": (a + b + 2) * f,
            "step": 3 * (a + b + 2) * f}


# ---------------------------------------------------------------------------
def read_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            with open(p) as f:
                return json.load(f)
        except Exception:
            return {}
    return {}


def hbm_peak(peaks: dict):
    for k in ("hbm_gbs", "hbm_GBs", "hbm_copy_gbs"):
        if k in peaks and peaks[k]:
            return float(peaks[k]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


def read_traffic(kernel: str, form: str, n: int, precision: str):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    from the committed ncu summary of that kernel, if there is one."""
    name = {"yinv": "yinv", "yfwd": "yfwd_rk3",
            "xpass": "xpass_bas" if form == "basdevant" else "xpass_rhs"}[kernel]
    p = os.path.join(ROOT, "profiles", f"{name}_n{n}_{precision}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if "traffic_bytes_per_launch" in line:
            digits = [c for c in line.split("|") if c.strip().isdigit()]
            if digits:
                return int(digits[0].strip())
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="s2d_clocks_", suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) < 9:
                    continue
                try:
                    sm.append(float(c[1]))
                    smax.append(float(c[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, c[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
def cpu_step_rate(n: int, steps: int, warmup: int, budget_s: float, cores: int | None = None,
                  min_steps: int = 5):
    """Time the oracle (FP64 CPU restatement) on all host cores (or on
    ``cores`` threads): ``warmup`` untimed steps, then steps timed one by one
    until ``steps`` or until ``budget_s`` seconds have passed after at least
    ``min_steps``.  Returns (Mpt*steps/s from the median step time, timed
    steps, cores, median seconds per step)."""
    import numpy as np
    import oracle as O
    cores = cores or O.cpu_count()
    O.set_workers(cores)
    g = O.get_grid_size(n, n)
    w, psi = O.set_turbulent(g, SEED, kind=O.SPECTRUM_K4_GAUSS, k0=10.0, tke_target=0.5)
    dt = O.cfl_dt(w, g, CFL)
    for _ in range(warmup):
        w, psi = O.integrate_one_step(w, psi, g, NU, dt)
    times, t0 = [], time.perf_counter()
    while len(times) < steps:
        t = time.perf_counter()
        w, psi = O.integrate_one_step(w, psi, g, NU, dt)
        times.append(time.perf_counter() - t)
        if len(times) >= min(min_steps, steps) and time.perf_counter() - t0 > budget_s:
            break
    med = float(np.median(times))
    return n * n / med / 1e6, len(times), cores, med


def run_reference(args, rank, world):
    metric = f"Mpt*steps/s at {args.n}^2 FP64 (RK3 step of the vorticity-streamfunction RHS)"
    if rank != 0:
        return 0
    warm = args.warmup   # 0.65 s per warm-up step on 16 Grace cores
    rate, done, cores, sps = cpu_step_rate(args.n, args.steps, warm, budget_s=args.ref_budget)
    line = {
        "impl": "reference", "metric": metric, "value": rate, "unit": "Mpt*steps/s",
        "n_gpus": world, "steps": done, "warmup": warm, "ms_per_step": sps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-phase IC)",
        "config": workload_config(args.n),
        "cpu_baseline": {"value": rate, "unit": "Mpt*steps/s", "cores": cores, "kind": "port",
                         "sample": f"median of {done} timed RK3 steps of the {args.n}^2 FP64 workload, "
                                   f"numpy/scipy.fft restatement of the reference, {cores} threads"},
        "e2e": {"value": rate, "unit": "Mpt*steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def ensemble_runs():
    """The batched-ensemble workload's runs in their global order: 32 x 128^2,
    32 x 256^2, 32 x 512^2 with nu ~ U[5e-4, 5e-3] (seeded); run i's initial
    condition uses seed i, whichever rank advances it."""
    import numpy as np
    rng = np.random.default_rng(0)
    nxs = [128] * 32 + [256] * 32 + [512] * 32
    nus = [float(x) for x in rng.uniform(5e-4, 5e-3, 96)]
    return nxs, nus


def dry_ms(nxs, steps, rank):
    """--dry-cpu: a stand-in for a rank's timed steps (no GPU): proportional
    to the rank's summed run cost, plus a rank-dependent offset so that the
    max over ranks is exercised."""
    from spectral2d_gb300.replicas import run_cost
    return steps * (1e-6 * sum(run_cost(n) for n in nxs) + 0.01 * (rank + 1))


def group(args, local):
    from spectral2d_gb300.replicas import ReplicaGroup
    return ReplicaGroup(backend="gloo" if args.dry_cpu else None, device=None if args.dry_cpu else local)


def run_ensemble(args, rank, world, local):
    """The batched-ensemble workload (not the headline line): 96 runs,
    32 x 128^2, 32 x 256^2, 32 x 512^2, nu ~ U[5e-4, 5e-3], per-run seeds and
    CFL-0.5 dt, one persistent launch per RK3 stage from a CUDA graph.  With
    N ranks the runs are split by cost (replicas.shard_runs, M^2 log2 M per
    run): each rank advances its share as one batch, and value = all runs'
    points x steps over the slowest rank's time (total work fixed: strong
    scaling)."""
    import numpy as np
    from spectral2d_gb300.replicas import run_cost, shard_runs
    nxs_all, nus_all = ensemble_runs()
    shards = shard_runs([run_cost(n) for n in nxs_all], world)
    mine = shards[rank]
    nxs = [nxs_all[i] for i in mine]
    nus = [nus_all[i] for i in mine]
    D = group(args, local)
    threads = cps = None
    check = None
    ens = None
    if args.dry_cpu:
        ms = dry_ms(nxs, args.steps, rank)
    elif mine:
        from spectral2d_gb300 import Ensemble
        ens = Ensemble(nxs, nus, precision=args.precision, device=local)
        dts = []
        for i, r in zip(mine, ens.runs):
            r.set_turbulent_velocity(seed=i, spectrum="k4gauss", k0=10.0, tke=0.5)
            dts.append(r.compute_time_step(CFL))
        ens.set_dt(dts)
        threads, cps, _ = ens.tune()
        ens.integrate_steps(args.warmup)
        ens.synchronize()
    D.barrier()
    if ens is not None:
        ms = ens.time_steps(args.steps)
        ens.status()
    elif not args.dry_cpu:
        ms = 0.0
    D.barrier()
    ms_max = D.reduce(ms, "MAX")
    ms_ranks = D.gather(ms)
    shards_seen = D.gather(mine)
    if ens is not None and args.ens_check_steps > 0:
        # every run advanced in both precisions from the same state; the FP64
        # batch equals single-run FP64 bit for bit (tests/test_gpu_ensemble.py)
        from spectral2d_gb300 import Ensemble
        other = "fp64" if args.precision == "fp32" else "fp32"
        ens2 = Ensemble(nxs, nus, precision=other, device=local)
        for i, r in enumerate(ens.runs):
            ens2.runs[i].set_state(r.get_state()[0])
        ens2.set_dt(dts)
        ens.integrate_steps(args.ens_check_steps)
        ens2.integrate_steps(args.ens_check_steps)
        ens.status()
        ens2.status()
        e32 = ens if args.precision == "fp32" else ens2
        e64 = ens2 if args.precision == "fp32" else ens
        errs = {}
        for i, n in enumerate(nxs):
            a, b = e32.runs[i].get_state()[0], e64.runs[i].get_state()[0]
            errs.setdefault(n, []).append(float(np.linalg.norm(a - b) / np.linalg.norm(b)))
        ens2.close()
        merged = {}
        for part in D.gather(errs):
            for n, v in part.items():
                merged.setdefault(n, []).extend(v)
        check = {"steps": args.ens_check_steps,
                 "fp32_vs_fp64_w_rel_l2": {str(n): {"max": max(v), "median": float(np.median(v))}
                                           for n, v in sorted(merged.items())}}
    pts = sum(n * n for n in nxs_all)
    if rank == 0:
        line = {
            "metric": "ensemble Mpt*steps/s (96 runs: 32x128^2, 32x256^2, 32x512^2)",
            "value": pts * args.steps / (ms_max * 1e-3) / 1e6, "unit": "Mpt*steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic (seeded random-phase ICs)",
            "config": {"workload": "batched ensemble, one persistent launch per RK3 stage",
                       "parallelism": f"runs split by cost over {world} rank(s) (M^2 log2 M per run)",
                       "tile_threads": threads, "ctas_per_sm": cps},
            "runs_per_rank": [len(x) for x in shards_seen], "ms_per_rank": ms_ranks,
            "gpu_launches": 3 * args.steps if not args.dry_cpu else 0, "precision_check": check}
        if args.dry_cpu:
            line["dry_cpu"] = True
            line["shards"] = shards_seen
        print(json.dumps(line), flush=True)
    if ens is not None:
        ens.close()
    D.close()
    return 0


def run_les_batch(args, rank, world, local):
    """Concurrent closure LES (not the headline line): args.les_runs runs of
    256^2 (384^2 collocation grid), decaying turbulence with per-run seeds,
    nu = 1e-4, CFL-0.5 dt; every step is one network forward over all runs
    (the trained 128^2 closure's weights when packaged, else a seeded random
    network) plus the batched transforms and three persistent stage launches,
    replayed from one CUDA graph.  Both precisions are timed; the FP32 runs'
    energy spectra are compared with the FP64 runs' after the same steps.
    With N ranks the runs are split evenly (equal cost): each rank advances
    its share as one batch with its own copy of the network, and value = all
    runs' steps over the slowest rank's time."""
    import os
    import numpy as np
    from spectral2d_gb300.replicas import run_cost, shard_runs
    nr_all, n, nu = args.les_runs, 256, 1e-4
    shards = shard_runs([run_cost(n)] * nr_all, world)
    mine = shards[rank]
    nr = len(mine)
    D = group(args, local)
    res, errs, weights = {}, [], None
    if args.dry_cpu:
        res = {p: dry_ms([n] * nr, 1, rank) for p in ("fp64", "fp32")}
        errs = [0.0] * nr
    elif nr:
        from spectral2d_gb300 import ClosureNet, Ensemble, closure
        grid = 3 * n // 2
        net = ClosureNet(grid, max_batch=nr, seed=0, device=local)
        wpath = os.path.join(os.path.dirname(os.path.abspath(__file__)), "spectral2d_gb300", "data",
                             "closure_les128.npz")
        if os.path.exists(wpath):
            closure.load_weights(net, wpath)
            weights = "trained 128^2 closure (spectral2d_gb300/data/closure_les128.npz)"
        else:
            net.set_scales([1.0, 1.0, 1.0])
            weights = "seeded random network"
        ens = {p: Ensemble([n] * nr, [nu] * nr, precision=p, device=local) for p in ("fp64", "fp32")}
        dts = []
        for j, i in enumerate(mine):
            r64 = ens["fp64"].runs[j]
            r64.set_turbulent_velocity(seed=i, spectrum="k4gauss", k0=10.0, tke=0.5)
            dts.append(r64.compute_time_step(CFL))
            ens["fp32"].runs[j].set_state(r64.get_state()[0])
        for p, e in ens.items():
            e.set_dt(dts)
            e.set_closure(net)
            e.integrate_steps(args.warmup)
            e.synchronize()
            D.barrier()
            ms = e.time_steps(args.steps)
            e.status()
            res[p] = ms / args.steps
        # the network's buffers are shared: the two batches ran one after the other
        for j in range(nr):
            _, e64, _, _, _ = ens["fp64"].runs[j].compute_spectrum()
            _, e32, _, _, _ = ens["fp32"].runs[j].compute_spectrum()
            kk = slice(1, 41)
            errs.append(float(np.max(np.abs(e32[kk] - e64[kk]) / e64[kk])))
        for e in ens.values():
            e.set_closure(None)
            e.close()
        net.close()
    else:
        res = {"fp64": 0.0, "fp32": 0.0}
    D.barrier()
    res_max = {p: D.reduce(v, "MAX") for p, v in res.items()}
    all_errs = [x for part in D.gather(errs) for x in part]
    shards_seen = D.gather(mine)
    p = args.precision
    if rank == 0:
        line = {
            "metric": f"closure-LES run-steps/s ({nr_all} concurrent 256^2 runs)",
            "value": nr_all / (res_max[p] * 1e-3), "unit": "run-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res_max[p],
            "higher_is_better": True, "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
            "dtype": "f64" if p == "fp64" else "f32",
            "data": "synthetic (seeded random-phase ICs)",
            "config": {"workload": "batched closure LES, one network forward + three persistent stage "
                                   "launches per step in one CUDA graph",
                       "runs": nr_all, "n": n, "nu": nu, "cfl": CFL, "network": weights,
                       "parallelism": f"runs split evenly over {world} rank(s)"},
            "ms_per_step_fp64": res_max["fp64"], "ms_per_step_fp32": res_max["fp32"],
            "mpt_steps_per_s": nr_all * n * n / (res_max[p] * 1e-3) / 1e6,
            "runs_per_rank": [len(x) for x in shards_seen],
            "fp32_vs_fp64_Ek_max_rel_err_k_le_40": {"max_over_runs": max(all_errs) if all_errs else None,
                                                    "mean_over_runs": float(np.mean(all_errs)) if all_errs else None,
                                                    "after_steps": args.warmup + args.steps}}
        if args.dry_cpu:
            line["dry_cpu"] = True
            line["shards"] = shards_seen
        print(json.dumps(line), flush=True)
    D.close()
    return 0


def run_les(args, rank, world, local):
    """Single-run closure LES against the DNS (not the headline line): the
    128^2 FP32 LES (192^2 collocation grid) with the trained closure
    (spectral2d_gb300/data/closure_les128.npz; a seeded random network of the
    same shape if absent), the same LES without it, and the 2048^2 FP64 DNS,
    all from the filtered state of one seeded DNS initial condition (nu = 1e-4,
    the DNS's CFL-0.5 dt for all three), timed with CUDA events on their
    streams after the warm-up steps.  value = DNS ms/step over closure-LES
    ms/step; the E(k) error of the closure at this ratio comes from the
    20000-step evaluation (python -m spectral2d_gb300.closure)."""
    import os
    from spectral2d_gb300 import (ClosureNet, Spectral2D, closure, filter_state, les_integrate_steps,
                                  les_set_closure, les_time_steps)
    nd, nl, nu = 2048, 128, 1e-4
    net = ClosureNet(3 * nl // 2, max_batch=1, seed=0, device=local)
    wpath = os.path.join(os.path.dirname(os.path.abspath(__file__)), "spectral2d_gb300", "data",
                         "closure_les128.npz")
    if os.path.exists(wpath):
        closure.load_weights(net, wpath)
        weights = "trained 128^2 closure (spectral2d_gb300/data/closure_les128.npz)"
    else:
        net.set_scales([1.0, 1.0, 1.0])
        weights = "seeded random network"
    dns = Spectral2D(nd, nu=nu, device=local)
    les = Spectral2D(nl, nu=nu, precision="fp32", device=local)
    bare = Spectral2D(nl, nu=nu, precision="fp32", device=local)
    dns.set_turbulent_velocity(seed=SEED + rank, spectrum="k4gauss", k0=10.0, tke=0.5)
    dt = dns.compute_time_step(CFL)
    filter_state(dns, les)
    filter_state(dns, bare)
    les_set_closure(les, net)
    les_integrate_steps(les, args.warmup, dt)
    bare.integrate_steps(args.warmup, dt)
    dns.integrate_steps(args.warmup, dt)
    for h in (les, bare, dns):   # nothing of another handle runs beside a timed one
        h.synchronize()
    ms_les = les_time_steps(les, args.steps, dt) / args.steps
    ms_bare = bare.time_steps(args.steps, dt) / args.steps
    kd = max(3, min(args.steps, 50))
    ms_dns = dns.time_steps(kd, dt) / kd
    les.check_finite()
    net.status()
    if rank == 0:
        print(json.dumps({
            "metric": "128^2 LES + learned closure: wall-clock per step vs the 2048^2 FP64 DNS at the same dt",
            "value": ms_dns / ms_les, "unit": "x", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_les, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (LES), bf16 network, f64 (DNS)",
            "data": "synthetic (seeded random-phase IC)",
            "config": {"workload": "single 128^2 FP32 LES with the learned closure, one CUDA graph per step "
                                   "(closure term on a second stream beside the first stage's transforms)",
                       "n_les": nl, "n_dns": nd, "nu": nu, "cfl": CFL, "network": weights},
            "ms_per_step_dns": ms_dns, "ms_per_step_les_no_closure": ms_bare,
            "speedup_no_closure": ms_dns / ms_bare,
            "speedup_at_10x_dns_dt": 10.0 * ms_dns / ms_les,
            # per step: the RK3 kernels plus the closure's four transform and six convolution kernels
            "gpu_launches": (les.kernels_per_step() + 10) * args.steps}), flush=True)
    les_set_closure(les, None)
    for h in (les, bare, dns):
        h.close()
    net.close()
    return 0


def free_port() -> int:
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def spawn_local_ranks(n: int) -> int:
    """--gpus N without a launcher (WORLD_SIZE unset): start N ranks of this
    script on this node with RANK, LOCAL_RANK, WORLD_SIZE, MASTER_ADDR
    (127.0.0.1) and MASTER_PORT set, as torchrun would, one GPU per rank
    (LOCAL_RANK).  Rank 0 prints the JSON line.  If a rank fails the others
    are stopped; returns the first non-zero exit code (0 if all succeed)."""
    port = free_port()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__), *sys.argv[1:]], env=env))
    rc = 0
    live = list(procs)
    while live:
        for p in list(live):
            code = p.poll()
            if code is None:
                continue
            live.remove(p)
            if code != 0 and rc == 0:
                rc = code if code > 0 else 1
                for q in live:
                    q.terminate()
        time.sleep(0.05)
    return rc


def run_dns_dry(args, rank, world, local):
    """--dry-cpu of the headline workload: one replica per rank (a single run
    does not shard), stand-in step times; value = the sum over ranks of the
    points x steps each replica advanced, over the slowest rank's time."""
    D = group(args, local)
    n = args.n
    D.barrier()
    ms = dry_ms([n], args.steps, rank)
    D.barrier()
    ms_max = D.reduce(ms, "MAX")
    value = D.reduce(n * n * args.steps / (ms_max * 1e-3) / 1e6, "SUM")
    ms_ranks = D.gather(ms)
    if rank == 0:
        print(json.dumps({
            "metric": f"Mpt*steps/s at {n}^2 {args.precision.upper()} (RK3 step of the "
                      "vorticity-streamfunction RHS)",
            "value": value, "unit": "Mpt*steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "none (dry run of the rank logic)", "config": workload_config(n, args.precision),
            "ms_per_rank": ms_ranks, "dry_cpu": True, "gpu_launches": 0}), flush=True)
    D.close()
    return 0


def workload_config(n, precision="fp64"):
    w = 16 if precision == "fp64" else 8
    ws = 2 * (n // 2 + 1) * (3 * n // 2) * w / 1e9   # the two half-spectral intermediates
    return {"workload": f"decaying 2-D turbulence DNS, N={n} (padded {3 * n // 2}^2, 3/2 rule), "
                        f"{precision.upper()}, nu={NU}, dt=CFL {CFL}, TVD-RK3",
            "n": n, "padded": 3 * n // 2, "nu": NU, "cfl": CFL, "seed": SEED,
            "ic": "E(k)~k^4 exp(-2(k/10)^2), TKE 0.5",
            "l2": f"no flush: each stage streams {ws:.2f} GB of intermediates (> 126 MB L2)",
            "parallelism": "replicas (one independent run per GPU)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=150)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--form", default="basdevant", choices=["basdevant", "conservative"])
    ap.add_argument("--workload", default="dns", choices=["dns", "ensemble", "les-batch", "les"])
    ap.add_argument("--les-runs", type=int, default=256)
    ap.add_argument("--ens-check-steps", type=int, default=0)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--ref-budget", type=float, default=150.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--dry-cpu", action="store_true",
                    help="rank logic only, on CPU over gloo: sharding, max/sum over ranks and the JSON "
                         "line, with stand-in step times and no GPU work (for tests)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return spawn_local_ranks(args.gpus)

    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "ensemble":
        return run_ensemble(args, rank, world, local)
    if args.workload == "les-batch":
        return run_les_batch(args, rank, world, local)
    if args.workload == "les":
        return run_les(args, rank, world, local)
    if args.dry_cpu:
        return run_dns_dry(args, rank, world, local)

    # CPU baseline first (no GPU context yet in this process)
    cpu = None
    if rank == 0 and not args.no_cpu:
        # a bounded sample: one warm-up step, then at least 5 timed steps and
        # more until cpu_budget seconds; the rate is that of the median step
        rate, done, cores, sps = cpu_step_rate(args.n, 10000, 1, budget_s=args.cpu_budget)
        cpu = {"value": rate, "unit": "Mpt*steps/s", "cores": cores, "kind": "port",
               "sample": f"median of {done} timed RK3 steps of the {args.n}^2 FP64 workload after 1 "
                         f"warm-up step, numpy/scipy.fft restatement of the reference on {cores} threads "
                         f"({sps:.2f} s/step)"}
        if cores > 1:
            r1, d1, _, s1 = cpu_step_rate(args.n, 10000, 1, budget_s=args.cpu_budget / 2, cores=1)
            cpu["one_core"] = {"value": r1, "unit": "Mpt*steps/s", "cores": 1, "steps": d1, "s_per_step": s1}

    import numpy as np
    from spectral2d_gb300 import Spectral2D, probe_fp64_peak

    from spectral2d_gb300.replicas import ReplicaGroup
    D = ReplicaGroup()
    n = args.n
    s = Spectral2D(n, nu=NU, precision=args.precision, device=local, nonlinear_form=args.form)
    s.set_turbulent_velocity(seed=SEED + rank, spectrum="k4gauss", k0=10.0, tke=0.5)
    dt = s.compute_time_step(CFL)

    # warm-up (graph build + first launches)
    s.integrate_steps(args.warmup, dt)
    s.synchronize()

    clocks = Clocks(local)
    D.barrier()
    clocks.start()
    ms = s.time_steps(args.steps, dt)          # events on the solver stream, synced both sides
    clk = clocks.stop()
    D.barrier()
    s.check_finite()
    ms_max = D.reduce(ms, "MAX")
    value = D.reduce(n * n * args.steps / (ms_max * 1e-3) / 1e6, "SUM")
    ms_per_step = ms_max / args.steps

    # per-kernel launch times (events between every launch) for the roofline
    kms_total, kms = s.time_steps(max(3, min(args.steps, 10)), dt, per_kernel=True)
    ksteps = max(3, min(args.steps, 10))
    launches_per_kernel = 3 * ksteps
    wbytes = 16 if args.precision == "fp64" else 8
    bm = byte_model(n, wbytes, args.form)
    fm = flop_model(n, args.form)
    names = ["yinv", "xpass", "yfwd"]
    avg = {k: kms[i] / launches_per_kernel for i, k in enumerate(names)}
    dom = max(names, key=lambda k: avg[k])
    peaks = read_peaks()
    hbm, hbm_src = hbm_peak(peaks)
    achieved = bm["per_kernel"][dom] / (avg[dom] * 1e-3) / 1e9
    fp64 = probe_fp64_peak(local) if rank == 0 else None
    alu = fm[dom] / (avg[dom] * 1e-3) / 1e12
    traffic = read_traffic(dom, args.form, n, args.precision)

    # e2e through the reference-facing C-ABI with host arrays
    e2e = None
    if args.e2e_steps > 0:
        from spectral2d_gb300.solver import pinned_array
        w0, _ = s.get_state()
        w_host = pinned_array(w0.shape)
        p_host = pinned_array(w0.shape)
        w_host[...] = w0
        s.integrate_one_step_host(w_host, dt, p_host, inplace=True)   # warm-up
        s.synchronize()
        D.barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            s.integrate_one_step_host(w_host, dt, p_host, inplace=True)
        t1 = time.perf_counter()
        el = D.reduce(t1 - t0, "MAX")
        nbytes = w_host.nbytes
        # in: the retained rectangle of wC (kx <= N/2, |ky| <= N/2); out: wC and psiC whole
        h2d = (n // 2 + 1) * 16 * (n + 1)
        e2e = {"value": D.reduce(n * n * args.e2e_steps / el / 1e6, "SUM"), "unit": "Mpt*steps/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 2 * nbytes,
               "steps": args.e2e_steps,
               "path": "s2d_integrate_one_step_host on pinned host arrays "
                       "(reference-layout wC in: its retained modes; wC, psiC out, their truncated "
                       "part written from a second stream during the step)"}

    hbm_view = {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "peak_source": f"{hbm_src} HBM copy bandwidth (MEASURED_PEAKS.json)",
                "algorithmic_bytes_per_launch": bm["per_kernel"][dom],
                "step_frac": bm["step"] / (ms_per_step * 1e-3) / 1e9 / hbm,
                "step_frac_reference_form_bytes": bm["step_reference_form"] / (ms_per_step * 1e-3) / 1e9 / hbm}
    common = {"kernel": dom, "traffic": traffic, "launch_ms": avg[dom], "nonlinear_form": args.form,
              "kernel_ms_per_step": {k: kms[i] / ksteps for i, k in enumerate(names)}}
    if args.precision == "fp64" and fp64:
        # FP64 on GB300: the FFT kernels keep the FP64 pipe ~90 % busy at a few
        # percent of the HBM roof, so the binding roof is the FP64 rate
        roofline = {"bound": "fp64", "achieved": alu, "peak": fp64, "unit": "TFLOP/s", "frac": alu / fp64,
                    "peak_source": "measured FP64 FMA loop on this GPU (s2d_probe_fp64_peak)",
                    "flops_per_launch": fm[dom], "flop_convention": "benchFFT 2.5 M log2 M per real 1-D FFT",
                    "hbm": hbm_view, **common}
    else:
        roofline = {"bound": "hbm", **{k: v for k, v in hbm_view.items()}, "traffic": traffic, **common}
    if rank == 0:
        line = {
            "metric": f"Mpt*steps/s at {n}^2 {args.precision.upper()} (RK3 step of the "
                      "vorticity-streamfunction RHS)",
            "value": value, "unit": "Mpt*steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic (seeded random-phase IC)",
            "config": workload_config(n, args.precision),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": s.kernels_per_step() * args.steps,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    s.close()
    D.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
