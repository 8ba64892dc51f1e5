#!/usr/bin/env python
"""Benchmark: converged RANS forward solves per second on one GB300.

Workload (the batched-theta configuration on the plane-channel case):
  * mesh: streamwise-periodic plane channel, 4 x 128 quads, geometric wall
    stretching ratio 1.08 from each wall (64 cells per half), half-height 1,
    Re_tau = 550 (nu = 1/550, body force 1), U0 = 20, k0 = 1e-2, omega0 = 10;
  * 256 theta draws from numpy.random.default_rng(11).uniform(0.8, 1.2, (256, 6))
    times the SST defaults of [beta*, sigma_k1, sigma_w1, a1, beta1, kappa];
    draws with kappa outside [0.35, 0.5] are InvalidParameters and are served
    without a solve, exactly as the reference's ForwardModel::evaluate does;
  * every valid theta: a cold SIMPLE solve to the reference's 1e-8 scaled
    residual (max 60000 outer iterations) in the batched mixed-precision form
    (FP32 bulk around an FP64 state, FP64 polishing stage; --precision fp64
    times the plain FP64 drop-in instead).
One step = the whole 256-theta batch in one persistent launch.

`value` is converged solves / device time of the launch (CUDA events on the
launching stream, inputs resident).  `e2e` is the same metric through the
public batched API (rans_sst_py.solve_batch) with host buffers: parameters
in, every instance's full flow state copied back to the host each step.
`latency_ms` gives p50/p99 of the per-instance completion times inside the
launch.  After the timed steps the same batch runs once through the plain
FP64 engine (`fp64_plain`: its throughput) and once through the FP64 engine
to stagnation: `error_vs_fp64_fixed_point` is the per-instance relative L2 of
the delivered mixed-precision fields and channel outputs (Cf, U+(y+),
nu_t/nu) against that fixed point, beside the FP64 drop-in's own.

`--impl reference` times the reference's CPU solver (the reference built from
its sources when oracle/_ref holds it, else the C restatement in oracle/) on
all host cores: complete cold solves of the same theta draw to the same 1e-8
scaled residual, one per core per step, timed by the wall clock.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import tempfile
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "bayesian-turbulence-modeling_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_THETA = 256
THETA_SEED = 11
ACTIVE = [8, 0, 1, 9, 2, 10]
NY, NX, RE_TAU, RATIO = 128, 4, 550.0, 1.08
MAX_ITER, TOL = 60000, 1e-8
INIT = dict(u=(20.0, 0.0, 0.0), p=0.0, k=1e-2, omega=10.0)
WORKLOAD = "theta256_channel4x128_re550"
PRECISION = "mixed"


def make_case_inputs():
    import rans_sst_py as rs
    m = rs.Mesh.make_channel_periodic_geometric(NX, NY, 1.0, 1.0, RATIO)
    m.compute_wall_distance()
    bcs = rs.FlowBoundaryConditions.channel_defaults(m, 0.0, 0.0, 0.0)
    s = rs.SolverSettings()
    s.verbose = False
    s.body_force = rs.Vec3(1.0, 0.0, 0.0)
    s.max_iterations = MAX_ITER
    s.convergence_tol = TOL
    s.precision = PRECISION
    return m, bcs, 1.0 / RE_TAU, s


def theta_set():
    import rans_sst_py as rs
    ps = rs.InferenceParameterSet.from_indices("c3", ACTIVE)
    base = np.array(ps.pack(rs.SSTCoefficients()))
    draws = np.random.default_rng(THETA_SEED).uniform(0.8, 1.2, (N_THETA, len(ACTIVE))) * base
    valid = [bool(ps.in_bounds(list(t))) for t in draws]
    coeffs = np.array([ps.unpack(list(t)).to_vector() for t in draws])
    return draws, coeffs, np.array(valid)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, gpu_index):
        # raw samples go next to the run's other outputs (BTM_CLOCKS_DIR, else
        # the system temporary directory); the JSON line carries the summary
        out_dir = os.environ.get("BTM_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(out_dir, f"clocks_bench_{os.getpid()}.csv")
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- algorithmic bytes (FP64, 2-D quads) -----------------------------------
# Compulsory traffic per cell: one outer iteration's assembly, gradients, SST
# closure, corrections and BCs (~1100 B) plus one Krylov/AMG inner iteration
# (~376 B: two LDU mat-vecs and 29 vector streams, the BiCGStab figure).
BYTES_PER_CELL_OUTER = 1100.0
BYTES_PER_CELL_INNER = 376.0
# Mixed precision: FP32 coefficient, gradient and closure streams plus the
# FP64 state and defect streams (~760 B per cell per outer iteration), FP32
# Krylov iterations (2 LDU mat-vecs at 44 B + 29 FP32 streams = 204 B).
BYTES_PER_CELL_OUTER_MIXED = 760.0
BYTES_PER_CELL_INNER_MIXED = 204.0
# ncu DRAM bytes (read + write) per cell-iteration of the profile case (304
# instances x 200 outer iterations of the 4x128 channel), per engine.
TRAFFIC_PER_CELL_ITER = {"fp64": 460.0, "mixed": 49.4}
FIXED_POINT_SUBSET = 8
FIXED_POINT_ITERS = 40000
FIXED_POINT_STAG_ITERS = 60000
FP64_RESIDUAL_FLOOR = 1e-10   # lowest tolerance the FP64 drop-in reaches on the 4x128 channel


def algorithmic_bytes(n_cells, outer, inner, mixed=False):
    if mixed:
        return n_cells * (BYTES_PER_CELL_OUTER_MIXED * outer + BYTES_PER_CELL_INNER_MIXED * inner)
    return n_cells * (BYTES_PER_CELL_OUTER * outer + BYTES_PER_CELL_INNER * inner)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# ---- CPU side (the reference algorithm on all host cores) -------------------
_CPU_CTX = {}


def _cpu_setup():
    """Per-process state of a CPU worker: the case inputs, the theta set and
    the solver the reference arm runs (the reference compiled from its own
    sources when oracle/_ref holds it, else the C restatement in oracle/)."""
    if _CPU_CTX:
        return _CPU_CTX
    sys.path.insert(0, ROOT)
    sys.path.insert(0, PKG)
    from oracle import port
    m, bcs, nu, s = make_case_inputs()
    _, coeffs, valid = theta_set()
    _CPU_CTX.update(m=m, bcs=bcs, nu=nu, s=s, coeffs=coeffs, ids=np.nonzero(valid)[0], kind=reference_kind())
    if _CPU_CTX["kind"] == "reference":
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import cases as tc
        from oracle import refdriver as rd
        path = os.path.join(tempfile.gettempdir(), f"btm_bench_mesh_{os.getpid()}.msh")
        with open(path, "wb") as fh:
            fh.write(tc.mesh_to_bytes(m))
        # the reference loader reports on stdout; keep the JSON line alone there
        saved = os.dup(1)
        devnull = os.open(os.devnull, os.O_WRONLY)
        os.dup2(devnull, 1)
        try:
            rm = rd.RefMesh.load(path)
            rm.wall_distance()
        finally:
            os.dup2(saved, 1)
            os.close(saved)
            os.close(devnull)
        bca, keep = port.bc_array(bcs)
        _CPU_CTX.update(rm=rm, bca=bca, keep=keep)
    return _CPU_CTX


def _cpu_solve(args):
    """One solve of valid theta number j (cycled) on this host core: the
    reference's ForwardModel path (cold uniform start, convergence test at
    `tol`, at most `max_iter` outer iterations).  Returns (converged,
    iterations, seconds)."""
    j, max_iter, tol = args
    from oracle import port
    ctx = _cpu_setup()
    s = ctx["s"].copy()
    s.max_iterations, s.convergence_tol = max_iter, tol
    c = ctx["coeffs"][ctx["ids"][j % len(ctx["ids"])]]
    t0 = time.perf_counter()
    if ctx["kind"] == "reference":
        ini, _ = port.make_init(**INIT)
        m = ctx["m"]
        _, hist, _ = ctx["rm"].solve(ctx["bca"], ctx["nu"], port.settings_struct(s), c, 0, ini, m.n_cells(),
                                     m.n_boundary_faces(), 0)
        conv, its = int(hist.converged), int(hist.iterations_run)
    else:
        _, h = port.solve(ctx["m"], ctx["bcs"], ctx["nu"], s, c, 0, **INIT)
        conv, its = int(h["converged"]), int(h["iterations_run"])
    return conv, its, time.perf_counter() - t0


def _cpu_pool(n_proc):
    from oracle import port
    port.build()
    return mp.get_context("spawn").Pool(n_proc)


def cpu_converged_solves(pool, n_proc, n_solves, first=0):
    """`n_solves` complete converged solves of consecutive valid theta on
    `n_proc` host processes, scheduled dynamically (a core takes the next
    theta as soon as its solve ends).  Returns the converged count, the wall
    time, the per-solve latencies and the outer iterations per solve."""
    jobs = [(first + j, MAX_ITER, TOL) for j in range(n_solves)]
    t0 = time.perf_counter()
    res = list(pool.imap_unordered(_cpu_solve, jobs))
    wall = time.perf_counter() - t0
    return sum(r[0] for r in res), wall, [r[2] for r in res], [r[1] for r in res]


def reference_kind():
    return "reference" if os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libref_driver.so")) else "port"


# ---- distributed helpers -----------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def rank_device_env(local, env=None):
    """The CUDA_VISIBLE_DEVICES value that gives local rank `local` its own
    GPU, set before the process makes its first CUDA call: the rank's entry of
    a list the launcher exported to every rank, the launcher's value when it
    already names one device per rank, else the local rank itself."""
    env = os.environ if env is None else env
    vis = env.get("CUDA_VISIBLE_DEVICES")
    if vis is None or not vis.strip():
        return str(local)
    ids = [v.strip() for v in vis.split(",") if v.strip()]
    return ids[local] if len(ids) > local else vis


def sampled_gpu(local):
    """The nvidia-smi id (index or UUID) of the GPU this process computes on:
    the first entry of CUDA_VISIBLE_DEVICES (nvidia-smi itself ignores that
    variable), else the local rank."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    ids = [v.strip() for v in vis.split(",") if v.strip()] if vis else []
    return ids[0] if ids else str(local)


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, x):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def dist_sum(world, x):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())
    return x


def aggregate_ranks(world, dev_ms, wall_s, conv_counts):
    """Whole-job figures over the ranks: the slowest rank's mean step time
    (device and end-to-end), the converged solves of all ranks per step, and
    the job throughput = all ranks' converged solves / the slowest step."""
    step_s = dist_max(world, statistics.mean(dev_ms) / 1e3)
    e2e_s = dist_max(world, statistics.mean(wall_s))
    converged = dist_sum(world, statistics.mean(conv_counts))
    return step_s, e2e_s, converged, converged / step_s, converged / e2e_s


def run_reference(args, world, rank):
    """The reference arm: the reference's own CPU solver (the build in
    oracle/_ref when present, else its C restatement) on every host core.
    One step = os.cpu_count() complete cold solves to the 1e-8 scaled
    residual, one per core, of consecutive valid theta of the same 256-theta
    draw (cycling through the 219 valid ones); the timed region is the wall
    clock around all timed steps' solves, scheduled dynamically over the
    cores.  Warm-up steps run one 100-iteration solve per process (process
    start-up, imports, first calls)."""
    if rank != 0:
        return
    n_proc = os.cpu_count() or 1
    _, _, valid = theta_set()
    with _cpu_pool(n_proc) as pool:
        for _ in range(args.warmup):
            pool.map(_cpu_solve, [(j, 100, 0.0) for j in range(n_proc)])
        conv, wall, lat, its = cpu_converged_solves(pool, n_proc, args.steps * n_proc)
    value = conv / wall
    kind = reference_kind()
    line = {"metric": "converged RANS solves/sec", "value": value, "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "precision": "fp64", "n_theta": N_THETA, "n_valid": int(valid.sum()),
                       "cells": NX * NY, "tol": TOL, "solves_per_step": n_proc,
                       "iters_per_converged_solve": float(np.mean(its))},
            "latency_ms": {"p50": 1e3 * float(np.percentile(lat, 50)), "p99": 1e3 * float(np.percentile(lat, 99)),
                           "note": "wall time of each solve on its host core"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": n_proc, "kind": kind,
                             "sample": f"{args.steps * n_proc} complete cold solves to the 1e-8 scaled residual "
                                       f"({n_proc} per step, consecutive valid theta of the draw), "
                                       f"{conv} converged, {wall:.1f} s wall on {n_proc} processes"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _batch_stats(outs):
    conv = sum(o.converged for o in outs)
    fin = np.array([o.finish_ms for o in outs])
    return conv, fin


def _output_errors(mesh, nu, a_outs, b_outs):
    """Per-instance errors of the channel outputs of a against b: the wall
    skin friction (mean over the bottom wall, relative), and the U+ and
    nu_t / nu profiles of the wall-to-centreline column (relative L2)."""
    from rans_sst_py import channel_profile
    errs = {"Cf": [], "U+(y+)": [], "nu_t/nu": []}
    for a, b in zip(a_outs, b_outs):
        pa, pb = channel_profile(mesh, a.state, nu), channel_profile(mesh, b.state, nu)
        errs["Cf"].append(abs(pa["cf"] - pb["cf"]) / abs(pb["cf"]))
        errs["U+(y+)"].append(float(np.linalg.norm(pa["U"] - pb["U"]) / np.linalg.norm(pb["U"])))
        errs["nu_t/nu"].append(float(np.linalg.norm(pa["nu_t"] - pb["nu_t"]) / np.linalg.norm(pb["nu_t"])))
    return {f: {"max": max(v), "p50": float(np.percentile(v, 50)), "p99": float(np.percentile(v, 99))}
            for f, v in errs.items()}


def _field_errors(a_outs, b_outs):
    """Per-instance relative L2 of a against b (U, k, omega, nu_t), and the
    pressure against the dynamic pressure scale with each field's mean
    removed: in the streamwise-periodic channel nothing fixes the pressure
    level (the corrections add a mean-free p' times alpha_p), so its level is
    set by the path to the fixed point and only differences are physical."""
    errs = {f: [] for f in ("U", "k", "omega", "nuT", "p")}
    for a, b in zip(a_outs, b_outs):
        for f in ("U", "k", "omega", "nuT"):
            errs[f].append(float(np.linalg.norm(a.state[f] - b.state[f]) / max(np.linalg.norm(b.state[f]), 1e-300)))
        U = b.state["U"]
        q = 0.5 * np.max(np.sum(U * U, axis=1))
        dp = (a.state["p"] - a.state["p"].mean()) - (b.state["p"] - b.state["p"].mean())
        errs["p"].append(float(np.linalg.norm(dp) / (q * np.sqrt(len(U)))))
    return {f: {"max": max(v), "p50": float(np.percentile(v, 50)), "p99": float(np.percentile(v, 99))}
            for f, v in errs.items()}


def run_gpu(args, world, rank, local):
    import rans_sst_py as rs
    from rans_sst_py._lib import lib

    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = rank_device_env(local)
    m, bcs, nu, s = make_case_inputs()
    draws, coeffs, valid = theta_set()
    case = rs.Case(m, bcs, nu, s)
    ids = np.nonzero(valid)[0]
    n = len(ids)
    cases = [case] * n
    cf = coeffs[ids]
    inits = [INIT] * n

    # One step = one call of the public batched API with host buffers: the
    # parameters go in, every instance's full flow state comes back.  The
    # device time of the persistent launch inside the call (CUDA events on
    # its stream) gives `value`; the wall time of the whole call gives `e2e`.
    def step(c=case):
        t0 = time.perf_counter()
        outs = rs.solve_batch([c] * n, cf, None, inits, want_state=True)
        return outs, lib().btm_last_launch_ms(), time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    dist_barrier(world)
    dev_ms, wall_s, conv_counts, outer, inner, fins = [], [], [], 0, 0, []
    with ClockSampler(sampled_gpu(local)) as clocks:
        for _ in range(args.steps):
            outs, ms, wall = step()
            dev_ms.append(ms)
            wall_s.append(wall)
            conv, fin = _batch_stats(outs)
            conv_counts.append(conv)
            fins.append(fin)
            outer += sum(o.iterations_run for o in outs)
            inner += sum(o.inner_iterations for o in outs)
    dist_barrier(world)
    clk = clocks.summary()
    step_s, e2e_s, converged_all, value, e2e_value = aggregate_ranks(world, dev_ms, wall_s, conv_counts)
    converged = statistics.mean(conv_counts)
    shape = case.launch_shape(PRECISION)
    h2d = n * (11 * 8 + 4 + 48)
    nb = m.n_boundary_faces()
    d2h = n * 8 * (m.n_cells() * 11 + nb * 6)
    fin = np.concatenate(fins)
    polish = [o.polish_start / max(1, o.iterations_run) for o in outs if o.polish_start >= 0]

    iters_per_solve = outer / max(1, args.steps * n)
    mixed = PRECISION == "mixed"
    bytes_per_launch = algorithmic_bytes(m.n_cells(), outer / args.steps, inner / args.steps, mixed)
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / step_s / 1e9
    cell_iters = m.n_cells() * outer / args.steps
    traffic = (TRAFFIC_PER_CELL_ITER[PRECISION] * cell_iters) if args.traffic is None else args.traffic
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_kind": peak_kind,
                "note": "algorithmic bytes of the persistent solve kernel over its CUDA-event time; the "
                        "per-instance working set lives in L2 / shared memory, so the kernel is bound by "
                        "barrier-separated phase latency and the FP64 pipe, not by HBM; traffic = ncu DRAM "
                        "bytes per cell-iteration of the profile case scaled to this launch"}
    line = {"metric": "converged RANS solves/sec", "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "precision": PRECISION, "n_theta": N_THETA, "n_valid": int(n),
                       "cells": m.n_cells(), "tol": TOL, "converged_per_step": converged,
                       "iters_per_converged_solve": iters_per_solve,
                       "inner_iters_per_outer": inner / max(1, outer),
                       "polish_start_frac": statistics.mean(polish) if polish else None,
                       "launch_shape": {"cta_threads": shape["threads"], "autotuned": shape["tuned"],
                                        "probe_instances": shape["probe"],
                                        "probe_ms_256_512": shape["probe_ms"]},
                       "l2": "working set L2/shared-memory resident; no flush needed for a single persistent "
                             "launch per step"},
            "latency_ms": {"p50": float(np.percentile(fin, 50)), "p99": float(np.percentile(fin, 99)),
                           "max": float(fin.max()),
                           "note": "per-instance device time from the launch's first instance start to the "
                                   "instance's end"},
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": args.steps, "clocks": clk, "roofline": roofline}
    fp64_iters = None
    if rank == 0 and mixed and not args.no_fp64_compare:
        # the plain FP64 drop-in on the same batch (one launch, untimed by the
        # bench clock): its throughput, and the per-instance field error of the
        # mixed-precision results against it
        s64 = s.copy()
        s64.precision = "fp64"
        case64 = rs.Case(m, bcs, nu, s64)
        outs64, ms64, _ = step(case64)
        conv64, fin64 = _batch_stats(outs64)
        fp64_iters = sum(o.iterations_run for o in outs64) / n
        line["fp64_plain"] = {"value": conv64 / (ms64 / 1e3), "unit": "solves/s", "ms": ms64,
                              "converged": conv64, "iters_per_converged_solve": fp64_iters,
                              "latency_ms": {"p50": float(np.percentile(fin64, 50)),
                                             "p99": float(np.percentile(fin64, 99))},
                              "speedup_of_mixed": value / (conv64 / (ms64 / 1e3))}
        # the FP64 fixed point of every instance (the FP64 engine, pinned to
        # the reference at stagnation, run well past convergence with the
        # test off): the error of what each engine delivers against it, per
        # field and per channel output
        sfp = s.copy()
        sfp.precision, sfp.convergence_tol, sfp.max_iterations = "fp64", 0.0, FIXED_POINT_STAG_ITERS
        outs_fp = rs.solve_batch([rs.Case(m, bcs, nu, sfp)] * n, cf, None, inits, want_state=True)
        ev = _field_errors(outs, outs_fp)
        ev.update(_output_errors(m, nu, outs, outs_fp))
        ev["note"] = (f"mixed solves as delivered (converged by the engine's rule) against the FP64 fixed point of "
                      f"the same theta ({FIXED_POINT_STAG_ITERS} FP64 iterations, convergence test off)")
        line["error_vs_fp64_fixed_point"] = ev
        e64 = _field_errors(outs64, outs_fp)
        e64.update(_output_errors(m, nu, outs64, outs_fp))
        e64["note"] = "the FP64 drop-in stopped by the reference's 1e-8 test, against the same fixed point"
        line["fp64_plain"]["error_vs_fp64_fixed_point"] = e64
        # the FP64 drop-in at the tolerance that gives it the accuracy the
        # mixed solves are delivered with: the distance to the fixed point is
        # proportional to the tolerance, so the tolerance is scaled by the
        # ratio of the two errors (largest over U, k, nu_t) and rounded to the
        # nearest power of ten, but not below FP64_RESIDUAL_FLOOR: the
        # reference iteration's scaled continuity residual settles at 3-7e-11
        # on this mesh (it reaches 1e-10 after 20-37k outer iterations and
        # 1e-11 never), so below that the leg is a lower bound of the speed-up
        # at equal accuracy and its own error is reported beside it
        worst = lambda e: max(e[f]["max"] for f in ("U", "k", "nuT"))  # noqa: E731
        ratio = worst(e64) / max(worst(ev), 1e-300)
        tol_eq = max(10.0 ** round(math.log10(s64.convergence_tol / max(ratio, 1.0))), FP64_RESIDUAL_FLOOR)
        s64t = s64.copy()
        s64t.convergence_tol = tol_eq
        s64t.max_iterations = 2 * MAX_ITER
        outs64t, ms64t, _ = step(rs.Case(m, bcs, nu, s64t))
        conv64t, _ = _batch_stats(outs64t)
        e64t = _field_errors(outs64t, outs_fp)
        e64t.update(_output_errors(m, nu, outs64t, outs_fp))
        v64t = conv64t / (ms64t / 1e3)
        line["fp64_plain_equal_accuracy"] = {
            "value": v64t, "unit": "solves/s", "ms": ms64t, "converged": conv64t,
            "tol": tol_eq, "iters_per_converged_solve": sum(o.iterations_run for o in outs64t) / n,
            "speedup_of_mixed": value / v64t if conv64t else None,
            "error_vs_fp64_fixed_point": e64t,
            "note": "the FP64 drop-in at the power of ten nearest to 1e-8 / (its error at 1e-8 over the mixed "
                    "solves' error), not below its residual floor (1e-10): at most the accuracy the mixed solves "
                    "are delivered with, so the speed-up is a lower bound at equal accuracy"}
        # precision error proper: a subset run to stagnation (convergence test
        # off, well past the converged iteration count) in both engines
        sub = list(range(0, n, max(1, n // FIXED_POINT_SUBSET)))[:FIXED_POINT_SUBSET]
        tight = {}
        for prec in ("mixed", "fp64"):
            st = s.copy()
            st.precision, st.convergence_tol, st.max_iterations = prec, 0.0, FIXED_POINT_ITERS
            ct = rs.Case(m, bcs, nu, st)
            tight[prec] = rs.solve_batch([ct] * len(sub), cf[sub], None, [INIT] * len(sub), want_state=True)
        fp = _field_errors(tight["mixed"], tight["fp64"])
        fp["instances"] = len(sub)
        fp["iterations"] = FIXED_POINT_ITERS
        fp["note"] = "mixed vs FP64, both run to stagnation (fixed-point error)"
        line["error_fixed_point"] = fp
    if rank == 0 and not args.no_cpu_baseline:
        # the reference algorithm on every host core, timed on complete
        # converged solves: one per core (about 10-20 s of CPU work)
        n_proc = os.cpu_count() or 1
        with _cpu_pool(n_proc) as pool:
            pool.map(_cpu_solve, [(j, 100, 0.0) for j in range(n_proc)])
            conv_cpu, wall_cpu, lat_cpu, its_cpu = cpu_converged_solves(pool, n_proc, n_proc)
        line["cpu_baseline"] = {"value": conv_cpu / wall_cpu, "unit": "solves/s", "cores": n_proc,
                                "kind": reference_kind(),
                                "sample": f"{n_proc} complete cold solves to the 1e-8 scaled residual, one per "
                                          f"host process ({conv_cpu} converged, {wall_cpu:.1f} s wall, "
                                          f"{np.mean(its_cpu):.0f} outer iterations per solve)"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_profile_case(mesh="channel4x128"):
    """A bounded launch of the same kernel for profilers: 304 instances (two
    per SM) of the 4x128 channel, 200 outer iterations each, or of the
    1920-cell permuted backward-facing step, 40 outer iterations each
    (reference BFS settings; its FP64 solves use the reference-order AMG,
    kernel k_simple_block_ref)."""
    import rans_sst_py as rs
    from rans_sst_py._lib import lib
    if mesh == "bfs1920":
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import cases as tc
        m, bcs, nu, init = tc.bfs_case()
        s = tc.bfs_settings(200, 0.0)
        s.precision = PRECISION
    else:
        m, bcs, nu, s = make_case_inputs()
        init = INIT
    s.max_iterations, s.convergence_tol = (40 if mesh == "bfs1920" else 200), 0.0
    case = rs.Case(m, bcs, nu, s)
    _, coeffs, valid = theta_set()
    cf = coeffs[np.nonzero(valid)[0]]
    cf = np.concatenate([cf, cf])[:304]
    outs = rs.solve_batch([case] * len(cf), cf, None, [init] * len(cf), want_state=False)
    it = sum(o.iterations_run for o in outs)
    inner = sum(o.inner_iterations for o in outs)
    ms = lib().btm_last_launch_ms()
    print(json.dumps({"profile_case": mesh, "instances": len(cf), "outer_iterations": it, "inner_iterations": inner,
                      "launch_ms": ms, "precision": PRECISION,
                      "bytes_algorithmic": algorithmic_bytes(m.n_cells(), it, inner, PRECISION == "mixed")}))


# ---- served stream ------------------------------------------------------------
SERVED_RATE = 200.0        # mean Poisson arrival rate (requests / s)
SERVED_SECONDS = 10.0      # arrival window
SERVED_CHAINS = 32
SERVED_SEED = 13
SERVED_MAX_ITER = 20000  # outer-iteration cap per request
SERVED_MAX_ITER_C4 = 100000   # the same on the 2,048-cell cases


def run_served(args):
    """Served stream: Poisson arrivals (default_rng(13).exponential(1/200)) of
    forward-solve requests from 32 MCMC chains random-walking in the 6-D
    theta space (theta <- theta * (1 + 0.02 N(0,1)), out-of-bounds steps are
    InvalidParameters without a solve), each chain on one case (chain mod 2:
    Re_tau 180 4x32 channel, or Re_tau 500 4x32 plane Couette), warm-started
    from the chain's last field kept on the device (tag = chain), converged to
    the 1e-8 scaled residual in the mixed-precision engine through the
    continuous-batching server.  Latency = completion - arrival (host clock),
    including any wait for a free slot."""
    import rans_sst_py as rs
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as tc
    ps = rs.InferenceParameterSet.from_indices("c4", ACTIVE)
    base = np.array(ps.pack(rs.SSTCoefficients()))
    if args.served_cases == "c4":
        # the configuration's 2,048-cell cases: the Re_tau 1000 channel (4x512)
        # and the Re_tau 500 plane Couette (16x128), first cells at y+ 0.4
        # (the 122,880-cell step of the configuration runs on the cooperative
        # grid, about 80k outer iterations per cold solve: not served here)
        cap = SERVED_MAX_ITER_C4
        m1, b1, nu1, i1 = tc.periodic_channel(512, 1000.0)
        m2, b2, nu2, i2 = tc.couette_case(16, 128)
        names = ("channel_re1000_4x512", "couette_re500_16x128")
    else:
        cap = SERVED_MAX_ITER
        m1, b1, nu1, i1 = tc.periodic_channel(32, 180.0)
        m2, b2, nu2, i2 = tc.couette_case(4, 32)
        names = ("channel_re180_4x32", "couette_re500_4x32")
    s1 = tc.channel_settings(cap, TOL)
    s1.precision = "mixed"
    s2 = tc.couette_settings(cap, TOL)
    s2.precision = "mixed"
    case_defs = [(rs.Case(m1, b1, nu1, s1), i1, names[0]), (rs.Case(m2, b2, nu2, s2), i2, names[1])]
    # each chain needs its likelihood: skin friction and two velocity probes,
    # evaluated on the device, are all that leaves it per request
    for cd, (m, wall) in zip(case_defs, ((m1, "bottom_wall"), (m2, "bottom_wall"))):
        op = rs.ObservationOperator()
        op.add_skin_friction(wall, rs.Vec3(0.5, 0.0, 0.5), 0.006, 0.001, 16.0)
        op.add_velocity_profile(rs.Vec3(0.5, 1.0, 0.5), 0, 18.0, 1.0)
        op.add_velocity_profile(rs.Vec3(0.5, 0.1, 0.5), 0, 9.0, 1.0)
        cd[0].set_observations(op)
    rng = np.random.default_rng(SERVED_SEED)
    rate = args.served_rate
    gaps = rng.exponential(1.0 / rate, int(rate * SERVED_SECONDS * 1.5) + 16)
    times = np.cumsum(gaps)
    times = times[times < SERVED_SECONDS]
    theta = np.tile(base, (SERVED_CHAINS, 1))
    reqs = []
    invalid = 0
    for j, t in enumerate(times):
        c = j % SERVED_CHAINS
        theta[c] = theta[c] * (1.0 + 0.02 * rng.standard_normal(len(ACTIVE)))
        if not ps.in_bounds(list(theta[c])):
            invalid += 1
            continue
        reqs.append((t, c, np.array(ps.unpack(list(theta[c])).to_vector())))
    srv = rs.Server(max_slots=304, hbm_budget_bytes=4 << 30)
    # warm-up: one solve per case (builds and loads the library, first launches)
    for cdef in case_defs:
        srv.submit(cdef[0], np.array(tc.COEFF_DEFAULTS), init=cdef[1])
    while srv.pending:
        srv.poll(timeout_ms=20)
    backlog, arrival_of, latency, iters, conv, service, lls = [], {}, [], [], 0, [], []
    t0 = time.perf_counter()
    k = 0
    max_inflight = 0
    while k < len(reqs) or backlog or srv.pending:
        now = time.perf_counter() - t0
        while k < len(reqs) and reqs[k][0] <= now:
            backlog.append(reqs[k])
            k += 1
        still = []
        for (ta, c, cf) in backlog:
            case, ini, _ = case_defs[c % 2]
            rid = srv.submit(case, cf, init=ini, tag=c, want_state=False, tag_norms=True)
            if rid is None:
                still.append((ta, c, cf))
            else:
                arrival_of[rid] = ta
        backlog = still
        for rid, out in srv.poll(timeout_ms=2):
            latency.append(time.perf_counter() - t0 - arrival_of.pop(rid))
            iters.append(out.iterations_run)
            service.append(out.solve_ms)
            conv += int(out.converged)
            lls.append(out.log_lik)
        max_inflight = max(max_inflight, srv.stats()["inflight"])
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array(latency) * 1e3
    line = {"metric": "served forward solves/sec", "value": len(latency) / wall, "unit": "solves/s",
            "higher_is_better": True, "n_gpus": 1, "dtype": "f32+f64", "data": "synthetic", "impl": "gb300",
            "config": {"workload": f"served_stream_32chains_poisson{rate:g}", "rate_per_s": rate,
                       "arrival_window_s": SERVED_SECONDS, "chains": SERVED_CHAINS,
                       "cases": [cd[2] for cd in case_defs], "tol": TOL, "precision": "mixed",
                       "warm_start": "device-resident tag per chain; residuals scaled by the chain's "
                                     "cold solve (BTM_REQ_TAG_NORMS)", "max_iterations": cap},
            "observables": {"per_request": 3, "log_lik_finite": int(np.isfinite(lls).sum()),
                            "note": "Cf + 2 velocity probes and the log-likelihood evaluated on the device; "
                                    "no field leaves the device"},
            "requests": int(len(times)), "invalid_parameters": invalid, "solved": len(latency),
            "converged": conv, "wall_s": wall, "mean_outer_iters": float(np.mean(iters)) if iters else None,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "max": float(lat.max()), "note": "arrival to completion, including the wait for a "
                           "free slot when the offered rate exceeds the service rate"},
            "service_ms": {"p50": float(np.percentile(service, 50)), "p99": float(np.percentile(service, 99)),
                           "note": "device time of each solve inside the server"},
            "server": {"slots": st["slots"], "bytes": st["bytes"], "max_inflight_seen": max_inflight}}
    print(json.dumps(line), flush=True)


def run_large(args):
    """One large mesh on the cooperative grid (a secondary measurement; the
    headline is the batch): the permuted 122,880-cell backward-facing step
    (Re_h 36000, reference BFS settings, FP64 drop-in by default) or the
    permuted 2.05M-cell periodic square duct (20x320x320, Re_tau 600, mixed
    precision by default), a fixed number of outer iterations from the cold
    start.  Reports ms per outer iteration and cell-iterations/s from the
    launch's CUDA-event time."""
    import rans_sst_py as rs
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as tc
    if args.large == "bfs120k":
        m = rs.Mesh.make_backward_facing_step_2d(64, 384, 192, 96, 4.0, 30.0, 1.0, 3.0, 36000.0, 1.0)
        m = m.permuted(np.random.default_rng(7).permutation(m.n_cells()))
        nu = 1.0 / 36000.0
        k_in = 1.5 * 0.01 ** 2
        om_in = k_in / (100.0 * nu)
        bcs_fn = lambda mm: rs.FlowBoundaryConditions.bfs_defaults(mm, 1.0, k_in, om_in)  # noqa: E731
        s = tc.bfs_settings(args.large_iters, 0.0)
        init = dict(u=(1.0, 0.0, 0.0), p=0.0, k=k_in, omega=om_in)
        prec = args.large_precision or "fp64"
    else:
        ratio = tc.ratio_for_first_cell(1.0 / 600.0, 160)
        m = rs.Mesh.make_square_duct_periodic_3d(20, 320, 320, 10.0, 2.0, ratio)
        m = m.permuted(np.random.default_rng(17).permutation(m.n_cells()))
        nu = 1.0 / 600.0
        bcs_fn = lambda mm: rs.FlowBoundaryConditions.channel_defaults(mm, 0.0, 0.0, 0.0)  # noqa: E731
        s = tc.channel_settings(args.large_iters, 0.0)
        init = dict(u=(15.0, 0.0, 0.0), p=0.0, k=1e-2, omega=10.0)
        prec = args.large_precision or "mixed"
    m.compute_wall_distance(device=True)
    s.precision = prec
    case = rs.Case(m, bcs_fn(m), nu, s)
    out = rs.solve(case, tc.COEFF_DEFAULTS, 0, init, want_state=False)
    ms = lib_launch_ms()
    n_it = max(out.iterations_run, 1)
    peak, kind = measured_peaks()
    alg = algorithmic_bytes(m.n_cells(), n_it, out.inner_iterations, prec == "mixed")
    achieved = alg / (ms * 1e-3) / 1e9
    line = {"metric": "cell-iterations/s", "value": m.n_cells() * n_it / (ms * 1e-3), "unit": "cell-it/s",
            "higher_is_better": True, "n_gpus": 1, "dtype": "f64" if prec == "fp64" else "f32+f64",
            "data": "synthetic", "impl": "gb300",
            "config": {"workload": args.large, "cells": m.n_cells(), "outer_iterations": n_it, "precision": prec,
                       "start": "cold", "team": "cooperative grid"},
            "ms_per_outer_iteration": ms / n_it, "inner_split_per_outer": [v / n_it for v in out.inner_split],
            "launch_ms": ms,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": kind,
                         "note": "algorithmic bytes (per cell-iteration and per inner iteration, as the batch) "
                                 "over the launch time; the working set of one mesh is L2-resident up to ~150k "
                                 "cells and the V-cycle is grid-barrier bound"}}
    print(json.dumps(line), flush=True)


# The batched mixed-precision mesh mix: streamwise-periodic 4 x ny channels,
# first cell at y+ 0.4 except the 4x128 Re_tau 550 channel of the headline
# (ratio 1.08): (wall-normal cells, Re_tau, ratio).
C3_MESHES = [(64, 180.0, None), (128, 550.0, 1.08), (256, 1000.0, None), (512, 2000.0, None)]
C3_MAX_ITER = 200000
C3_FP64_CHECK = 2            # instances per mesh checked against the FP64 engine
C3_FP64_ITERS = 40000        # FP64 outer iterations continued from each checked mixed result


def run_c3(args):
    """The 256-theta draw spread over four channel meshes (theta i on mesh
    i mod 4; out-of-bounds draws are InvalidParameters and not solved), all
    valid instances in one call: cold starts to the 1e-8 scaled residual in
    the mixed engine.  Instances of different CTA sizes run as concurrent
    launches.  After the timed steps the first C3_FP64_CHECK instances of
    every mesh are continued by the FP64 engine for C3_FP64_ITERS iterations
    (convergence test off): the distance the FP64 iteration moves them is
    their distance to its fixed point where that iteration converges within
    the count (meshes up to Re_tau 1000 here; the reference algorithm does not
    converge on the Re_tau 2000 mesh from the cold start within 200k
    iterations)."""
    import rans_sst_py as rs
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import cases as tc
    _, coeffs, valid = theta_set()
    mesh_cases, by_mesh = [], []
    for ny, re, ratio in C3_MESHES:
        m, bcs, nu, init = tc.periodic_channel(ny, re, ratio=ratio)
        s = tc.channel_settings(C3_MAX_ITER, TOL)
        s.precision = "mixed"
        mesh_cases.append((m, bcs, nu, init, rs.Case(m, bcs, nu, s)))
    ids = [i for i in range(N_THETA) if valid[i]]
    tags = [i % len(C3_MESHES) for i in ids]
    batch = [mesh_cases[t][4] for t in tags]
    inits = [mesh_cases[t][3] for t in tags]
    cf = coeffs[ids]

    def step():
        t0 = time.perf_counter()
        outs = rs.solve_batch(batch, cf, None, inits, want_state=True)
        return outs, lib_launch_ms(), time.perf_counter() - t0

    for _ in range(args.warmup):
        step()
    dev_ms, wall_s = [], []
    with ClockSampler(sampled_gpu(0)) as clocks:
        for _ in range(args.steps):
            outs, ms, wall = step()
            dev_ms.append(ms)
            wall_s.append(wall)
    conv = sum(o.converged for o in outs)
    per_mesh = []
    for t, (ny, re, _) in enumerate(C3_MESHES):
        mo = [o for o, tg in zip(outs, tags) if tg == t]
        it = np.array([o.iterations_run for o in mo])
        fin = np.array([o.finish_ms for o in mo])
        per_mesh.append({"mesh": f"4x{ny}", "re_tau": re, "cells": mesh_cases[t][0].n_cells(), "instances": len(mo),
                         "converged": int(sum(o.converged for o in mo)), "iters_mean": float(it.mean()),
                         "iters_max": int(it.max()), "finish_ms_p50": float(np.percentile(fin, 50)),
                         "finish_ms_max": float(fin.max())})
    # FP64 continuation of the first instances of every mesh, one batch
    chk, chk_cases, chk_cf, chk_warm = [], [], [], []
    for t in range(len(C3_MESHES)):
        m, bcs, nu, _, _ = mesh_cases[t]
        s = tc.channel_settings(C3_FP64_ITERS, 0.0)
        c = rs.Case(m, bcs, nu, s)
        for j in [j for j, tg in enumerate(tags) if tg == t][:C3_FP64_CHECK]:
            chk.append((t, j))
            chk_cases.append(c)
            chk_cf.append(cf[j])
            chk_warm.append(outs[j].state)
    fps = rs.solve_batch(chk_cases, np.array(chk_cf), None, chk_warm, want_state=True)
    for (t, j), f in zip(chk, fps):
        d = {k: float(np.linalg.norm(outs[j].state[k] - f.state[k]) / np.linalg.norm(f.state[k]))
             for k in ("U", "k", "omega", "nuT")}
        per_mesh[t].setdefault("distance_to_fp64_continuation", []).append(d)
    step_ms = statistics.mean(dev_ms)
    line = {"metric": "converged RANS solves/sec", "value": conv / (step_ms * 1e-3), "unit": "solves/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic", "impl": "gb300",
            "config": {"workload": "c3_theta256_channels_4x64_128_256_512_re180_550_1000_2000", "precision": "mixed",
                       "n_theta": N_THETA, "n_valid": len(ids), "tol": TOL, "max_iterations": C3_MAX_ITER},
            "converged_per_step": int(conv),
            "e2e": {"value": conv / statistics.mean(wall_s), "unit": "solves/s"},
            "per_mesh": per_mesh, "clocks": clocks.summary(),
            "fp64_check": {"instances_per_mesh": C3_FP64_CHECK, "fp64_iterations": C3_FP64_ITERS,
                           "note": "relative L2 between each mixed result and the FP64 engine continued from it"}}
    print(json.dumps(line), flush=True)


def lib_launch_ms():
    from rans_sst_py._lib import lib
    return float(lib().btm_last_launch_ms())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--traffic", type=float, default=None, help="ncu DRAM bytes per launch, if measured")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-case", action="store_true",
                    help="one launch of 304 instances capped at 200 outer iterations (for ncu captures)")
    ap.add_argument("--profile-mesh", choices=["channel4x128", "bfs1920"], default="channel4x128",
                    help="--profile-case: the mesh")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"],
                    help="engine of the timed arm (mixed: the batched mixed-precision form)")
    ap.add_argument("--served", action="store_true",
                    help="the served-stream workload (continuous batching server) instead of the batch")
    ap.add_argument("--served-rate", type=float, default=SERVED_RATE, help="served stream: arrivals per second")
    ap.add_argument("--served-cases", choices=["small", "c4"], default="small",
                    help="served stream: the 4x32 channel / Couette, or the configuration's 2,048-cell cases "
                         "(c4: most requests start cold, as they arrive before their chain's previous solve "
                         "ends; expect well over 400 s on one GPU)")
    ap.add_argument("--no-fp64-compare", action="store_true",
                    help="skip the plain-FP64 launch of the same batch and the error report")
    ap.add_argument("--large", choices=["bfs120k", "duct2m"], default=None,
                    help="one large mesh on the cooperative grid instead of the batch")
    ap.add_argument("--large-iters", type=int, default=20, help="--large: outer iterations from the cold start")
    ap.add_argument("--large-precision", choices=["fp64", "mixed"], default=None,
                    help="--large: engine (default fp64 for bfs120k, mixed for duct2m)")
    ap.add_argument("--c3", action="store_true",
                    help="the 256-theta mesh mix over the 4x64/128/256/512 channels instead of the batch "
                         "(give --warmup 1: one step takes about a minute)")
    args = ap.parse_args()
    global PRECISION
    PRECISION = args.precision
    world, rank, local = dist_setup()
    if args.profile_case:
        run_profile_case(args.profile_mesh)
        return
    if args.c3:
        if rank == 0:
            run_c3(args)
        return
    if args.served:
        if rank == 0:
            run_served(args)
        return
    if args.large:
        if rank == 0:
            run_large(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
