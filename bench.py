"""Benchmark: one transport sweep (Epetra_Operator::Apply, y = x - D L^-1 M2D S x)
per step on the 2-D heterogeneous anisotropic workload -- 256 x 256 cells, DG Q2
(9 dofs/cell), level-symmetric S16 (144 directions), P3 scattering (10
moments), 8 x 8 seeded material blocks -- i.e. 9,437,184 cell-direction solves
per step.  Prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default): the GB300 operator through the C-ABI.
  value    = cell-direction solves/s over the timed steps, inputs resident in
             HBM, device time from CUDA events on the operator's stream, L2
             flushed (256 MiB write) before every step outside the timed span.
             FP64 arithmetic is the default double-float form ("arithmetic");
             fp64_native_apply times the same Apply in native FP64.
  e2e      = the same call with pinned host buffers (host->device copy of x and
             device->host copy of y inside the timed span), wall clock.
  roofline = the sweep kernel against measured HBM bandwidth, with the
             algorithmic bytes per solve of the sweep's face hand-off model;
             traffic from the ncu capture of the current sweep source, else null.
  cpu_baseline = the CPU restatement of the reference sweep (oracle/), all
             host threads, on the same workload and the same x (rank 0 at
             N = 1 only); the same leg checks the timed Apply's output against
             the oracle's (parity_rel_err) and solves the reduced thick map in
             FP64 for the time-to-solution error check.
  time_to_solution = time to a 1e-8 residual on the 64^3 thick map: plain FP64
             GMRES(30) against FGMRES(30) with FP32 sweeps and the diffusion
             synthetic acceleration, with its CG started from the trained
             network's prediction (the metric's learned leg) and from zero;
             scalar-flux errors against the FP64 solve and (on the reduced
             map) against the FP64 oracle.
--impl reference: the CPU restatement of the reference's sweep (the reference
  itself needs deal.II/Trilinos/p4est/MPI, absent here), all host threads,
  timed per step, on inputs from the oracle's own generator (nothing of the
  product is loaded).  Under torchrun only rank 0 runs it.

Multi-GPU: replicas only (each rank sweeps its own seeded problem, no
collective on the data path); value is the sum over ranks of solves divided by
the slowest rank's time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("time-to-1e-8 residual: learned+FP32 FGMRES vs plain FP64 GMRES; "
          "cell-dir solves/s")
UNIT = "cell-dir solves/s"
WORKLOAD = "2d-hetero-256x256-dgq2-ls16-p3"


WORKLOAD_ARGS = dict(seed=1001, n=256, fe_order=2, sn=16, l_max=3, blocks=8)


def workload_problem(seed=1001):
    import ouranos_gb300 as og
    return og.heterogeneous_2d(**dict(WORKLOAD_ARGS, seed=seed))


def workload_config(cells, directions, moments, dofs_per_cell, world):
    """The `config` object of both arms' lines (the same keys and values)."""
    return {"workload": WORKLOAD, "cells": cells, "directions": directions, "moments": moments,
            "dofs_per_cell": dofs_per_cell, "solves_per_step": cells * directions,
            "parallelism": "replicas" if world > 1 else "none"}


# DRAM traffic of one sweep launch on the default workload
# (dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of the
# default tiling, 16 x 1 cells with two lanes per cell, in the default FP64
# arithmetic and in FP32), keyed by a digest of the sweep kernel's sources at
# the time of the capture: after any change to those sources the figure no
# longer describes the kernel and the line reports traffic as null.
PROFILED_TILING = (16, 1, 1)
SWEEP_SOURCES = ("sweep.cuh", "sweep_df64.cu", "sweep_f32.cu", "df64.cuh")
SWEEP_TRAFFIC = {"digest": "67f909790da3fada", "bytes": {"fp64": 701016576 + 663608064}}


def sweep_source_digest():
    import hashlib
    h = hashlib.sha256()
    for name in SWEEP_SOURCES:
        with open(os.path.join(ROOT, "ouranos_gb300", "csrc", name), "rb") as f:
            h.update(name.encode() + f.read())
    return h.hexdigest()[:16]


def bytes_per_solve(prob, real_bytes=8):
    """Algorithmic HBM bytes per cell-direction solve: each outflow face value
    written once and read once downwind (2 * dim * fd values), the source and
    flux moments read and written once per sweep (amortised over the
    directions), and the 4-byte material id per cell (amortised)."""
    dim, n = prob.dim, prob.dofs_per_cell
    fd = (prob.fe_order + 1) ** (dim - 1)
    nd, nm = prob.quad.n_dir, prob.quad.n_mom
    return 2 * real_bytes * dim * fd + 2 * real_bytes * n * nm / nd + 4.0 / nd


def flops_per_solve(prob):
    dim, n = prob.dim, prob.dofs_per_cell
    fd = (prob.fe_order + 1) ** (dim - 1)
    nm = prob.quad.n_mom
    return 2 * n * n + 2 * dim * (fd * fd + fd) + 4 * n * nm


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def start(self, settle_s=3.0):
        """Start sampling and return once the first sample is in (or after
        settle_s): nvidia-smi's start-up, which can stall the GPU briefly,
        then happens before the timed region rather than inside it."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_id), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and time.time() - t0 < settle_s:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def faithful_scheduler_fit(target_tasks):
    """The reference's own task scheduler (src/RadiativeTransfer.cc:605-692:
    every get_next_task/send_angular_flux scans the task list, O(T^2) per
    sweep), restated in the oracle, timed single-threaded on small 2-D Q1 LS
    S8 meshes; the power law t = a T^k fitted to them is reported with the
    time it predicts for `target_tasks` -- a fitted figure, not a
    measurement."""
    import numpy as np
    import ouranos_gb300 as og
    from oracle import pyoracle
    pts = []
    for n in (8, 12, 16, 24):
        p = og.config_small(n=n, sn=8)
        O = pyoracle.OracleProblem(p.arrays())
        O.scattering_source(np.random.default_rng(n).standard_normal(O.length))
        t0 = time.perf_counter()
        O.sweep(scheduler=1, threads=1)
        pts.append((n * n * p.quad.n_dir, time.perf_counter() - t0))
    T = np.log([t for t, _ in pts])
    S = np.log([s for _, s in pts])
    k, loga = np.polyfit(T, S, 1)
    return {"tasks": [int(t) for t, _ in pts], "seconds": [round(s, 4) for _, s in pts],
            "fit": "t = a T^k", "k": round(float(k), 3),
            "predicted_seconds_per_sweep_of_this_workload": float(np.exp(loga) * target_tasks ** k),
            "note": "fitted to the small meshes, not measured at this size"}


def single_core_rate():
    """The linear-scheduler port on one core: one Apply of the bench
    workload's physics on a 64 x 64 mesh (590 k solves) -- the per-solve
    rate, whose mesh dependence is only the scheduler's linear bookkeeping."""
    import ouranos_gb300 as og
    p = og.heterogeneous_2d(seed=1001, n=64, fe_order=2, sn=16, l_max=3, blocks=8)
    rate, times = cpu_reference_rate(p, 1, reps=1)
    return {"value": rate, "unit": UNIT, "cores": 1,
            "sample": "one Apply of the same physics on 64 x 64 cells (%.2f s)" % times[0]}


def cpu_reference_rate(prob, threads, reps=1):
    """The reference's sweep restated on the CPU (oracle/), all threads."""
    import numpy as np
    from oracle import pyoracle
    O = pyoracle.OracleProblem(prob.arrays())
    x = np.random.default_rng(0).standard_normal(prob.vector_length)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        O.apply(x, threads=threads)
        times.append(time.perf_counter() - t0)
    solves = prob.total_cells * prob.quad.n_dir
    return solves / (sum(times) / len(times)), times


def run_reference(args):
    """The reference's sweep restated on the CPU (the oracle, all host
    threads), one full sweep of the workload per step.  Its inputs come from
    the oracle's own generator (oracle/workloads.py), so this arm loads
    nothing of the product."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    import numpy as np
    from oracle import pyoracle, workloads
    spec = workloads.heterogeneous_2d(**WORKLOAD_ARGS)
    threads = os.cpu_count() or 1
    O = pyoracle.OracleProblem(spec)
    x = np.random.default_rng(0).standard_normal(workloads.vector_length(spec))
    for _ in range(args.warmup):
        O.apply(x, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.apply(x, threads=threads)
    dt = time.perf_counter() - t0
    cells = int(np.prod(spec["n_cells"]))
    nd, nm = spec["m2d"].shape
    n = (spec["fe_order"] + 1) ** spec["dim"]
    solves = cells * nd
    value = solves * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "arithmetic": "FP64",
        "data": "synthetic (seeded SplitMix64 material map, random flux moments)",
        "config": workload_config(cells, nd, nm, n, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "full sweep of the workload per step (oracle/ C++ restatement "
                                   "of src/RadiativeTransfer.cc sweep + Crout LU, linear "
                                   "ready-counter scheduler, directions split over threads)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_leg(prob, x, y_device, y_host, threads, reps, solve_check):
    """The CPU baseline, and the oracle as the checker of what the GPU arm
    computed (outside every timed region):
      - the oracle's sweep timed on all host cores over `reps` full sweeps of
        the workload, its result compared with the GPU Apply of the same x
        (the device-vector and the host-vector call);
      - the reference scheduler's O(T^2) fit and the single-core rate;
      - with solve_check, the FP64 oracle solve of a reduced thick map that
        the time-to-solution figures are checked against."""
    import numpy as np
    from oracle import pyoracle
    O = pyoracle.OracleProblem(prob.arrays())
    times, y_ref = [], None
    for _ in range(reps):
        t0 = time.perf_counter()
        y_ref = O.apply(x, threads=threads)
        times.append(time.perf_counter() - t0)
    solves = prob.total_cells * prob.quad.n_dir
    rate = solves / (sum(times) / len(times))
    out = {"cpu": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": "%d full sweep(s) of the workload (%.1f s of CPU work) with the oracle/ C++ "
                             "restatement of the reference sweep, directions split over threads"
                             % (len(times), sum(times)),
                   "faithful_scheduler": faithful_scheduler_fit(solves),
                   "single_core": single_core_rate()},
           "parity": {"rel_err": rel_l2(y_device, y_ref), "rel_err_e2e": rel_l2(y_host, y_ref),
                      "bound": 1e-12, "against": "oracle FP64 Apply of the same x"}}
    if solve_check:
        out["oracle_solve"] = oracle_reduced_solve(solve_check, threads)
    return out


def rel_l2(a, b):
    import numpy as np
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def oracle_reduced_solve(args, threads):
    """FP64 GMRES(30) of the oracle to a 1e-10 residual on the reduced thick
    map (the same seed, material distribution and quadrature as the
    time-to-solution workload, n^3 cells)."""
    import ouranos_gb300 as og
    from oracle import pyoracle
    prob = og.thick_3d(seed=args["seed"], n=args["n"], sn=12)
    O = pyoracle.OracleProblem(prob.arrays(), order="cartesian")
    t0 = time.perf_counter()
    x, it, _ = O.solve("gmres", tol=1e-10, max_it=5000, restart=30, threads=threads)
    return {"n": args["n"], "seed": args["seed"], "iterations": int(it), "seconds": time.perf_counter() - t0,
            "tol": 1e-10, "solution": x}


def replica_max(values, dist, device):
    """Each figure's maximum over the ranks (the slowest replica bounds the
    whole job); every rank gets the same numbers.  dist None: one process."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job_rate(world, units_per_rank, seconds):
    """Units all ranks processed (each the same work) over the job's time."""
    return world * units_per_rank / seconds


def run_ours(args):
    import numpy as np
    import torch
    import ouranos_gb300 as og

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    prob = workload_problem(seed=1001 + rank)
    rt = og.RadiativeTransfer(prob, device=local, precision=args.precision)
    if args.precision == "fp32":
        rt.set_fp32_contractions(args.fp32_contractions)
    else:
        rt.set_fp64_contractions(args.fp64_contractions)
    stream = torch.cuda.current_stream(dev)
    rt.set_stream(stream.cuda_stream)
    L = prob.vector_length
    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    x = torch.randn(L, dtype=torch.float64, device=dev, generator=gen)
    y = torch.empty_like(x)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    solves = prob.total_cells * prob.quad.n_dir

    for _ in range(max(args.warmup, 3)):
        rt.Apply(x, y)
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    props = torch.cuda.get_device_properties(dev)
    uid = str(getattr(props, "uuid", "") or "")
    sampler = ClockSampler(("GPU-" + uid if uid and not uid.startswith("GPU-") else uid) or local)
    sampler.start()
    step_ms, sweep_ms = [], []
    launches = 0
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    for _ in range(args.steps):
        flush.zero_()                      # L2 flush, outside the timed span
        ev0.record(stream)
        rt.Apply(x, y)
        ev1.record(stream)
        ev1.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
        ms, k = rt.last_sweep_ms()
        sweep_ms.append(ms)
        launches += k  # the Apply's kernels, as the library counts them
    torch.cuda.synchronize(dev)
    clocks = sampler.stop()
    total_ms = replica_max([sum(step_ms)], dist, dev)[0]
    if dist:
        dist.barrier()
    value = whole_job_rate(world, solves * args.steps, total_ms / 1e3)

    # end-to-end through the C-ABI with pinned host buffers
    xh = x.cpu().pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    rt.set_stream(None)
    rt.Apply(xh, yh)
    e2e_times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rt.Apply(xh, yh)
        e2e_times.append(time.perf_counter() - t0)
    e2e_total = replica_max([sum(e2e_times)], dist, dev)[0]
    e2e_value = whole_job_rate(world, solves * args.steps, e2e_total)
    if not np.isfinite(yh.numpy()).all():
        raise RuntimeError("non-finite operator output")

    # the same Apply with native FP64 arithmetic (the double-float default is
    # the line's value), a few steps timed the same way
    native = None
    if args.precision == "fp64":
        rt.set_stream(stream.cuda_stream)
        rt.set_fp64_contractions("native")
        for _ in range(3):
            rt.Apply(x, y)
        nms = []
        for _ in range(max(3, min(args.steps, 10))):
            flush.zero_()
            ev0.record(stream)
            rt.Apply(x, y)
            ev1.record(stream)
            ev1.synchronize()
            nms.append(ev0.elapsed_time(ev1))
        native = {"ms_per_step": sum(nms) / len(nms), "value": solves / (sum(nms) / len(nms) / 1e3),
                  "unit": UNIT, "steps": len(nms)}
        # the double-float Apply with its two contractions on the CUDA cores
        # and on the tensor cores (exact BF16 digit products)
        engines = {}
        for mode, key in (("df64_sweep", "cuda_cores"), ("df64_sweep_tc", "tensor")):
            try:
                rt.set_fp64_contractions(mode)
            except Exception as exc:  # more directions or moments than the tensor form takes
                engines[key] = {"unavailable": str(exc)}
                continue
            for _ in range(3):
                rt.Apply(x, y)
            ems = []
            for _ in range(max(3, min(args.steps, 10))):
                flush.zero_()
                ev0.record(stream)
                rt.Apply(x, y)
                ev1.record(stream)
                ev1.synchronize()
                ems.append(ev0.elapsed_time(ev1))
            engines[key] = {"ms_per_step": sum(ems) / len(ems), "value": solves / (sum(ems) / len(ems) / 1e3),
                            "unit": UNIT, "steps": len(ems)}
        native["fp64_contractions"] = engines
        rt.set_fp64_contractions(args.fp64_contractions)
        rt.Apply(x, y)
        torch.cuda.synchronize(dev)
        # the FP32 Apply (the Arnoldi operator of the mixed-precision solves)
        # with its contractions on the CUDA cores and on the tensor cores
        fp32 = {}
        rt.set_precision("fp32")
        for mode in ("cuda_cores", "tensor"):
            rt.set_fp32_contractions(mode)
            for _ in range(3):
                rt.Apply(x, y)
            fms, fsw = [], []
            for _ in range(max(3, min(args.steps, 10))):
                flush.zero_()
                ev0.record(stream)
                rt.Apply(x, y)
                ev1.record(stream)
                ev1.synchronize()
                fms.append(ev0.elapsed_time(ev1))
                fsw.append(rt.last_sweep_ms()[0])
            fp32[mode] = {"ms_per_step": sum(fms) / len(fms), "value": solves / (sum(fms) / len(fms) / 1e3),
                          "sweep_ms": sum(fsw) / len(fsw), "unit": UNIT, "steps": len(fms)}
        rt.set_precision("fp64")
        rt.Apply(x, y)
        torch.cuda.synchronize(dev)
        native["fp32_apply"] = fp32

    peak, peak_kind = measured_peaks()
    # the captured configuration only: default seed, tiling and FP64 arithmetic,
    # and the sweep sources unchanged since the capture
    digest = sweep_source_digest()
    profiled = (rank == 0 and rt.tiling() == PROFILED_TILING and world == 1)
    fresh = digest == SWEEP_TRAFFIC["digest"]
    traffic = SWEEP_TRAFFIC["bytes"].get(args.precision) if (profiled and fresh) else None
    rb = 8 if args.precision == "fp64" else 4
    bps = bytes_per_solve(prob, rb)
    avg_sweep_s = sum(sweep_ms) / len(sweep_ms) / 1e3
    achieved = bps * solves / avg_sweep_s / 1e9
    fps = flops_per_solve(prob)

    cpu = None
    parity = None
    oracle_solve = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        leg = cpu_baseline_leg(prob, x.cpu().numpy(), y.cpu().numpy(), yh.numpy(), threads,
                               max(1, args.cpu_reps),
                               None if args.no_solve else {"seed": args.solve_seed, "n": args.oracle_n})
        cpu, parity, oracle_solve = leg["cpu"], leg["parity"], leg.get("oracle_solve")
    tts = None
    if rank == 0 and world == 1 and not args.no_solve:
        tts = time_to_solution(args.solve_seed, args.solve_n, args.tol, args.dsa_cg, args.max_it, oracle_solve)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32",
            "arithmetic": (("double-float (FP32 pairs, ~48-bit significand) sweep; contractions on the tensor "
                            "cores as exact BF16 digit products; FP64 vectors"
                            if args.fp64_contractions == "df64_sweep_tc" else
                            "double-float (FP32 pairs, ~48-bit significand) sweep and contractions, FP64 vectors")
                           if args.precision == "fp64" else "FP32 sweep, FP64 vectors"),
            "data": "synthetic (seeded SplitMix64 material map, random flux moments)",
            "config": workload_config(prob.total_cells, prob.quad.n_dir, prob.quad.n_mom,
                                      prob.dofs_per_cell, world),
            "timing": {"l2": "flushed (256 MiB write) before every timed step",
                       "tiling": list(rt.tiling()), "events": "CUDA events on the operator's stream"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * L,
                    "d2h_bytes_per_step": 8 * L},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": traffic,
                         "traffic_source": ("ncu capture of this kernel source (digest %s)" % digest
                                            if traffic is not None else
                                            "none: sweep sources (digest %s) differ from the last capture "
                                            "(%s) or the run is not the captured configuration"
                                            % (digest, SWEEP_TRAFFIC["digest"])),
                         "peak_kind": peak_kind, "bytes_per_solve": bps,
                         "sweep_ms": avg_sweep_s * 1e3,
                         "fp_flops_per_solve": fps,
                         "fp_tflops": fps * solves / avg_sweep_s / 1e12},
            "gpu_launches": launches,
            "clocks": clocks,
        }
        if native:
            line["fp32_apply"] = native.pop("fp32_apply")
            line["fp64_contractions"] = native.pop("fp64_contractions")
            line["fp64_native_apply"] = native
        if parity:
            line["parity_rel_err"] = parity["rel_err"]
            line["parity"] = parity
        if cpu:
            line["cpu_baseline"] = cpu
        if tts:
            line["time_to_solution"] = tts
        print(json.dumps(line), flush=True)
    rt.close()
    if dist:
        dist.destroy_process_group()


def flux_errors(x, ref, n0):
    """Scalar-flux (moment 0) relative L2 and relative max error of x against ref."""
    import numpy as np
    a, b = np.asarray(x)[:n0], np.asarray(ref)[:n0]
    return {"rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
            "rel_max": float(np.abs(a - b).max() / np.abs(b).max())}


LEARNED_WEIGHTS = os.path.join(ROOT, "ouranos_gb300", "weights", "dsa_guess_thick3d.npz")
LEARNED_CG = 3  # CG steps of the diffusion correction in the learned leg (and its comparison)


def time_to_solution(seed, n, tol, dsa_cg, max_it, oracle_solve=None, learned_cg=LEARNED_CG):
    """Time to a `tol` relative residual on the 3-D thick diffusive map (n^3
    hexes, DG Q1, GLC S12), every method FGMRES(30)/GMRES(30) on the device:
      fp64_gmres              plain FP64 GMRES (the reference's method);
      fp32_fgmres_learned_dsa FP32 sweeps, FP64 restarts, right preconditioner
                              the diffusion correction with learned_cg CG steps
                              started from the trained network's prediction;
      fp32_fgmres_dsa_same_cg the same without the network (zero start);
      fp32_fgmres_dsa         the same with dsa_cg CG steps.
    Wall time of each ouranos_solve call (right-hand side, solve and final
    FP64 residual), iterations, final FP64 residual.  Scalar-flux errors: at
    n^3 against the GPU's FP64 GMRES solve; and, when the CPU leg has solved
    the reduced map of the same seed with the FP64 oracle, every method on that
    map against the oracle."""
    import ouranos_gb300 as og
    from ouranos_gb300.learned import Network, install
    if not os.path.exists(LEARNED_WEIGHTS):
        raise FileNotFoundError("trained network weights missing: %s" % LEARNED_WEIGHTS)
    prob = og.thick_3d(seed=seed, n=n, sn=12)
    out = {"workload": "3d-thick-%d^3-dgq1-glc12-seed%d" % (n, seed), "tol": tol, "dsa_cg_steps": dsa_cg,
           "learned_cg_steps": learned_cg, "learned_weights": os.path.relpath(LEARNED_WEIGHTS, ROOT),
           "cell_dir_solves_per_sweep": prob.total_cells * prob.quad.n_dir}
    keys = ("seconds", "iterations", "restarts", "residual", "converged")

    def run_all(rt, grid):
        sols, infos = {}, {}
        net = Network.load(LEARNED_WEIGHTS, grid)
        try:
            sols["fp64_gmres"], infos["fp64_gmres"], _ = rt.solve("gmres", tol=tol, max_it=max_it, restart=30)
            rt.set_dsa(dsa_cg)
            sols["fp32_fgmres_dsa"], infos["fp32_fgmres_dsa"], _ = rt.solve(
                "fgmres_mixed", tol=tol, max_it=max_it, restart=30, dsa=True)
            rt.set_dsa(learned_cg)
            sols["fp32_fgmres_dsa_same_cg"], infos["fp32_fgmres_dsa_same_cg"], _ = rt.solve(
                "fgmres_mixed", tol=tol, max_it=max_it, restart=30, dsa=True)
            install(rt, net)
            sols["fp32_fgmres_learned_dsa"], infos["fp32_fgmres_learned_dsa"], _ = rt.solve(
                "fgmres_learned", tol=tol, max_it=max_it, restart=30, dsa=True)
            install(rt, None)
        finally:
            net.close()
        return sols, infos

    with og.RadiativeTransfer(prob) as rt:
        sols, infos = run_all(rt, (n, n, n))
    n0 = prob.total_cells * prob.dofs_per_cell
    for name, info in infos.items():
        out[name] = {k: info[k] for k in keys}
        if name != "fp64_gmres":
            out[name]["flux_vs_gpu_fp64"] = flux_errors(sols[name], sols["fp64_gmres"], n0)
            out[name]["speedup_vs_fp64_gmres"] = infos["fp64_gmres"]["seconds"] / info["seconds"]
    out["speedup"] = out["fp32_fgmres_learned_dsa"]["speedup_vs_fp64_gmres"]
    out["learned_gain_same_cg"] = {
        "iterations": [infos["fp32_fgmres_dsa_same_cg"]["iterations"], infos["fp32_fgmres_learned_dsa"]["iterations"]],
        "seconds": [infos["fp32_fgmres_dsa_same_cg"]["seconds"], infos["fp32_fgmres_learned_dsa"]["seconds"]]}
    if oracle_solve is not None:
        m = oracle_solve["n"]
        small = og.thick_3d(seed=oracle_solve["seed"], n=m, sn=12)
        ref = oracle_solve["solution"]
        m0 = small.total_cells * small.dofs_per_cell
        check = {"workload": "3d-thick-%d^3-dgq1-glc12-seed%d" % (m, oracle_solve["seed"]),
                 "oracle": {k: oracle_solve[k] for k in ("iterations", "seconds", "tol")}}
        with og.RadiativeTransfer(small) as rt:
            ssols, sinfos = run_all(rt, (m, m, m))
        for name, info in sinfos.items():
            check[name] = dict(flux_errors(ssols[name], ref, m0), iterations=info["iterations"],
                               residual=info["residual"])
        out["vs_fp64_oracle"] = check
    return out


def run_solve(args):
    """Time to a 1e-8 relative residual on the 3-D thick diffusive workload
    (64^3 hexes, DG Q1, GLC S12 = 168 directions, 4^3-cell blocks of
    (sigma_t, c) = (100, 0.999) or (1, 0.9)): plain FP64 GMRES(30) against
    FGMRES(30) with FP32 sweeps and FP64 refinement, each also with the
    diffusion synthetic acceleration as right preconditioner ("+dsa").  Reports wall time,
    iterations, the FP64 true residual and the scalar-flux error of the mixed
    solve against the FP64 solve."""
    import numpy as np
    import ouranos_gb300 as og
    n = args.solve_n
    prob = og.thick_3d(seed=args.solve_seed, n=n, sn=12)
    out = {"workload": "3d-thick-%d^3-dgq1-glc12" % n, "tol": args.tol}
    with og.RadiativeTransfer(prob) as rt:
        res = {}
        methods = args.methods.split(",")
        if any(m.startswith("fgmres_learned") for m in methods):
            from ouranos_gb300.learned import Network, install
            install(rt, Network.load(LEARNED_WEIGHTS, (n, n, n)))
            out["learned_weights"] = os.path.relpath(LEARNED_WEIGHTS, ROOT)
        if any(m.endswith("+dsa") for m in methods):
            rt.set_dsa(args.dsa_cg)
            out["dsa_cg_steps"] = args.dsa_cg
        for method in methods:
            base, dsa = (method[:-4], True) if method.endswith("+dsa") else (method, False)
            x, info, hist = rt.solve(base, tol=args.tol, max_it=args.max_it, restart=30, dsa=dsa)
            res[method] = (x, info)
            out[method] = {k: info[k] for k in ("iterations", "restarts", "residual", "seconds",
                                                "converged")}
        if "gmres" in res:
            ref = res["gmres"][0]
            n0 = prob.total_cells * prob.dofs_per_cell
            for m, (x, info) in res.items():
                if m != "gmres":
                    out[m]["flux_vs_gpu_fp64"] = flux_errors(x, ref, n0)
                    out[m]["speedup_vs_fp64_gmres"] = res["gmres"][1]["seconds"] / info["seconds"]
    print(json.dumps({"solve": out}), flush=True)


def run_batch(args):
    """Batched uneven workload: `count` independent 2-D problems (side drawn
    from {32, 64, 128, 256, 512}, DG Q1 or Q2, LS S4/S8/S12/S16, P1 scattering
    with g ~ U[0, 0.8], seeded material maps) behind one batch handle.  Times
    the batched FP32 Apply (one persistent sweep launch per class, replayed
    from a CUDA graph) on device vectors and through host vectors, then solves
    every problem to `tol` with FP32 Arnoldi sweeps and FP64 restarts and with
    the plain FP64 method."""
    import time
    import numpy as np
    import torch
    import ouranos_gb300 as og
    probs = og.batch_2d(seed=args.batch_seed, count=args.batch_count)
    solves = int(sum(p.total_cells * p.quad.n_dir for p in probs))
    t0 = time.perf_counter()
    b = og.Batch(probs)
    t_create = time.perf_counter() - t0
    t0 = time.perf_counter()
    tiling = b.autotune(reps=2)
    t_tune = time.perf_counter() - t0
    x = torch.randn(b.length, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)

    def timed(fn, steps):
        for _ in range(max(args.warmup, 3)):
            fn()
        torch.cuda.synchronize()
        t = []
        for _ in range(steps):
            t0 = time.perf_counter()
            fn()  # returns after its result is written
            t.append(time.perf_counter() - t0)
        return 1e3 * sum(t) / len(t)

    ms_graph = timed(lambda: b.apply(x, "fp32", out=y), args.steps)
    sweep_ms, graph_launches = b.stats()
    b.set_graphs(False)
    ms_eager = timed(lambda: b.apply(x, "fp32", out=y), max(3, args.steps // 4))
    b.set_graphs(True)
    xh = x.cpu().numpy()
    yh = np.empty_like(xh)
    ms_host = timed(lambda: b.apply(xh, "fp32", out=yh), max(3, args.steps // 4))
    out = {
        "metric": "batched FP32 Apply throughput, %d uneven 2-D problems" % len(probs),
        "value": solves / (ms_graph * 1e-3), "unit": "cell-dir solves/s",
        "ms_per_apply": ms_graph, "ms_per_apply_no_graph": ms_eager, "ms_per_apply_host_vectors": ms_host,
        "sweep_ms_last": sweep_ms, "graph_launches": graph_launches,
        "config": {"workload": "batch-2d-%d-seed%d" % (len(probs), args.batch_seed),
                   "cell_dir_solves_per_apply": solves, "vector_length": int(b.length),
                   "create_s": t_create, "autotune_s": t_tune,
                   "tilings": {"%dx%d/%d" % tuple(t): int(c) for t, c in
                               zip(*np.unique(tiling, axis=0, return_counts=True))}},
    }
    if args.batch_solve:
        res = {}
        b.set_dsa(args.dsa_cg)
        for name, inner, dsa in (("fp32", "fp32", False), ("fp64", "fp64", False), ("fp32+dsa", "fp32", True)):
            xs, infos = b.solve(inner=inner, tol=args.tol, max_it=args.max_it, dsa=dsa)
            res[name] = (xs.copy(), infos)
            its = [i["iterations"] for i in infos]
            out["solve_" + name] = {"seconds": infos[0]["seconds"], "converged": sum(i["converged"] for i in infos),
                                    "iterations_max": max(its), "iterations_mean": float(np.mean(its)),
                                    "residual_max": max(i["residual"] for i in infos)}
        x64 = res["fp64"][0]
        for name in ("fp32", "fp32+dsa"):
            out["solve_" + name]["flux_rel_l2_vs_fp64_max"] = max(
                float(np.linalg.norm(a - c) / max(np.linalg.norm(c), 1e-300))
                for a, c in zip(b.slices(res[name][0]), b.slices(x64)))
            out["solve_" + name]["speedup_vs_fp64"] = out["solve_fp64"]["seconds"] / out["solve_" + name]["seconds"]
    b.close()
    print(json.dumps(out), flush=True)


def run_time(args):
    """3-D time-dependent workload: [0,20]^3, 128^3 hexes, DG Q1, LS S8 (80
    directions), implicit Euler with 1/(v dt) = 0.5, a Gaussian pulse
    (peak 10 at step 20, width 5 steps) in a seeded 8^3-cell box, two-material
    map.  Every step is solved to `tol` by FGMRES with FP32 sweeps and FP64
    restarts (and the diffusion acceleration unless --time-no-dsa),
    warm-started from the previous step; phi and psi^n (FP32) stay on the
    device.  The first `time_compare` steps are repeated with plain FP64
    GMRES."""
    import time
    import numpy as np
    import ouranos_gb300 as og
    prob = og.time_dependent_3d(seed=args.time_seed, n=args.time_n)
    inv_vdt = prob.meta["inv_vdt"]
    out = {"workload": "3d-td-%d^3-dgq1-ls8-%dsteps" % (args.time_n, args.time_steps), "tol": args.tol,
           "inv_vdt": inv_vdt}

    import torch

    def run(method, steps, dsa=False):
        with og.RadiativeTransfer(prob) as rt:
            rt.set_time_step(inv_vdt)
            if dsa:
                rt.set_dsa(args.dsa_cg)
            # phi stays on the device between steps (each call takes and returns device vectors)
            phi = torch.zeros(rt.length, dtype=torch.float64, device="cuda")
            its, secs = [], []
            t0 = time.perf_counter()
            for n in range(steps):
                rt.set_source([[0.0], [og.pulse_strength(n)]])
                info = rt.time_advance(phi, method=method, tol=args.tol, max_it=args.max_it, dsa=dsa)
                its.append(info["iterations"])
                secs.append(info["seconds"])
            wall = time.perf_counter() - t0
            return phi.cpu().numpy(), its, secs, wall

    dsa = not args.time_no_dsa
    main_name = "fgmres_mixed+dsa" if dsa else "fgmres_mixed"
    phi, its, secs, wall = run("fgmres_mixed", args.time_steps, dsa)
    out[main_name] = {"wall_s": wall, "s_per_step": wall / args.time_steps,
                           "iterations_total": int(sum(its)), "iterations_max": int(max(its)),
                           "iterations_at_peak": int(its[min(20, len(its) - 1)]),
                           "scalar_flux_max_final": float(phi.max())}
    if args.time_compare:
        k = min(args.time_compare, args.time_steps)
        p32, i32, s32, w32 = run("fgmres_mixed", k, dsa)
        p64, i64, s64, w64 = run("gmres", k)
        out["compare_first_steps"] = {
            "steps": k, main_name + "_s": w32, "gmres_fp64_s": w64, "speedup": w64 / w32,
            "iterations_" + main_name: int(sum(i32)), "iterations_fp64": int(sum(i64)),
            "flux_rel_l2_vs_fp64": float(np.linalg.norm(p32 - p64) / max(np.linalg.norm(p64), 1e-300))}
        if dsa:
            pm, im_, sm, wm = run("fgmres_mixed", k)
            out["compare_first_steps"].update({"fgmres_mixed_s": wm, "iterations_fgmres_mixed": int(sum(im_))})
    print(json.dumps({"time": out}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--fp32-contractions", default="cuda_cores", choices=["cuda_cores", "tensor"],
                    help="where an FP32 run's moment/direction contractions run")
    ap.add_argument("--fp64-contractions", default="df64_sweep", choices=["df64_sweep", "df64_sweep_tc"],
                    help="where the double-float Apply's two contractions run: CUDA cores or tensor cores")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-reps", type=int, default=14, help="full CPU sweeps timed (~10 s on 16 cores)")
    ap.add_argument("--no-solve", action="store_true",
                    help="skip the time-to-solution comparison of the default line")
    ap.add_argument("--solve", action="store_true", help="time-to-solution mode")
    ap.add_argument("--solve-n", type=int, default=64)
    ap.add_argument("--solve-seed", type=int, default=7000, help="evaluation map (training uses 2000+)")
    ap.add_argument("--oracle-n", type=int, default=16,
                    help="side of the reduced thick map solved by the FP64 oracle for the error check")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-it", type=int, default=3000)
    ap.add_argument("--methods", default="gmres,fgmres_mixed,gmres+dsa,fgmres_mixed+dsa,fgmres_learned+dsa")
    ap.add_argument("--dsa-cg", type=int, default=20, help="CG steps of the diffusion correction")
    ap.add_argument("--batch", action="store_true", help="batched uneven 2-D workload")
    ap.add_argument("--batch-count", type=int, default=64)
    ap.add_argument("--batch-seed", type=int, default=3000)
    ap.add_argument("--batch-solve", action="store_true")
    ap.add_argument("--time", action="store_true", help="time-dependent 3-D workload")
    ap.add_argument("--time-n", type=int, default=128)
    ap.add_argument("--time-steps", type=int, default=100)
    ap.add_argument("--time-seed", type=int, default=4000)
    ap.add_argument("--time-compare", type=int, default=5)
    ap.add_argument("--time-no-dsa", action="store_true", help="steps without the diffusion acceleration")
    args = ap.parse_args()
    if args.time:
        import __graft_entry__
        __graft_entry__.build()
        run_time(args)
        return
    if args.batch:
        import __graft_entry__
        __graft_entry__.build()
        run_batch(args)
        return
    if args.solve:
        import __graft_entry__
        __graft_entry__.build()
        run_solve(args)
        return
    if args.impl == "reference":
        import importlib.util
        spec = importlib.util.spec_from_file_location("_ob", os.path.join(ROOT, "oracle", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
        run_reference(args)
    else:
        import __graft_entry__
        __graft_entry__.build()
        run_ours(args)


if __name__ == "__main__":
    main()
