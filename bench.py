"""Benchmark: ECP shell-pair integrals/s on the batched 50-centre cluster.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--mode batched|fp64] [--workload cluster|mixed_batch|sweep|...]
                    [--serve-rate R] [--serve-seconds S] [--serve-mixed-seconds S]
                    [--mixed-report 0|1] [--compare-plain 0|1]

Workload (per rank, default): the batched cluster -- 50 ECP centres (L up to
4, 2-6 terms per channel), 63 contracted shells (l = 0..3 with weights
.4/.3/.2/.1, contraction 1..8) giving 2016 shell pairs, i.e. 100,800
(shell pair, centre) units of which the screening keeps ~91k.  A step is one
pass of the whole getIntegrals path over that job: shell radii, centre
potentials, angular tables, F tables, every unit's type-1 and type-2 block,
and the AO-matrix scatter.  The unit of the metric is one emitted unit (a
type-1 + type-2 block pair handed to the reference's callback).  The other
workloads (--workload) are the 20,000-pair mixed batch and the 100,000-pair
high-accuracy sweep.

Path: the batched FP64 engine (ECPGB_FAST) by default -- the autotuner picks
its launch configuration first (including per-(la, lb)-class settings), then
the job replays as a captured CUDA graph; the plain FP64 drop-in kernels
(ECPGB_FP64) run two steps on the same job for the batched / plain ratio.

value   : device-resident job (inputs in HBM before the timed region); per step
          CUDA events on the engine's stream; L2 flushed (256 MiB write) between
          steps, outside the timed spans.
e2e     : ecpgb_getIntegrals (the getIntegrals call with the path chosen) with
          host buffers: one packed H2D copy of the inputs and a D2H copy of the
          matrix per step.
roofline: the unit kernel against the FP64 FMA pipe measured live (the path is
          FP64-latency bound; DRAM traffic is a few hundred bytes per unit):
          achieved = FP64 operations the kernel executed per emitted unit (ncu
          counts on the cluster's first 8 centres, profiles/roofline_inputs.txt;
          cluster workload only) x emitted units / the unit kernel's CUDA-event
          time; alg_* = the reference's algorithmic FLOPs counted by the oracle
          on its control flow over the CPU-baseline sample.
cpu_baseline: the oracle restatement (or the reference build where one exists
          on the machine) on a bounded sample of the workload, on all host cores
          the process may use and on one core.
mixed_precision: the mixed-precision engine on the same job: speed, its error
          against the plain FP64 path over every unit, and per L class against
          the oracle on the job's first two ECP centres.
serving : Poisson streams of molecules through the request server (continuous
          batching) near one GPU's capacity, FP64 and mixed precision, latency
          percentiles from the server's own clock.
Multi-GPU: weak scaling, one independent cluster per rank (seed = rank), no
          collective on the data path; max over ranks of the timed span.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ECP shell-pair integrals/s"
UNIT = "integrals/s"
WORKLOAD = "batched_cluster: 50 ECP centres x 2016 shell pairs (63 shells, l<=3, K 1-8), FP64"

# Algorithmic FLOP weights of the reference control flow, counted by the oracle:
# 4 per quadrature point, Bessel 30 per row + 80 per call, exp 20, table 3 per
# row, 2 per contraction multiply-add.
def algorithmic_flops(st: dict) -> float:
    return (4.0 * (st["ps93_points"] + st["psm92_points"]) + 33.0 * st["bessel_rows"]
            + 80.0 * st["bessel_calls"] + 20.0 * st["exp_calls"] + 2.0 * st["contraction_fma"])


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows if len(r) >= 8
                          for n, v in zip(names, r[4:8]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


# the workloads: name -> (description, builder)
WORKLOADS = {
    "cluster": WORKLOAD,
    "cluster8": WORKLOAD + " [first 8 centres]",
    "mixed_batch": "mixed_batch: 200 shells (20,100 pairs, l<=4, K 1-10, exponents 0.02-200) x 10 ECP centres, FP64",
    "sweep": "large_sweep: 447 shells (99,681 pairs, l<=4, K 1-6, exponents 0.01-500) x 4 ECP centres "
             "(L<=5, 6 terms), tolerance 1e-12, FP64",
}


def cpu_sample_system(system, workload="cluster"):
    """Bounded CPU sample of the workload (the port's time per unit is
    extrapolated to the whole job)."""
    centres = [a for a in range(system.n_atoms) if system.shellsECP[a] > 0]
    if workload in ("cluster", "cluster8"):
        return system.subset(centres=centres[:16], basis_atoms=range(11)), \
            "16 of 50 centres x 561 pairs (basis atoms 0-10) of the same cluster"
    if workload == "mixed_batch":
        return system.subset(centres=centres[:2], basis_atoms=range(12)), \
            "2 of 10 centres x the shells of atoms 0-11 of the same batch"
    return system.subset(centres=centres[:1], basis_atoms=range(12)), \
        "1 of 4 centres x the shells of atoms 0-11 of the same sweep"


_REF_CHILD = """
import json, sys, time, concurrent.futures as cf
sys.path.insert(0, {root!r})
from oracle import oracle as O
import bench
from libecp_gb300 import workloads as W
sample, _ = bench.cpu_sample_system(bench.make_workload({workload!r}, {seed}), {workload!r})
cs = [a for a in range(sample.n_atoms) if sample.shellsECP[a] > 0]
parts = [sample.subset(centres=cs[i::{threads}]) for i in range({threads})]
t0 = time.perf_counter()
with cf.ThreadPoolExecutor({threads}) as ex:
    list(ex.map(O.ref_matrix, parts))
print(json.dumps({{"t": time.perf_counter() - t0}}))
"""


def cpu_pieces(system, workload, n):
    """The larger workloads' CPU sample as n independent jobs of one ECP
    centre and six basis atoms each (centres taken in turn, atom windows
    advancing), so that all host cores have work: the restatement parallelises
    one job over its centres only, and these workloads have 4 to 10."""
    centres = [a for a in range(system.n_atoms) if system.shellsECP[a] > 0]
    basis = [a for a in range(system.n_atoms) if system.shellsBS[a] > 0]
    pieces = []
    for i in range(n):
        c = centres[i % len(centres)]
        w = (6 * (i // len(centres))) % max(1, len(basis) - 6)
        pieces.append(system.subset(centres=[c], basis_atoms=basis[w:w + 6]))
    text = (f"{n} jobs of one ECP centre x 6 basis atoms of the same "
            f"{'batch' if workload == 'mixed_batch' else 'sweep'} (centres in turn, atom windows advancing)")
    return pieces, text


def _run_pieces(pieces, threads):
    """The restatement over independent jobs on `threads` threads (the C code
    runs outside the interpreter lock): units/s, merged counters, units, s."""
    import concurrent.futures as cf
    from oracle import oracle as O
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(lambda p: O.oracle_matrix(p, nthreads=1, with_stats=True), pieces))
    t = time.perf_counter() - t0
    st = {}
    for _, _, s in res:
        for k, v in s.items():
            st[k] = st.get(k, 0) + v
    return st["blocks"] / t, st, st["blocks"], t


def host_cores() -> int:
    """Cores this process may run on (the affinity mask, not the machine's count)."""
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def run_cpu_single(system, workload="cluster"):
    """The port on one core over a quarter of the bounded sample (its first
    centres): units/s, the number of units and the seconds."""
    from oracle import oracle as O
    if workload in ("mixed_batch", "sweep"):
        v, st, units, t = _run_pieces(cpu_pieces(system, workload, 3)[0], 1)
        return v, units, t
    sample, text = cpu_sample_system(system, workload)
    cs = [a for a in range(sample.n_atoms) if sample.shellsECP[a] > 0]
    part = sample.subset(centres=cs[:max(1, len(cs) // 4)])
    t0 = time.perf_counter()
    rc, I, st = O.oracle_matrix(part, nthreads=1, with_stats=True)
    t = time.perf_counter() - t0
    return st["blocks"] / t, st["blocks"], t


def run_cpu_baseline(system, threads, workload="cluster", seed=0):
    """Times the reference's CPU path on the sample, on this machine's cores.

    The oracle restatement (kind "port") always runs: its counters give the
    algorithmic work of the reference's control flow.  Where the unmodified
    reference was built for this machine (oracle/_ref), it is timed too, in a
    child process, because it aborts on units whose large-grid quadrature runs
    out of levels (heap corruption after using a freed table); its time is
    reported only if it completes.  Returns (units/s, kind, stats, text, units, s).
    """
    from oracle import oracle as O
    if workload in ("mixed_batch", "sweep"):
        # three jobs per thread, taken as threads free up (the jobs differ in size)
        pieces, text = cpu_pieces(system, workload, 3 * threads)
        v, st, units, t = _run_pieces(pieces, threads)
        return v, "port", st, text, units, t
    sample, text = cpu_sample_system(system, workload)
    t0 = time.perf_counter()
    rc, I, st = O.oracle_matrix(sample, nthreads=threads, with_stats=True)
    t_port = time.perf_counter() - t0
    units = st["blocks"]
    kind, t = "port", t_port
    if O.ref_available():
        code = _REF_CHILD.format(root=ROOT, workload=workload, seed=seed, threads=threads)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
        if r.returncode == 0:
            kind, t = "reference", json.loads(r.stdout.strip().splitlines()[-1])["t"]
        else:
            text += (f"; the unmodified reference aborted on this sample (exit {r.returncode}: "
                     f"{r.stderr.strip().splitlines()[-1] if r.stderr.strip() else 'no message'})")
    return units / t, kind, st, text, units, t


def make_workload(name, seed):
    from libecp_gb300 import workloads as W
    if name == "mixed_batch":
        return W.mixed_batch(seed)
    if name == "sweep":
        return W.large_sweep(seed)
    s = W.batched_cluster(seed=seed)
    if name == "cluster8":
        s = s.subset(centres=[a for a in range(s.n_atoms) if s.shellsECP[a] > 0][:8])
    return s


def ours(args, rank, world):
    import libecp_gb300 as eg
    from libecp_gb300 import workloads as W
    local = int(os.environ.get("LOCAL_RANK", 0))
    eg.set_device(local)
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    system = make_workload(args.workload, rank)
    peaks = eg.measure_peaks()
    mode = eg.ECPGB_FAST if args.mode == "batched" else eg.ECPGB_FP64
    job = eg.Job(system, mode=mode)
    tuned = None
    if mode == eg.ECPGB_FAST:
        # the autotuner picks the launch configuration (outside the timed region)
        chosen, trials = job.tune()
        chosen["class_config"] = job.class_config()
        tuned = {"chosen": chosen, "trials": trials}
    job.run(args.warmup, flush_l2=True)
    n_units, emitted = job.units()
    if world > 1:
        dist.barrier()
        torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms, mu = job.run(args.steps, flush_l2=True)
    t_step = float(np.mean(ms))
    t_unit = float(np.mean(mu))
    if world > 1:
        t = torch.tensor([t_step, t_unit], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_step, t_unit = float(t[0]), float(t[1])
        e = torch.tensor([float(emitted)], device="cuda", dtype=torch.float64)
        dist.all_reduce(e)
        total_units = float(e[0])
    else:
        total_units = float(emitted)
    value = total_units / (t_step / 1e3)
    launches = job.launches_per_run() * args.steps
    job.close()
    plain = None
    if mode != eg.ECPGB_FP64 and args.compare_plain:
        # the plain FP64 drop-in kernels on the same job, for the batched / plain ratio
        pj = eg.Job(system, mode=eg.ECPGB_FP64)
        pj.run(1, flush_l2=True)
        pms, _ = pj.run(2, flush_l2=True)
        pj.close()
        plain = total_units / (float(np.mean(pms)) / 1e3)

    # end to end through the C ABI with host buffers (ecpgb_getIntegrals: the
    # getIntegrals call with the path chosen; one packed H2D, one D2H per step)
    rc, _, info = eg.get_integrals_info(system, mode=mode)
    h2d, d2h = info["h2dBytes"], info["d2hBytes"]
    e2e_t = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        eg.get_integrals_info(system, mode=mode)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_t.append(dt)
    e2e_step = float(np.mean(e2e_t))
    if world > 1:
        t = torch.tensor([e2e_step], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_step = float(t[0])
    e2e_value = total_units / e2e_step

    serving = None
    if rank == 0 and args.serve_seconds > 0 and mode == eg.ECPGB_FAST:
        serving = serving_run(eg, args.serve_rate, args.serve_seconds)
        if args.serve_mixed_seconds > 0:
            serving = {"batched_fp64": serving,
                       "mixed": serving_run(eg, args.serve_rate, args.serve_mixed_seconds, eg.ECPGB_MIXED)}

    mixed = None
    if rank == 0 and args.mixed_report and mode != eg.ECPGB_FP64:
        # the mixed-precision path on the same job: speed, its error against
        # the plain FP64 path over every unit, and per L class against the
        # oracle on the job's first two ECP centres
        from libecp_gb300.precision import oracle_class_errors
        mj = eg.Job(system, mode=eg.ECPGB_MIXED)
        mchosen, _ = mj.tune()
        mchosen["class_config"] = mj.class_config()
        mj.run(args.warmup, flush_l2=True)
        mms, mmu = mj.run(args.steps, flush_l2=True)
        mj.close()
        mval = total_units / (float(np.mean(mms)) / 1e3)
        v1, o1, st1, _ = eg.raw_blocks(system, eg.ECPGB_FP64)
        v3, o3, st3, _ = eg.raw_blocks(system, eg.ECPGB_MIXED)
        cs = [a for a in range(system.n_atoms) if system.shellsECP[a] > 0]
        rep = oracle_class_errors(system.subset(centres=cs[:2]), eg.ECPGB_MIXED)
        mixed = {"value": mval, "unit": UNIT, "ms_per_step": float(np.mean(mms)),
                 "unit_kernel_ms": float(np.mean(mmu)), "launch_config": mchosen,
                 "vs_batched_fp64": mval / value, "vs_plain_fp64": (mval / plain) if plain else None,
                 "max_abs_error_vs_plain_fp64_all_units": float(np.max(np.abs(v3 - v1))),
                 "statuses_equal_fp64": bool(np.array_equal(st1, st3)),
                 "error_vs_oracle_per_l_class_first_2_centres": rep["classes"]}

    line = None
    if rank == 0:
        cores = host_cores()
        cpu_v, kind, st, text, s_units, s_time = run_cpu_baseline(system, cores, args.workload, rank)
        cpu1_v, cpu1_units, cpu1_t = run_cpu_single(system, args.workload)
        f_unit = algorithmic_flops(st) / max(st["blocks"], 1)
        alg_achieved = f_unit * emitted / (t_unit / 1e3) / 1e12
        peak = peaks["fp64_fma_tflops"]
        if mode == eg.ECPGB_FP64:
            kernel = "k_unit"
        else:
            kernel = "k_unit_queue" if tuned["chosen"]["queue"] else "k_unit_fast"
        # executed work: FP64 operations the unit kernel executed per emitted
        # unit (ncu: 2 DFMA + DMUL + DADD thread instructions of one launch on
        # the cluster's first 8 centres, divided by its emitted units), FP64
        # pipe utilisation and DRAM bytes, from profiles/roofline_inputs.txt
        # (measured on the cluster: other workloads have no executed-work figure)
        entry = {}
        prof = os.path.join(ROOT, "profiles", "roofline_inputs.txt")
        if os.path.exists(prof) and args.workload == "cluster":
            with open(prof) as f:
                inputs = json.load(f)
            key = {"k_unit": "k_unit", "k_unit_queue": "k_unit_queue", "k_unit_fast": "k_unit_queue"}[kernel]
            entry = inputs.get(key + ("_mixed" if mode == eg.ECPGB_MIXED else ""), {})
        f_exec = entry.get("fp64_flops_per_emitted_unit")
        achieved = f_exec * emitted / (t_unit / 1e3) / 1e12 if f_exec else None
        traffic = entry["dram_bytes_per_emitted_unit"] * emitted if entry.get("dram_bytes_per_emitted_unit") else None
        pipe = entry.get("fp64_pipe_active")
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload],
                       "units_per_rank": int(n_units),
                       "emitted_units_per_rank": int(emitted),
                       "path": "batched FP64 (ECPGB_FAST)" if mode != eg.ECPGB_FP64 else "plain FP64 drop-in (ECPGB_FP64)",
                       "plain_fp64_value": plain,
                       "batched_over_plain": (value / plain) if plain else None,
                       "launch_config": tuned["chosen"] if tuned else None,
                       "autotuner_trials": tuned["trials"] if tuned else None,
                       "l2": "flushed between steps (256 MiB write)", "parallelism": "replicas"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "api": "ecpgb_getIntegrals (the getIntegrals call, host buffers, path = mode)"},
            "roofline": {"bound": "fp64", "kernel": kernel,
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if achieved else None,
                         "traffic": traffic,
                         "peak_source": "FP64 FMA pipe measured live by ecpgb_measure_peaks (of measured)",
                         "executed_fp64_flops_per_unit": f_exec,
                         "fp64_pipe_active_ncu": pipe,
                         "unit_kernel_ms": t_unit,
                         "alg_flops_per_unit": f_unit, "alg_achieved": alg_achieved,
                         "alg_frac": alg_achieved / peak,
                         "inputs": entry.get("source"),
                         "note": ("achieved = FP64 operations the kernel executed (ncu counts per emitted "
                                  "unit on the cluster's first 8 centres) x emitted units / the unit kernel's "
                                  "CUDA-event time; alg_* = the reference's work counted by the oracle on its "
                                  "control flow, which includes the full 1023-point tabulation of every "
                                  "large-grid fallback the kernel skips, so alg_frac can exceed 1")},
            "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"{text}: {s_units} units in {s_time:.1f} s on {cores} threads "
                                       + ("(jobs taken by threads as they free up)"
                                          if args.workload in ("mixed_batch", "sweep")
                                          else "(ECP centres dealt round-robin to threads)"),
                             "single_core": {"value": cpu1_v, "cores": 1,
                                             "sample": ("the first three of those jobs: "
                                                        if args.workload in ("mixed_batch", "sweep")
                                                        else "the first quarter of the sample's centres: ")
                                                       + f"{cpu1_units} units in {cpu1_t:.1f} s"}},
            "clocks": clk.summary(),
            "serving": serving,
            "mixed_precision": mixed,
            "gpu_launches": launches,
            "peaks_measured": peaks,
        }
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return line


def serving_run(eg, rate, seconds, mode=None, slots=32):
    """The serving stream (molecules of 5-200 atoms, 1-40 ECP centres, s..f
    shells of 1-6 primitives) at `rate` requests/s for `seconds` through the
    request server; latency percentiles as the server measured them."""
    from libecp_gb300 import serve
    mode = eg.ECPGB_FAST if mode is None else mode
    arrivals = serve.poisson_arrivals(rate, seconds, seed=7)
    systems = serve.request_stream(len(arrivals), seed=7)
    with eg.Server(mode=mode, budget_bytes=64 << 30, slots=slots) as sv:
        r = serve.run_stream(sv, systems, arrivals)
    return {"path": "batched FP64" if mode == eg.ECPGB_FAST else "mixed precision",
            "stream": "Poisson; 5-200 atoms (log-uniform), 1-40 ECP centres, s..f shells of 1-6 primitives",
            "offered_rate_per_s": rate, "seconds": seconds, "requests": r["requests"],
            "errors": len(r["errors"]), "served_rate_per_s": r["served_rate"],
            "units_per_s": r["units_per_s"], "latency_ms": r["latency_ms"], "queued_ms": r["queued_ms"],
            "gpu_ms": r["gpu_ms"], "hbm_budget_bytes": 64 << 30, "slots": slots,
            "max_inflight": r["stats"]["maxInflight"],
            "batching": "continuous: jobs overlap on per-slot streams; each CTA takes at most 8 units, "
                        "jobs under 100k units on high-priority streams"}


def reference_arm(args, rank, world):
    """The reference's CPU implementation on this machine's host cores."""
    if rank != 0:
        return None
    from libecp_gb300 import workloads as W
    from oracle import oracle as O
    system = W.batched_cluster(seed=0)
    cores = host_cores()
    vals = []
    for i in range(args.warmup + args.steps):
        v, kind, st, text, units, t = run_cpu_baseline(system, cores)
        if i >= args.warmup:
            vals.append(v)
    v = float(np.mean(vals))
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * units / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": text,
                       "note": "reference built from its sources where present, else the C restatement"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": text},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="batched", choices=["batched", "fp64"],
                    help="batched: the fast FP64 path; fp64: the plain drop-in kernels")
    ap.add_argument("--compare-plain", type=int, default=1,
                    help="also time the plain FP64 path (2 steps) for the ratio")
    ap.add_argument("--serve-rate", type=float, default=3.0,
                    help="serving stream arrival rate (requests/s; one GB300 serves about 3.5 of this "
                         "stream's requests per second)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="serving stream length on the batched FP64 path (0: no serving run)")
    ap.add_argument("--serve-mixed-seconds", type=float, default=30.0,
                    help="serving stream length on the mixed-precision path (0: none)")
    ap.add_argument("--workload", default="cluster", choices=list(WORKLOADS),
                    help="cluster (the headline), cluster8 (its first 8 centres: profiler captures), "
                         "mixed_batch and sweep (the other configurations)")
    ap.add_argument("--mixed-report", type=int, default=1,
                    help="also run the mixed-precision mode and report its speed and errors")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.warmup < 3:
        args.warmup = 3
    line = reference_arm(args, rank, world) if args.impl == "reference" else ours(args, rank, world)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
