"""Serving driver: a Poisson stream of ECP integral jobs through the request
server (continuous batching, HBM-budget admission), with latency percentiles.

The stream follows the serving configuration: molecules of 5-200 atoms
(log-uniform), 1-40 ECP centres each (never more than the atoms), s..f basis
shells of 1-6 primitives, arrivals at a fixed Poisson rate.  Every molecule is
generated before the clock starts; a submitter thread submits each at its
arrival time and a collector waits for the results in arrival order.  The
server measures each request's latency (submit -> result ready) itself.
"""
from __future__ import annotations

import threading
import time

import numpy as np

from . import workloads as W


def poisson_arrivals(rate: float, duration: float, seed: int = 0) -> np.ndarray:
    """Arrival times (s) of a Poisson process of `rate` per second on [0, duration)."""
    rng = np.random.default_rng(seed)
    n = max(1, int(rate * duration * 1.5) + 16)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    while t[-1] < duration:
        t = np.concatenate([t, t[-1] + np.cumsum(rng.exponential(1.0 / rate, n))])
    return t[t < duration]


def request_stream(n: int, seed: int = 0, min_atoms: int = 5, max_atoms: int = 200,
                   max_centres: int = 40):
    """n molecules of the serving stream (deterministic in seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        atoms = int(round(np.exp(rng.uniform(np.log(min_atoms), np.log(max_atoms)))))
        centres = int(rng.integers(1, min(max_centres, atoms) + 1))
        out.append(W.serving_molecule(rng, atoms, centres))
    return out


def percentiles(x) -> dict:
    x = np.asarray(x, dtype=np.float64)
    if x.size == 0:
        return {"p50": None, "p90": None, "p99": None, "mean": None, "max": None}
    return {"p50": float(np.percentile(x, 50)), "p90": float(np.percentile(x, 90)),
            "p99": float(np.percentile(x, 99)), "mean": float(x.mean()), "max": float(x.max())}


def run_stream(server, systems, arrivals, keep_results: bool = False) -> dict:
    """Submits systems[i] at arrivals[i] seconds after the start; returns the
    per-request infos, wall time and throughput figures."""
    n = len(systems)
    ids = [None] * n
    submitted = threading.Event()
    errors = []

    def submitter():
        t0 = time.perf_counter()
        for i in range(n):
            dt = arrivals[i] - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
            try:
                ids[i] = server.submit(systems[i])
            except Exception as e:  # noqa: BLE001 - reported below
                errors.append((i, str(e)))
        submitted.set()

    t_start = time.perf_counter()
    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    infos, results, rcs = [], [], []
    for i in range(n):
        while ids[i] is None and not submitted.is_set():
            time.sleep(0.0002)
        if ids[i] is None:  # its submission failed
            continue
        try:
            rc, I, info = server.wait(ids[i])
        except RuntimeError as e:
            errors.append((i, str(e)))
            continue
        rcs.append(rc)
        infos.append(info)
        if keep_results:
            results.append(I)
    th.join()
    wall = time.perf_counter() - t_start
    units = sum(f["units"] for f in infos)
    lat = [f["msLatency"] for f in infos]
    return {"requests": len(infos), "errors": errors, "wall_s": wall,
            "offered_rate": n / max(arrivals[-1], 1e-9) if n else 0.0,
            "served_rate": len(infos) / wall, "units": units, "units_per_s": units / wall,
            "latency_ms": percentiles(lat), "queued_ms": percentiles([f["msQueued"] for f in infos]),
            "gpu_ms": percentiles([f["msGpu"] for f in infos]), "rcs": rcs, "infos": infos,
            "results": results, "stats": server.stats()}
