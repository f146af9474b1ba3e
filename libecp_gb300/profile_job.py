"""One run of a device-resident job on the first 8 ECP centres of the
50-centre cluster, for profiler captures of the unit kernels:

    python -m libecp_gb300.profile_job fast|mixed|plain

The batched modes use a fixed launch configuration (persistent queue,
class-major order, step-table cap 45, screening stage), so that the unit
kernel launches exactly once; no CUDA graph.  Prints the run's times and the
job's unit counts as one JSON line.
"""
from __future__ import annotations

import json
import sys

import libecp_gb300 as eg
from libecp_gb300 import workloads as W


def main(which: str = "fast") -> dict:
    mode = {"fast": eg.ECPGB_FAST, "mixed": eg.ECPGB_MIXED, "plain": eg.ECPGB_FP64}[which]
    s = W.batched_cluster(0)
    s = s.subset(centres=[a for a in range(s.n_atoms) if s.shellsECP[a] > 0][:8])
    j = eg.Job(s, mode=mode)
    if mode != eg.ECPGB_FP64:
        j.config(queue=1, sorted=2, gcap=45, balance=0, screen=1)
    j.use_graph(False)
    ms, mu = j.run(1, flush_l2=True)
    n, em = j.units()
    j.close()
    return {"mode": which, "ms": float(ms[0]), "unit_ms": float(mu[0]), "units": int(n), "emitted": int(em)}


if __name__ == "__main__":
    print(json.dumps(main(sys.argv[1] if len(sys.argv) > 1 else "fast")))
