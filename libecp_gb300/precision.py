"""Error of a GPU path per L class, against the FP64 oracle or another path.

An L class is the (la, lb) angular-momentum pair of a shell pair.  For each
class: the largest absolute error over the class's block elements, the
root-mean-square error, and the largest error relative to the largest
element of the same block (so that blocks of very different magnitude are
comparable).  Units the screening skips carry no block and are left out.

oracle_class_errors compares a GPU path with the CPU restatement of the
reference (oracle/), so it needs the oracle's library; class_errors compares
two sets of raw blocks (two GPU paths).
"""
from __future__ import annotations

import numpy as np

from . import blocks, raw_blocks, unit_table


def _accumulate(acc, la, lb, ref, test):
    d = np.abs(ref - test)
    scale = max(float(np.abs(ref).max()), 1e-300) if ref.size else 1e-300
    for key in (f"{la},{lb}", "all"):
        e = acc.setdefault(key, {"max_abs": 0.0, "sq": 0.0, "max_rel_block": 0.0,
                                 "n_values": 0, "n_units": 0})
        if d.size:
            e["max_abs"] = max(e["max_abs"], float(d.max()))
            e["sq"] += float((d * d).sum())
            e["max_rel_block"] = max(e["max_rel_block"], float(d.max()) / scale)
        e["n_values"] += int(d.size)
        e["n_units"] += 1


def _finish(acc):
    for e in acc.values():
        e["rms"] = (e.pop("sq") / max(e["n_values"], 1)) ** 0.5
    return acc


def class_errors(s, ref, test) -> dict:
    """ref, test: (values, offsets, status, info) of raw_blocks for the same
    system.  Returns {"classes": {"la,lb" | "all": stats}, "statuses_equal"}."""
    v_ref, offs, st_ref, _ = ref
    v_test, offs_t, st_test, _ = test
    assert np.array_equal(offs, offs_t)
    units = unit_table(s)
    acc = {}
    for u, row in enumerate(units):
        if st_ref[u] == 1 or st_test[u] == 1:  # skipped
            continue
        la, lb = row[2], row[5]
        n = 2 * ((la + 1) * (la + 2) // 2) * ((lb + 1) * (lb + 2) // 2)
        _accumulate(acc, la, lb, v_ref[offs[u]:offs[u] + n], v_test[offs[u]:offs[u] + n])
    return {"classes": _finish(acc), "statuses_equal": bool(np.array_equal(st_ref, st_test))}


def oracle_class_errors(s, mode) -> dict:
    """The GPU path `mode` against the oracle on system s (both blocks of a
    unit together).  Returns {"classes": {...}}."""
    from oracle import oracle as O
    rc, mo, do = O.oracle_blocks(s)
    mg, dg = blocks(s, mode=mode)
    assert np.array_equal(mg, mo), "block lists differ"
    acc = {}
    off = 0
    for i in range(0, len(mo), 2):
        la, lb = int(mo[i][2]), int(mo[i][5])
        n = 2 * ((la + 1) * (la + 2) // 2) * ((lb + 1) * (lb + 2) // 2)
        _accumulate(acc, la, lb, do[off:off + n], dg[off:off + n])
        off += n
    return {"classes": _finish(acc)}
