"""Error of a reduced-precision result against an FP64 one, per L class.

An L class is the (la, lb) angular-momentum pair of a shell pair.  For each
class: the largest absolute error over the class's block elements, the
root-mean-square error, and the largest error relative to the largest
element of the same block (so that blocks of very different magnitude are
comparable).  Units the screening skips carry no block and are left out.
"""
from __future__ import annotations

import numpy as np

from . import raw_blocks, unit_table


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
        a = v_ref[offs[u]:offs[u] + n]
        d = np.abs(a - v_test[offs[u]:offs[u] + n])
        scale = max(float(np.abs(a).max()), 1e-300)
        for key in (f"{la},{lb}", "all"):
            e = acc.setdefault(key, {"max_abs": 0.0, "sq": 0.0, "max_rel_block": 0.0,
                                     "n_values": 0, "n_units": 0})
            e["max_abs"] = max(e["max_abs"], float(d.max()))
            e["sq"] += float((d * d).sum())
            e["max_rel_block"] = max(e["max_rel_block"], float(d.max()) / scale)
            e["n_values"] += int(d.size)
            e["n_units"] += 1
    for e in acc.values():
        e["rms"] = (e.pop("sq") / max(e["n_values"], 1)) ** 0.5
    return {"classes": acc, "statuses_equal": bool(np.array_equal(st_ref, st_test))}


def mixed_report(s) -> dict:
    """The mixed-precision path against the plain FP64 path on system s."""
    from . import ECPGB_FP64, ECPGB_MIXED
    return class_errors(s, raw_blocks(s, ECPGB_FP64), raw_blocks(s, ECPGB_MIXED))
