"""Writes ecp_exp2_table.h: the constants of fast_exp (ecp_fastmath.h).

  2^(j/512), j = 0..511, each rounded to the nearest double (computed with
  256-bit mpmath arithmetic, then rounded once);
  ln2/512 split as L1 + L2, L1 with 32 significant bits (so n * L1 is exact
  for |n| < 2^21), L2 the nearest double to ln2/512 - L1;
  512/ln2 rounded to nearest.

Run from anywhere: python libecp_gb300/csrc/gen_exp2_table.py [output]
(default output: ecp_exp2_table.h beside this script).
"""
import math
import os
import sys

import mpmath

N = 512


def main() -> None:
    mpmath.mp.prec = 256
    ln2 = mpmath.log(2)
    step = ln2 / N
    e = mpmath.floor(mpmath.log(step, 2))
    scale = mpmath.mpf(2) ** (31 - e)  # 32 significant bits
    l1 = mpmath.floor(step * scale) / scale
    L1, L2, inv = float(l1), float(step - l1), float(N / ln2)
    assert mpmath.mpf(L1) == l1
    vals = [float(mpmath.power(2, mpmath.mpf(j) / N)) for j in range(N)]
    lines = [
        "// Generated by gen_exp2_table.py: constants of fast_exp (ecp_fastmath.h).",
        "#pragma once",
        f"#define ECPGB_EXP2_N {N}",
        f"#define ECPGB_EXP2_LOG2N {int(math.log2(N))}",
        f"#define ECPGB_EXP2_INV {inv.hex()}   // {N}/ln2",
        f"#define ECPGB_EXP2_L1 {L1.hex()}   // ln2/{N}, leading 32 bits",
        f"#define ECPGB_EXP2_L2 {L2.hex()}   // ln2/{N} - L1",
        "#define ECPGB_EXP2_TABLE \\",
        "  { \\",
    ]
    for i in range(0, N, 4):
        lines.append("    " + ", ".join(v.hex() for v in vals[i:i + 4]) + ", \\")
    lines.append("  }")
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                             "ecp_exp2_table.h")
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
