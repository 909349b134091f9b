"""Generates dsf_tables.cuh: the coefficient tables of the double-single
erfc and exp in dsf.cuh.

    python gen_dsf_tables.py          (needs mpmath, which ships with sympy)

erfcx(x) = exp(x^2) erfc(x) on [0, 6) in 24 pieces of width 1/4: on each
piece the degree-11 polynomial in t = x - centre that interpolates erfcx at
the 12 Chebyshev nodes (computed in 40-digit arithmetic), whose relative
error is below 1e-17 there.  exp uses Tang's table-driven reduction: the
table holds 2^(j/64), j = 0..63.  Every constant is written as the double
nearest to its exact value; the device splits it into a float pair.
"""
import os

import mpmath as mp

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "dsf_tables.cuh")

NPIECE = 24
WIDTH = mp.mpf(1) / 4
DEG = 11


def erfcx(x):
    return mp.exp(x * x) * mp.erfc(x)


def pieces():
    rows = []
    for p in range(NPIECE):
        a = p * WIDTH
        c = a + WIDTH / 2
        h = WIDTH / 2
        nodes = [h * mp.cos(mp.pi * (k + mp.mpf(1) / 2) / (DEG + 1)) for k in range(DEG + 1)]
        A = mp.matrix([[t ** n for n in range(DEG + 1)] for t in nodes])
        co = mp.lu_solve(A, mp.matrix([erfcx(c + t) for t in nodes]))
        rows.append([co[n] for n in range(DEG + 1)])
    return rows


def main():
    mp.mp.dps = 40
    rows = pieces()
    lines = ["// Generated by gen_dsf_tables.py; do not edit.",
             "#pragma once",
             "#define RSD_ERFCX_NPIECE %d" % NPIECE,
             "#define RSD_ERFCX_DEG %d" % DEG,
             "#define RSD_ERFCX_WIDTH 0.25",
             "#if defined(__CUDACC__)",
             "#define RSD_DSF_TABLE static __constant__ const double",
             "#else",
             "#define RSD_DSF_TABLE static const double",
             "#endif",
             "// erfcx on piece p: sum_n c[p][n] (x - (p + 1/2) / 4)^n",
             "RSD_DSF_TABLE rsd_erfcx_coef[RSD_ERFCX_NPIECE][RSD_ERFCX_DEG + 1] = {"]
    for r in rows:
        lines.append("  {" + ", ".join(mp.nstr(v, 20, min_fixed=-1, max_fixed=-1) for v in r) + "},")
    lines.append("};")
    lines.append("// 2^(j/64), j = 0..63")
    lines.append("RSD_DSF_TABLE rsd_exp2_table[64] = {")
    vals = [mp.power(2, mp.mpf(j) / 64) for j in range(64)]
    for i in range(0, 64, 4):
        lines.append("  " + ", ".join(mp.nstr(v, 20) for v in vals[i:i + 4]) + ",")
    lines.append("};")
    with open(OUT, "w") as fp:
        fp.write("\n".join(lines) + "\n")
    print(OUT)


if __name__ == "__main__":
    main()
