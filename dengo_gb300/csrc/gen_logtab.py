"""Writes dg_logtab.h: the reduction table of dg_log (see dg_math.h).

For j = 0..128, c_j = 1 + j/128 and inv_j is the double nearest 1/c_j;
the table holds inv_j and -log(inv_j) as an unevaluated sum hi + lo,
computed with 200-bit arithmetic (mpmath).  LN2_HI carries 42 significant
bits so that e * LN2_HI is exact for every binary exponent e of a double.
"""
import math
import os

import mpmath


def main():
    mpmath.mp.prec = 200
    lines = ["/* Generated by gen_logtab.py; do not edit. */",
             "#ifndef DG_LOGTAB_H", "#define DG_LOGTAB_H", ""]
    ln2 = mpmath.log(2)
    m, e = math.frexp(float(ln2))
    hi = math.ldexp(math.floor(m * 2**42), e - 42)
    lo = float(ln2 - mpmath.mpf(hi))
    lines.append("#define DG_LN2_HI %s" % float.hex(hi))
    lines.append("#define DG_LN2_LO %s" % float.hex(lo))
    lines.append("")
    lines.append("#define DG_LOGTAB_DATA { \\")
    for j in range(129):
        c = mpmath.mpf(1) + mpmath.mpf(j) / 128
        inv = float(1 / c)
        t = -mpmath.log(mpmath.mpf(inv))
        thi = float(t)
        tlo = float(t - mpmath.mpf(thi))
        lines.append("    {%s, %s, %s}, \\" % (float.hex(inv), float.hex(thi), float.hex(tlo)))
    lines += ["}", "", "#endif", ""]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dg_logtab.h")
    with open(path, "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
