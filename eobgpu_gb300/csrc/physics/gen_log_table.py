"""Write log_table.h: the table of eob_log (fastlog.h).

Tang's table-driven logarithm (P. T. P. Tang, "Table-driven implementation of
the logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
1990): for breakpoints F_j = 1 + j/128, j = 0..128, the table holds
inv_j = RN(1/F_j) and T_j = -log(inv_j) split as thi_j + tlo_j, where thi_j
keeps 40 significant bits (so that e*ln2_hi + thi_j is exact in FP64 for
|e| < 1024) and tlo_j = RN(T_j - thi_j).  ln2 is split the same way.  Values
come from mpmath at 60 digits; the output is hexadecimal floating point, so the
header is the same on every machine.

    python gen_log_table.py > log_table.h
"""
import mpmath

mpmath.mp.dps = 60


def rn(x):
    """Round an mpf to the nearest double."""
    return float(mpmath.mpf(x))


def hi40(x):
    """x rounded to 40 significant bits (as a double)."""
    x = mpmath.mpf(x)
    if x == 0:
        return 0.0
    m, e = mpmath.frexp(x)  # x = m 2^e, 0.5 <= |m| < 1
    return float(mpmath.ldexp(mpmath.nint(mpmath.ldexp(m, 40)), e - 40))


def main():
    ln2 = mpmath.log(2)
    l2hi = hi40(ln2)
    l2lo = rn(ln2 - mpmath.mpf(l2hi))
    rows = []
    for j in range(129):
        F = mpmath.mpf(1) + mpmath.mpf(j) / 128
        inv = rn(1 / F)
        T = -mpmath.log(mpmath.mpf(inv))
        if j == 128:  # inv = 1/2 exactly: T = ln2, split as ln2 itself so e = -1 cancels exactly
            thi, tlo = l2hi, l2lo
        else:
            thi = hi40(T)
            tlo = rn(T - mpmath.mpf(thi))
        rows.append((inv, thi, tlo))
    print("// Generated by gen_log_table.py (Tang's table-driven logarithm); do not edit.")
    print("#pragma once")
    print(f"#define EOB_LN2_HI {l2hi.hex()}")
    print(f"#define EOB_LN2_LO {l2lo.hex()}")
    print("// {RN(1/F_j), -log(inv_j) high 40 bits, remainder}, F_j = 1 + j/128")
    print("#define EOB_LOGTAB_INIT \\")
    print("    { \\")
    for j, (a, b, c) in enumerate(rows):
        sep = "," if j < 128 else ""
        print(f"        {{{a.hex()}, {b.hex()}, {c.hex()}}}{sep} \\")
    print("    }")


if __name__ == "__main__":
    main()
