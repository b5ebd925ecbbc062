"""Generate ss_log_table.inc: the breakpoint table of the FP64 ln(1 + u) in
ss_device.cuh (a table-driven logarithm after P. T. P. Tang, "Table-driven
implementation of the logarithm function in IEEE floating-point arithmetic",
ACM TOMS 16(4), 1990).

Entry j (0 <= j <= 128) holds G_j = 1/F_j rounded to the nearest double,
F_j = 1 + j/128, and L_j = -ln(G_j) rounded to the nearest double, computed
with 60 significant digits.  Because L_j is the logarithm of the rounded G_j
itself, ln(m) = L_j + ln(m G_j) holds exactly for any m, and r = m G_j - 1
is formed with one FMA.  Also emitted: ln 2 split as LN2_HI (the leading 42
bits, so that k LN2_HI is exact for |k| < 2^11) + LN2_LO.

Run from this directory: python gen_log_table.py > ss_log_table.inc
"""
import mpmath

mpmath.mp.dps = 60


def hexd(x: float) -> str:
    return float.hex(x)


def main():
    print("// Generated by gen_log_table.py: G_j = 1 / (1 + j / 128) rounded to double,")
    print("// L_j = -ln(G_j) rounded to double (60-digit arithmetic).  Do not edit.")
    print("__device__ const double2 g_ln_tab[129] = {")
    for j in range(129):
        g = float(1 / (1 + mpmath.mpf(j) / 128))
        L = float(-mpmath.log(mpmath.mpf(g)))
        print(f"    {{{hexd(g)}, {hexd(L)}}},")
    print("};")
    ln2 = mpmath.log(2)
    ln2_hi = float(ln2)
    # keep the leading 42 significant bits
    m, e = mpmath.frexp(mpmath.mpf(ln2_hi))
    ln2_hi = float(mpmath.floor(m * 2 ** 42) / 2 ** 42 * 2 ** e)
    ln2_lo = float(ln2 - mpmath.mpf(ln2_hi))
    print(f"constexpr double SS_LN2_HI = {hexd(ln2_hi)};")
    print(f"constexpr double SS_LN2_LO = {hexd(ln2_lo)};")


if __name__ == "__main__":
    main()
