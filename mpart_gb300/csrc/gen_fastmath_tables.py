"""Writes mpgb_fastmath_tables.h: the tables of the table-driven exponential
and logarithm in mpgb_fastmath.cuh, from 60-digit decimal arithmetic
(Python's decimal module), each value rounded once to the nearest double.

    python gen_fastmath_tables.py > mpgb_fastmath_tables.h
"""
from decimal import Decimal, getcontext

getcontext().prec = 60
LN2 = Decimal(2).ln()


def dbl(d):
    return float.hex(float(d))


def split(d, bits):
    """d as hi + lo, hi with `bits` significant bits (so that k * hi is exact
    for small integers k), lo the double nearest d - hi."""
    v = float(d)
    m, e = __import__("math").frexp(v)
    hi = float(round(m * (1 << bits))) * 2.0 ** (e - bits)
    return hi, float(d - Decimal(hi))


def main():
    out = []
    out.append("// Generated by gen_fastmath_tables.py; do not edit.")
    out.append("#pragma once")
    out.append("namespace mpgb {")
    out.append("namespace fm {")
    hi, lo = split(LN2 / 64, 32)
    out.append(f"constexpr double kInvLn2x64 = {dbl(64 / LN2)};  // 64 / ln 2")
    out.append(f"constexpr double kLn2x64Hi = {float.hex(hi)};  // ln 2 / 64, 32 significant bits")
    out.append(f"constexpr double kLn2x64Lo = {float.hex(lo)};")
    hi2, lo2 = split(LN2, 32)
    out.append(f"constexpr double kLn2Hi = {float.hex(hi2)};  // ln 2, 32 significant bits")
    out.append(f"constexpr double kLn2Lo = {float.hex(lo2)};")
    out.append("// 2^(j/64), j = 0..63.")
    vals = [dbl((LN2 * j / 64).exp()) for j in range(64)]
    out.append("__device__ const double kExp2Tab[64] = {")
    for i in range(0, 64, 4):
        out.append("    " + ", ".join(vals[i:i + 4]) + ",")
    out.append("};")
    inv, lg = [], []
    for j in range(129):
        f = Decimal(1) + Decimal(j) / 128
        iv = float(Decimal(1) / f)
        inv.append(float.hex(iv))
        lg.append(dbl(-(Decimal(iv).ln())))
    out.append("// inv[j]: the double nearest 1 / (1 + j/128); logInv[j] = -log(inv[j]) of that")
    out.append("// double, j = 0..128.")
    for name, vals in (("kLogInvTab", inv), ("kLogTab", lg)):
        out.append(f"__device__ const double {name}[129] = {{")
        for i in range(0, 129, 4):
            out.append("    " + ", ".join(vals[i:i + 4]) + ",")
        out.append("};")
    out.append("}  // namespace fm")
    out.append("}  // namespace mpgb")
    print("\n".join(out))


if __name__ == "__main__":
    main()
