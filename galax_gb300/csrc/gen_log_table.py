"""Writes log_table.h: F_j = 1 + j/128 (j = 0..128), 1/F_j and log(F_j) as a
(hi, lo) pair of doubles, for the table-driven logarithm in potentials.cuh
(Tang, ACM TOMS 16(4), 1990). The logarithms are evaluated with Python's
decimal module at 50 significant digits. Run from this directory:

    python gen_log_table.py > log_table.h
"""

from __future__ import annotations

from decimal import Decimal, getcontext


def table():
    getcontext().prec = 50
    rows = []
    for j in range(129):
        F = Decimal(1) + Decimal(j) / Decimal(128)
        lg = F.ln()
        hi = float(lg)
        lo = float(lg - Decimal(hi))
        rows.append((1.0 / float(F), hi, lo))
    return rows


def main() -> None:
    rows = table()
    print("// Generated by gen_log_table.py: 1/F_j, log(F_j) hi, lo for F_j = 1 + j/128, j = 0..128.")
    print("#pragma once")
    print("namespace gal {")
    print("__device__ const double kLogTable[129][3] = {")
    for inv, hi, lo in rows:
        print(f"    {{{inv.hex()}, {hi.hex()}, {lo.hex()}}},".replace("0x", "0x"))
    print("};")
    print("}  // namespace gal")


if __name__ == "__main__":
    main()
