"""Writes exp_table.cuh: 2^(j/256), j = 0..255, each correctly rounded to
IEEE double (60-digit decimal arithmetic), and the two-part split of
ln2/256 used for the argument reduction of exp_neg (pair_math.cuh).

Usage: python mdynamix_gb300/csrc/make_exp_table.py
"""
import os
import struct
from decimal import Decimal, getcontext

getcontext().prec = 60
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ln2 = Decimal(2).ln()
    step = ln2 / 256
    bits = struct.unpack("<Q", struct.pack("<d", float(step)))[0]
    hi = struct.unpack("<d", struct.pack("<Q", bits & ~((1 << 21) - 1)))[0]  # 32 significant bits
    lo = float(step - Decimal(hi))
    tab = [float(Decimal(2) ** (Decimal(j) / 256)) for j in range(256)]
    rows = []
    for k in range(0, 256, 4):
        rows.append("    " + ", ".join(f"{v!r}" for v in tab[k:k + 4]) + ",")
    text = f"""// exp_table.cuh -- generated by make_exp_table.py; do not edit.
// 2^(j/256) for j = 0..255 (correctly rounded), and ln2/256 = EXP_L_HI +
// EXP_L_LO with EXP_L_HI holding 32 significant bits, so that n * EXP_L_HI
// is exact for |n| < 2^21.
#pragma once

constexpr double EXP_INV_L = {float(256 / ln2)!r};  // 256 / ln2
constexpr double EXP_L_HI = {hi!r};
constexpr double EXP_L_LO = {lo!r};

__device__ const double k_exp2_256[256] = {{
{chr(10).join(rows)}
}};
"""
    with open(os.path.join(HERE, "exp_table.cuh"), "w") as f:
        f.write(text)


if __name__ == "__main__":
    main()
