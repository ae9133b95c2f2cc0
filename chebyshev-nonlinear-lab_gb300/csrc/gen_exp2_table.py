"""Writes exp2_table.cuh: 2^(j/256), j = 0..255, as hi + lo FP64 pairs (hi = RN(2^(j/256)),
lo = RN(2^(j/256) - hi)) and as FP32 pairs, plus the split of ln2/256 used by the reduction
x = N ln2/256 + r, all computed in 60-digit decimal arithmetic.

    python gen_exp2_table.py > exp2_table.cuh
"""
from __future__ import annotations

import struct
from decimal import Decimal, getcontext

getcontext().prec = 60


def f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def main() -> None:
    two = Decimal(2)
    ln2 = two.ln()
    rows, rows_f = [], []
    for j in range(256):
        v = two ** (Decimal(j) / Decimal(256))
        hi = float(v)
        lo = float(v - Decimal(hi))
        rows.append(f"    {{{hi.hex()}, {lo.hex()}}},")
        rows_f.append(f"    {{{f32(hi).hex()}f, {f32(lo).hex()}f}},")
    l1 = float(ln2 / 256)
    l2 = float(ln2 / 256 - Decimal(l1))
    inv = f32(float(256 / ln2))
    print("// Generated by gen_exp2_table.py: 2^(j/256) = hi + lo (FP64 pairs; FP32 pairs beside them)")
    print("// and ln2/256 = kExpL1 + kExpL2 (+ under 2^-115), from 60-digit decimal arithmetic.")
    print("#pragma once")
    print(f"constexpr double kExpL1 = {l1.hex()};")
    print(f"constexpr double kExpL2 = {l2.hex()};")
    print(f"constexpr float kExpL1f = {f32(l1).hex()}f;")
    print(f"constexpr float kExpL2f = {f32(l2).hex()}f;")
    print(f"constexpr float kExpInvL = {inv.hex()}f;  // RN32(256/ln2)")
    print("__device__ const double2 kExp2Frac[256] = {")
    print("\n".join(rows))
    print("};")
    print("__device__ const float2 kExp2FracF[256] = {")
    print("\n".join(rows_f))
    print("};")


if __name__ == "__main__":
    main()
