"""Writes exp2_table.cuh: 2^(j/T), j = 0..T-1 (T = 2048), as hi + lo FP64 pairs (hi = RN(2^(j/T)),
lo = RN(2^(j/T) - hi)) and as FP32 pairs, plus the split of ln2/T used by the reduction
x = N ln2/T + r, all computed in 60-digit decimal arithmetic.

    python gen_exp2_table.py > exp2_table.cuh
"""
from __future__ import annotations

import struct
from decimal import Decimal, getcontext

getcontext().prec = 60
T = 2048


def f32(x: float) -> float:
    return struct.unpack("<f", struct.pack("<f", x))[0]


def main() -> None:
    two = Decimal(2)
    ln2 = two.ln()
    rows, rows_f = [], []
    for j in range(T):
        v = two ** (Decimal(j) / Decimal(T))
        hi = float(v)
        lo = float(v - Decimal(hi))
        rows.append(f"    {{{hi.hex()}, {lo.hex()}}},")
        rows_f.append(f"    {{{f32(hi).hex()}f, {f32(lo).hex()}f}},")
    l1 = float(ln2 / T)
    l2 = float(ln2 / T - Decimal(l1))
    inv = f32(float(T / ln2))
    print(f"// Generated by gen_exp2_table.py: 2^(j/{T}) = hi + lo (FP64 pairs; FP32 pairs beside them)")
    print(f"// and ln2/{T} = kExpL1 + kExpL2 (+ under 2^-118), from 60-digit decimal arithmetic.")
    print("#pragma once")
    print(f"constexpr int kExpTableBits = {T.bit_length() - 1};")
    print(f"constexpr double kExpL1 = {l1.hex()};")
    print(f"constexpr double kExpL2 = {l2.hex()};")
    print(f"constexpr float kExpL1f = {f32(l1).hex()}f;")
    print(f"constexpr float kExpL2f = {f32(l2).hex()}f;")
    print(f"constexpr float kExpInvL = {inv.hex()}f;  // RN32({T}/ln2)")
    print(f"__device__ const double2 kExp2Frac[{T}] = {{")
    print("\n".join(rows))
    print("};")
    print(f"__device__ const float2 kExp2FracF[{T}] = {{")
    print("\n".join(rows_f))
    print("};")


if __name__ == "__main__":
    main()
