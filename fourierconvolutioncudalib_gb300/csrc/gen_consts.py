"""Generate fc_consts.cuh: the DFT constants of the in-register butterflies.

The values are cos(2*pi*j/P) and sin(2*pi*j/P) for the odd prime radices
P = 3, 5, 7, 11, 13, the internal twiddles of the composite radices
6, 9, 10, 12, 14, 15 and of the radix-16 butterfly (exp(-2*pi*i*j/16)).  They are evaluated in double precision with Python's
math module and rounded once to float32 (repr of the float32 value, so the
literal is exact).  Run:  python gen_consts.py > fc_consts.cuh
"""
import math
import struct


def f32(x: float) -> str:
    v = struct.unpack("<f", struct.pack("<f", x))[0]
    s = repr(v)
    if "e" not in s and "." not in s:
        s += ".0"
    return s + "f"


def emit_table(name: str, p: int, fn) -> str:
    lines = [f"template <> __device__ __forceinline__ float {name}<{p}>(int j) {{", "  switch (j) {"]
    for j in range(p):
        lines.append(f"    case {j}: return {f32(fn(2.0 * math.pi * j / p))};")
    lines.append("    default: return 0.0f;")
    lines.append("  }")
    lines.append("}")
    return "\n".join(lines)


def main() -> None:
    out = [
        "// Generated by gen_consts.py -- DFT constants rounded once from double precision.",
        "#pragma once",
        "",
        "// cos(2*pi*j/P) and sin(2*pi*j/P), j = 0..P-1, for the odd prime butterflies.",
        "template <int P> __device__ __forceinline__ float fc_dft_cos(int j);",
        "template <int P> __device__ __forceinline__ float fc_dft_sin(int j);",
    ]
    for p in (3, 5, 7, 11, 13):
        out.append(emit_table("fc_dft_cos", p, math.cos))
        out.append(emit_table("fc_dft_sin", p, math.sin))
    out.append("")
    out.append("// cos(2*pi*j/R), sin(2*pi*j/R), j = 0..R-1, for the internal twiddles of the")
    out.append("// composite butterflies R = A*B (Cooley-Tukey inside the registers).")
    out.append("template <int R> __device__ __forceinline__ float fc_tw_cos(int j);")
    out.append("template <int R> __device__ __forceinline__ float fc_tw_sin(int j);")
    for r in (6, 9, 10, 12, 14, 15):
        out.append(emit_table("fc_tw_cos", r, math.cos))
        out.append(emit_table("fc_tw_sin", r, math.sin))
    out.append("")
    out.append("// cos(2*pi*j/16), sin(2*pi*j/16) for the radix-16 internal twiddles.")
    out.append("#define FC_C16_1 " + f32(math.cos(2 * math.pi / 16)))
    out.append("#define FC_S16_1 " + f32(math.sin(2 * math.pi / 16)))
    out.append("#define FC_SQRT1_2 " + f32(math.sqrt(0.5)))
    out.append("")
    print("\n".join(out))


if __name__ == "__main__":
    main()
