"""Emit ``windows_gen.cuh``: straight-line register code for window stages.

A *window* is a block of ``B`` consecutive orbitals.  Strings of one spin
sector that share their occupation outside the window form a *group*; a
group with ``K`` electrons inside the window has ``C(B, K)`` members, listed
here in colexicographic (= ascending integer) order of their window bits.
Every orbital rotation acting only inside the window maps the group to
itself, so one thread can hold the whole group in registers and apply all of
the window's Givens rotations without touching shared memory in between.

For each (B, K) this script writes:

* ``win_givens_B_K(v, gp)`` -- the fixed triangular Givens network of a
  ``B x B`` window unitary (host side: ``triangle_decompose`` in plan.cpp)
  applied to the member array ``v``; ``gp`` holds ``(c, Re s, Im s)`` per
  rotation in network order.  The network is: for r in 0..B-2, for col from
  B-1 down to r+1, rotate local orbitals (col-1, col).
* ``win_group_B_K(s, off, ...)`` -- loads the members ``s[off[j]]`` into
  registers, applies the network and stores them back; ``WinDispatch<B>``
  selects the function for a runtime K.
* ``win_rows_B_K(si, so, ld, off, ...)`` -- the same on members that are rows
  ``off[j]`` of a row-major array (one column per thread), with optional
  per-row phases multiplied in after the loads (``ph_in``) and before the
  stores (``ph_out``).

The output is a pure function of the window sizes, so it is regenerated at
build time and is not stored in the repository.
"""

from __future__ import annotations

import itertools
import math
import sys
from pathlib import Path

MAX_B = 8


def members(b: int, k: int) -> list[int]:
    out = [sum(1 << i for i in c) for c in itertools.combinations(range(b), k)]
    return sorted(out)


def triangle(b: int) -> list[int]:
    """Local lower index l of each rotation (l, l+1) in network order."""
    seq = []
    for r in range(b - 1):
        for col in range(b - 1, r, -1):
            seq.append(col - 1)
    return seq


def emit_givens(b: int, k: int) -> str:
    """Triangle network as a runtime loop over its rows r with the rotations of
    each row unrolled: rotation (col-1, col) runs when col > r.  Only b-1
    distinct orbital pairs exist, so the code holds b-1 pair patterns instead of
    b(b-1)/2 (keeps the instruction footprint small)."""
    ms = members(b, k)
    index = {w: j for j, w in enumerate(ms)}
    n = len(ms)
    lines = [
        "template <bool COMP>",
        f"__device__ __forceinline__ void win_givens_{b}_{k}(float2 (&v)[{max(n, 1)}], const float* __restrict__ gp,"
        " const float* __restrict__ gl) {",
    ]
    if b < 2:
        lines.append("}")
        return "\n".join(lines)
    lines.append("  int g = 0;")
    lines.append("#pragma unroll 1")
    lines.append(f"  for (int r = 0; r < {b - 1}; ++r) {{")
    for col in range(b - 1, 0, -1):
        l = col - 1
        pairs = []
        for w in ms:
            if (w >> l) & 1 and not (w >> (l + 1)) & 1:
                pairs.append((index[w], index[w ^ (3 << l)]))
        lines.append(f"    if ({col} > r) {{")
        if pairs:
            lines.append("      const float c = gp[3 * g], sr = gp[3 * g + 1], si = gp[3 * g + 2];")
            lines.append("      const float cl = COMP ? gl[3 * g] : 0.f, srl = COMP ? gl[3 * g + 1] : 0.f,"
                         " sil = COMP ? gl[3 * g + 2] : 0.f;")
            for x, y in pairs:
                lines.append(f"      rot_pair<COMP>(v[{x}], v[{y}], c, sr, si, cl, srl, sil);")
        lines.append("      ++g;")
        lines.append("    }")
    lines.append("  }")
    lines.append("}")
    return "\n".join(lines)


def emit_groups(b: int) -> str:
    """One group function per (b, k): members at s[off[j]] (off is the identity for
    groups that are contiguous runs), so the low- and high-half stages share code."""
    lines = []
    for k in range(0, b + 1):
        m = math.comb(b, k)
        lines.append(
            f"template <bool COMP> static __device__ __noinline__ void win_group_{b}_{k}(float2* __restrict__ s,"
            f" const int* __restrict__ off, const float* __restrict__ gp, const float* __restrict__ gl) {{\n"
            f"  float2 v[{m}];\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) v[j] = s[off[j]];\n"
            f"  win_givens_{b}_{k}<COMP>(v, gp, gl);\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) s[off[j]] = v[j];\n}}"
        )
    for k in range(0, b + 1):
        m = math.comb(b, k)
        lines.append(
            f"template <bool COMP> static __device__ __noinline__ void win_rows_{b}_{k}(const float2* __restrict__ si,"
            f" float2* __restrict__ so, long long ld, const int* __restrict__ off, const float* __restrict__ gp,"
            f" const float* __restrict__ gl, const float2* __restrict__ ph_in, const float2* __restrict__ ph_out) {{\n"
            f"  float2 v[{m}];\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) v[j] = si[(long long)off[j] * ld];\n"
            f"  if (ph_in) {{\n"
            f"#pragma unroll\n    for (int j = 0; j < {m}; ++j) v[j] = cmulf2(v[j], ph_in[off[j]]);\n  }}\n"
            f"  win_givens_{b}_{k}<COMP>(v, gp, gl);\n"
            f"  if (ph_out) {{\n"
            f"#pragma unroll\n    for (int j = 0; j < {m}; ++j) v[j] = cmulf2(v[j], ph_out[off[j]]);\n  }}\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) so[(long long)off[j] * ld] = v[j];\n}}"
        )
    lines.append(f"template <> struct WinDispatch<{b}> {{")
    lines.append("  template <bool COMP> static __device__ __forceinline__ void rows(int k, const float2* si, float2* so,"
                 " long long ld, const int* off, const float* gp, const float* gl, const float2* ph_in,"
                 " const float2* ph_out) {")
    lines.append("    switch (k) {")
    for k in range(0, b + 1):
        lines.append(f"      case {k}: win_rows_{b}_{k}<COMP>(si, so, ld, off, gp, gl, ph_in, ph_out); break;")
    lines.append("      default: break;\n    }\n  }")
    lines.append("  template <bool COMP> static __device__ __forceinline__ void group(int k, float2* s, const int* off,"
                 " const float* gp, const float* gl) {")
    lines.append("    switch (k) {")
    for k in range(0, b + 1):
        lines.append(f"      case {k}: win_group_{b}_{k}<COMP>(s, off, gp, gl); break;")
    lines.append("      default: break;\n    }\n  }")
    lines.append("};")
    return "\n".join(lines)


def main(out_path: str) -> None:
    parts = [
        "// Generated by gen_windows.py -- do not edit.",
        "#pragma once",
        "",
        "__host__ __device__ constexpr int win_members(int b, int k) {",
        "  return (k < 0 || k > b) ? 0 : (k == 0 || k == b) ? 1 : win_members(b - 1, k - 1) + win_members(b - 1, k);",
        "}",
        "template <int B> struct WinDispatch;",
        "__device__ __forceinline__ float2 cmulf2(float2 a, float2 b) {",
        "  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);",
        "}",
    ]
    for b in range(1, MAX_B + 1):
        for k in range(0, b + 1):
            parts.append(emit_givens(b, k))
    for b in range(1, MAX_B + 1):
        parts.append(emit_groups(b))
    Path(out_path).write_text("\n".join(parts) + "\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "windows_gen.cuh")
    assert math.comb(8, 4) == len(members(8, 4))
