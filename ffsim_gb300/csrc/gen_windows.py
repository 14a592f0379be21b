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
* ``cs_site_H_K(i, ...)`` -- for the cross-half rotation on orbitals
  (i, H + i): the members of a K-family of the low half that have bit i set,
  their partner index in the (K-1)-family with bit i cleared, and the parity
  of the occupied low-half orbitals above i (the fermionic sign).

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
    ms = members(b, k)
    index = {w: j for j, w in enumerate(ms)}
    n = len(ms)
    lines = [
        f"__device__ __forceinline__ void win_givens_{b}_{k}(float2 (&v)[{max(n, 1)}], const float* __restrict__ gp) {{"
    ]
    for g, l in enumerate(triangle(b)):
        pairs = []
        for w in ms:
            if (w >> l) & 1 and not (w >> (l + 1)) & 1:
                pairs.append((index[w], index[w ^ (3 << l)]))
        if not pairs:
            continue
        lines.append(f"  {{ const float c = gp[{3 * g}], sr = gp[{3 * g + 1}], si = gp[{3 * g + 2}];")
        for x, y in pairs:
            lines.append(f"    rot_pair(v[{x}], v[{y}], c, sr, si);")
        lines.append("  }")
    lines.append("}")
    return "\n".join(lines)


def emit_cs(h: int, k: int) -> str:
    """Pairs of the cross-half rotation at low-half site i (K-family -> (K-1)-family)."""
    ms = members(h, k)
    prev = {w: j for j, w in enumerate(members(h, k - 1))} if k >= 1 else {}
    lines = [
        f"template <class F> __device__ __forceinline__ void cs_site_{h}_{k}(int i, F&& f) {{",
        "  switch (i) {",
    ]
    for i in range(h):
        lines.append(f"  case {i}:")
        for j, w in enumerate(ms):
            if (w >> i) & 1:
                par = bin(w >> (i + 1)).count("1") & 1
                lines.append(f"    f({j}, {prev[w ^ (1 << i)]}, {par});")
        lines.append("    break;")
    lines.append("  default: break;\n  }\n}")
    return "\n".join(lines)


def emit_groups(b: int) -> str:
    """Group load/compute/store functions and the per-window dispatch struct."""
    lines = []
    for k in range(0, b + 1):
        m = math.comb(b, k)
        lines.append(
            f"static __device__ __noinline__ void win_contig_{b}_{k}(float2* __restrict__ s, const float* __restrict__ gp) {{\n"
            f"  float2 v[{m}];\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) v[j] = s[j];\n"
            f"  win_givens_{b}_{k}(v, gp);\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) s[j] = v[j];\n}}"
        )
        lines.append(
            f"static __device__ __noinline__ void win_table_{b}_{k}(float2* __restrict__ s, const int* __restrict__ off, const float* __restrict__ gp) {{\n"
            f"  float2 v[{m}];\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) v[j] = s[off[j]];\n"
            f"  win_givens_{b}_{k}(v, gp);\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) s[off[j]] = v[j];\n}}"
        )
    lines.append(f"template <> struct WinDispatch<{b}> {{")
    lines.append("  static __device__ __forceinline__ void contig(int k, float2* s, const float* gp) {")
    lines.append("    switch (k) {")
    for k in range(0, b + 1):
        lines.append(f"      case {k}: win_contig_{b}_{k}(s, gp); break;")
    lines.append("      default: break;\n    }\n  }")
    lines.append("  static __device__ __forceinline__ void table(int k, float2* s, const int* off, const float* gp) {")
    lines.append("    switch (k) {")
    for k in range(0, b + 1):
        lines.append(f"      case {k}: win_table_{b}_{k}(s, off, gp); break;")
    lines.append("      default: break;\n    }\n  }")
    lines.append("  template <class F> static __device__ __forceinline__ void cs(int k, int i, F&& f) {")
    lines.append("    switch (k) {")
    for k in range(1, b + 1):
        lines.append(f"      case {k}: cs_site_{b}_{k}(i, f); break;")
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
    ]
    for b in range(1, MAX_B + 1):
        for k in range(0, b + 1):
            parts.append(emit_givens(b, k))
    for h in range(1, MAX_B + 1):
        for k in range(1, h + 1):
            parts.append(emit_cs(h, k))
    for b in range(1, MAX_B + 1):
        parts.append(emit_groups(b))
    Path(out_path).write_text("\n".join(parts) + "\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "windows_gen.cuh")
    assert math.comb(8, 4) == len(members(8, 4))
