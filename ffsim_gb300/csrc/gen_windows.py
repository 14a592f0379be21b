"""Emit ``windows_gen.cuh``: straight-line register code for window stages.

A *window* is a block of ``B`` consecutive orbitals.  Strings of one spin
sector that share their occupation outside the window form a *group*; a
group with ``K`` electrons inside the window has ``C(B, K)`` members, listed
here in colexicographic (= ascending integer) order of their window bits.
Every orbital rotation acting only inside the window maps the group to
itself, so one thread can hold the whole group in registers and apply all of
the window's Givens rotations without touching shared memory in between.

For each (B, K) this script writes:

* ``win_givens_B_K<MODE>(v, gp, gl, gt, rng)`` -- the fixed triangular Givens
  network of a ``B x B`` window unitary (host side: ``triangle_decompose`` in
  plan.cpp) applied to the member array ``v``; the coefficients
  ``(c, Re s, Im s)`` of each rotation, in network order, are read by
  ``win_coef<MODE>``.  The network is: for r in 0..B-2, for col from B-1 down
  to r+1, rotate local orbitals (col-1, col).
* ``WinNet<B, K>`` -- the member count and the network as a template, for the
  stage kernels of stages.cuh.
* ``win_group_B_K(s, off, ...)`` -- loads the members ``s[off[j]]`` into
  registers, applies the network and stores them back; ``WinDispatch<B>``
  selects the function for a runtime K (shared-memory sector kernel).

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
    b(b-1)/2 (keeps the instruction footprint small).  MODE selects how the
    coefficients are read (see ``win_coef`` in kernels.cuh)."""
    ms = members(b, k)
    index = {w: j for j, w in enumerate(ms)}
    n = len(ms)
    lines = [
        "template <int MODE>",
        f"__device__ __forceinline__ void win_givens_{b}_{k}(float2 (&v)[{max(n, 1)}], const float* __restrict__ gp,"
        " const float* __restrict__ gl, const unsigned* __restrict__ gt, unsigned& rng) {",
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
            lines.append("      float c, sr, si, cl, srl, sil;")
            lines.append("      win_coef<MODE>(gp, gl, gt, g, rng, c, sr, si, cl, srl, sil);")
            for x, y in pairs:
                lines.append(f"      rot_pair<MODE == 1>(v[{x}], v[{y}], c, sr, si, cl, srl, sil);")
        lines.append("      ++g;")
        lines.append("    }")
    lines.append("  }")
    lines.append("}")
    return "\n".join(lines)


def emit_groups(b: int) -> str:
    """Per (b, k): ``WinNet<b, k>`` (member count and network) and, for the
    shared-memory sector kernel, a group function on members at s[off[j]]."""
    lines = []
    for k in range(0, b + 1):
        m = math.comb(b, k)
        lines.append(
            f"template <> struct WinNet<{b}, {k}> {{\n"
            f"  static constexpr int M = {m};\n"
            f"  template <int MODE> static __device__ __forceinline__ void apply(float2 (&v)[{m}], const float* gp,"
            f" const float* gl, const unsigned* gt, unsigned& rng) {{\n"
            f"    win_givens_{b}_{k}<MODE>(v, gp, gl, gt, rng);\n  }}\n}};"
        )
        lines.append(
            f"template <bool COMP> static __device__ __noinline__ void win_group_{b}_{k}(float2* __restrict__ s,"
            f" const int* __restrict__ off, const float* __restrict__ gp, const float* __restrict__ gl) {{\n"
            f"  float2 v[{m}];\n"
            f"  unsigned rng = 0;\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) v[j] = s[off[j]];\n"
            f"  win_givens_{b}_{k}<COMP ? 1 : 0>(v, gp, gl, nullptr, rng);\n"
            f"#pragma unroll\n  for (int j = 0; j < {m}; ++j) s[off[j]] = v[j];\n}}"
        )
    lines.append(f"template <> struct WinDispatch<{b}> {{")
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
        "template <int B, int K> struct WinNet;",
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
