"""Emit ``windows_gen.cuh``: straight-line register code for window stages.

A *window* is a block of ``B`` consecutive orbitals.  Strings of one spin
sector that share their occupation outside the window form a *group*; a
group with ``K`` electrons inside the window has ``C(B, K)`` members, listed
here in colexicographic (= ascending integer) order of their window bits.
Every orbital rotation acting only inside the window maps the group to
itself, so one thread can hold the whole group in registers and apply all of
the window's Givens rotations without touching shared memory in between.

For each (B, K) this script writes:

* ``win_givens_B_K<MODE>(v, gp, gl, gt, rng)`` -- the rectangular ("brick")
  Givens network of a ``B x B`` window unitary (host side: ``brick_decompose``
  in plan.cpp) applied to the member array ``v``; the coefficients
  ``(c, Re s, Im s)`` of each rotation, in network order, are read by
  ``win_coef<MODE>``.  The network is B layers alternating the rotations
  (0,1),(2,3),... and (1,2),(3,4),..., emitted as a loop over layer pairs whose
  body has no conditionals.
* ``WinNet<B, K>`` -- the member count and the network as a template, for the
  stage kernels of stages.cuh.
* ``win_group_B_K(s, off, ...)`` -- loads the members ``s[off[j]]`` into
  registers, applies the network and stores them back; ``WinDispatch<B>``
  selects the function for a runtime K (shared-memory sector kernel).
* ``win_pair_B_K`` / ``win_self_B_K`` and ``WinPack<B, K>`` -- the same
  network on complement-packed members (see the section below), checked
  against the plain network by a model run at generation time.

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


def layer_pairs(b: int, parity: int) -> list[int]:
    """Lower orbital l of the rotations (l, l+1) of one brick layer."""
    return list(range(parity, b - 1, 2))


def brick(b: int) -> list[int]:
    """Local lower index l of each rotation in network order (b layers,
    alternating even and odd pairs; plan.cpp brick_order)."""
    return [l for t in range(b) for l in layer_pairs(b, t % 2)]


def _rolled(b: int, layer_code) -> list[str]:
    """Brick network as a loop over (even, odd) layer pairs with one trailing
    even layer for odd b: the loop body has no conditionals, so the members
    stay in the same registers across iterations."""
    ne, no = len(layer_pairs(b, 0)), len(layer_pairs(b, 1))
    lines = []
    if b < 2:
        return lines
    lines.append("  int g = 0;")
    lines.append("#pragma unroll 1")
    lines.append(f"  for (int t = 0; t < {b // 2}; ++t) {{")
    lines += ["  " + x for x in layer_code(0, "g")]
    lines += ["  " + x for x in layer_code(1, f"g + {ne}")]
    lines.append(f"    g += {ne + no};")
    lines.append("  }")
    if b % 2:
        lines += layer_code(0, "g")
    return lines


def emit_givens(b: int, k: int) -> str:
    ms = members(b, k)
    index = {w: j for j, w in enumerate(ms)}
    n = len(ms)

    def layer(parity, g0):
        out = []
        for i, l in enumerate(layer_pairs(b, parity)):
            pairs = [(index[w], index[w ^ (3 << l)]) for w in ms if (w >> l) & 1 and not (w >> (l + 1)) & 1]
            if not pairs:
                continue
            out.append("  {")
            out.append("    float c, sr, si, cl, srl, sil;")
            out.append(f"    win_coef<MODE>(gp, gl, gt, {g0} + {i}, rng, c, sr, si, cl, srl, sil);")
            for x, y in pairs:
                out.append(f"    rot_pair<MODE == 1>(v[{x}], v[{y}], c, sr, si, cl, srl, sil);")
            out.append("  }")
        return out

    lines = [
        "template <int MODE>",
        f"__device__ __forceinline__ void win_givens_{b}_{k}(float2 (&v)[{max(n, 1)}], const float* __restrict__ gp,"
        " const float* __restrict__ gl, const unsigned* __restrict__ gt, unsigned& rng) {",
    ]
    lines += _rolled(b, layer)
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


# ---------------------------------------------------------------------------
# complement-packed networks
# ---------------------------------------------------------------------------
# A pack holds two members whose window patterns are complements, in split
# form: R = (re0, re1), I = (im0, im1) as two FP32x2 registers.  An adjacent
# rotation (l, l+1) maps complement pairs to complement pairs, and the two
# lanes of a pack always play opposite roles (one holds the lower orbital,
# the other the upper one), so one rotation of two packs is 12 packed FMAs with
# no lane swaps (complex rotations on (re, im) pairs need two swaps each).
#   pair: lane 0 = member j of a group with K electrons in the window, lane 1 =
#         the complement member of a group with B - K electrons (K < B - K).
#   self: K = B/2; the members with window bit 0 clear take lane 0.  Only
#         rotation (0, 1) then pairs lane 0 with lane 1 of the partner pack,
#         which costs lane swaps (it occurs once per network).


def comp_index(b: int, k: int) -> list[int]:
    """For member j of class k: index of its complement in class b - k."""
    full = (1 << b) - 1
    other = {w: j for j, w in enumerate(members(b, b - k))}
    return [other[full ^ w] for w in members(b, k)]


def pack_lanes(b: int, k: int, kind: str) -> list[tuple[int, int]]:
    """Window patterns (lane 0, lane 1) of every pack."""
    full = (1 << b) - 1
    if kind == "pair":
        return [(w, full ^ w) for w in members(b, k)]
    return [(w, full ^ w) for w in members(b, k) if not w & 1]


def pack_schedule(b: int, k: int, kind: str) -> list[list[tuple[int, int, bool, bool, bool]]]:
    """Per rotation pattern col (b-1 down to 1; pair (col-1, col)): the ops
    (p, q, swap, vp_a, vq_a).  swap: lane 0 of p partners lane 1 of q.
    vp_a: lane 0 of p holds the lower orbital (coefficients (s, -conj s)),
    otherwise (-conj s, s); likewise vq_a for q."""
    lanes = pack_lanes(b, k, kind)
    where = {}
    for p, (w0, w1) in enumerate(lanes):
        where[w0] = (p, 0)
        where[w1] = (p, 1)
    out = []
    for col in range(b - 1, 0, -1):
        l = col - 1
        m = 3 << l
        ops, seen = [], set()
        for p, (w0, _) in enumerate(lanes):
            if ((w0 >> l) & 1) == ((w0 >> (l + 1)) & 1) or p in seen:
                continue
            q, lam = where[w0 ^ m]
            seen.add(p)
            seen.add(q)
            vp_a = bool((w0 >> l) & 1)
            swap = lam == 1
            q0 = lanes[q][0]
            vq_a = bool((q0 >> l) & 1)
            ops.append((p, q, swap, vp_a, vq_a))
        out.append(ops)
    return out


def _model_check(b: int, k: int, kind: str) -> None:
    """Packed schedule == plain network on random data (complex128 model)."""
    import random

    rnd = random.Random(1000 * b + k)
    nrot = b * (b - 1) // 2
    coefs = []
    for _ in range(nrot):
        c = rnd.uniform(-1, 1)
        ph = rnd.uniform(0, 6.283)
        r = (1 - c * c) ** 0.5
        coefs.append((c, complex(r * __import__("math").cos(ph), r * __import__("math").sin(ph))))

    def plain(bb, kk, v):
        ms = members(bb, kk)
        idx = {w: j for j, w in enumerate(ms)}
        v = list(v)
        for g, l in enumerate(brick(bb)):
            c, s = coefs[g]
            for w in ms:
                if (w >> l) & 1 and not (w >> (l + 1)) & 1:
                    x, y = idx[w], idx[w ^ (3 << l)]
                    v[x], v[y] = c * v[x] + s * v[y], -s.conjugate() * v[x] + c * v[y]
        return v

    lanes = pack_lanes(b, k, kind)
    sched = pack_schedule(b, k, kind)
    if kind == "pair":
        va = [complex(rnd.gauss(0, 1), rnd.gauss(0, 1)) for _ in members(b, k)]
        vb = [complex(rnd.gauss(0, 1), rnd.gauss(0, 1)) for _ in members(b, b - k)]
        ia = {w: j for j, w in enumerate(members(b, k))}
        ib = {w: j for j, w in enumerate(members(b, b - k))}
        P = [[va[ia[w0]], vb[ib[w1]]] for w0, w1 in lanes]
        want_a, want_b = plain(b, k, va), plain(b, b - k, vb)
    else:
        v = [complex(rnd.gauss(0, 1), rnd.gauss(0, 1)) for _ in members(b, k)]
        iv = {w: j for j, w in enumerate(members(b, k))}
        P = [[v[iv[w0]], v[iv[w1]]] for w0, w1 in lanes]
        want = plain(b, k, v)
    for g, l in enumerate(brick(b)):
        ci = b - 1 - (l + 1)
        if True:
            c, s = coefs[g]
            A, Bv = (s, -s.conjugate()), (-s.conjugate(), s)
            for p, q, swap, vp_a, vq_a in sched[ci]:
                Pp, Qq = P[p], P[q]
                Qx = [Qq[1], Qq[0]] if swap else Qq
                Px = [Pp[1], Pp[0]] if swap else Pp
                vp, vq = (A if vp_a else Bv), (A if vq_a else Bv)
                P[p] = [c * Pp[t] + vp[t] * Qx[t] for t in range(2)]
                P[q] = [c * Qq[t] + vq[t] * Px[t] for t in range(2)]
    if kind == "pair":
        for pi, (w0, w1) in enumerate(lanes):
            assert abs(P[pi][0] - want_a[ia[w0]]) < 1e-9 and abs(P[pi][1] - want_b[ib[w1]]) < 1e-9, (b, k)
    else:
        for pi, (w0, w1) in enumerate(lanes):
            assert abs(P[pi][0] - want[iv[w0]]) < 1e-9 and abs(P[pi][1] - want[iv[w1]]) < 1e-9, (b, k)


def pack_kind(b: int, k: int) -> str | None:
    if 2 * k == b:
        return "self"
    if 2 * k < b and math.comb(b, k) <= 35:
        return "pair"
    return None


def emit_packed(b: int, k: int, kind: str) -> str:
    lanes = pack_lanes(b, k, kind)
    sched = pack_schedule(b, k, kind)  # indexed by col = l + 1 from b - 1 down to 1
    n = len(lanes)
    name = f"win_{kind}_{b}_{k}"

    def layer(parity, g0):
        out = []
        for i, l in enumerate(layer_pairs(b, parity)):
            ops = sched[b - 1 - (l + 1)]
            if not ops:
                continue
            out.append("  {")
            out.append("    PackCoef pc;")
            out.append(f"    pack_coef<MODE>(gp, gl, gt, {g0} + {i}, rng, pc);")
            for p, q, swap, vp_a, vq_a in ops:
                fn = "rot_pack_x" if swap else "rot_pack"
                out.append(f"    {fn}<{str(vp_a).lower()}, {str(vq_a).lower()}>(R[{p}], I[{p}], R[{q}], I[{q}], pc);")
            out.append("  }")
        return out

    lines = [
        "template <int MODE>",
        f"__device__ __forceinline__ void {name}(float2 (&R)[{n}], float2 (&I)[{n}], const float* __restrict__ gp,"
        " const float* __restrict__ gl, const unsigned* __restrict__ gt, unsigned& rng) {",
    ]
    lines += _rolled(b, layer)
    lines.append("}")
    # lane tables: member index (class K, and class B-K for lane 1 of pairs)
    ia = {w: j for j, w in enumerate(members(b, k))}
    ib = {w: j for j, w in enumerate(members(b, b - k))}
    l0 = ", ".join(str(ia[w0]) for w0, _ in lanes)
    l1 = ", ".join(str((ib if kind == "pair" else ia)[w1]) for _, w1 in lanes)
    p0 = ", ".join(str(w0) for w0, _ in lanes)
    p1 = ", ".join(str(w1) for _, w1 in lanes)
    lines.append(
        f"template <> struct WinPack<{b}, {k}> {{\n"
        f"  static constexpr int NP = {n};\n"
        f"  static constexpr bool PAIR = {'true' if kind == 'pair' else 'false'};\n"
        f"  // member index of lane 0 / lane 1 (lane 1 indexes class B - K for pairs) and window patterns\n"
        f"  static __host__ __device__ constexpr int lane0(int q) {{ constexpr int t[{n}] = {{{l0}}}; return t[q]; }}\n"
        f"  static __host__ __device__ constexpr int lane1(int q) {{ constexpr int t[{n}] = {{{l1}}}; return t[q]; }}\n"
        f"  static __host__ __device__ constexpr unsigned pat0(int q) {{ constexpr unsigned t[{n}] = {{{p0}}}; return t[q]; }}\n"
        f"  static __host__ __device__ constexpr unsigned pat1(int q) {{ constexpr unsigned t[{n}] = {{{p1}}}; return t[q]; }}\n"
        f"  template <int MODE> static __device__ __forceinline__ void apply(float2 (&R)[{n}], float2 (&I)[{n}],"
        f" const float* gp, const float* gl, const unsigned* gt, unsigned& rng) {{\n"
        f"    {name}<MODE>(R, I, gp, gl, gt, rng);\n  }}\n}};"
    )
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
    parts.append("template <int B, int K> struct WinPack { static constexpr int NP = 0; };")
    for b in range(2, MAX_B + 1):
        for k in range(0, b + 1):
            kind = pack_kind(b, k)
            if kind:
                _model_check(b, k, kind)
                parts.append(emit_packed(b, k, kind))
    Path(out_path).write_text("\n".join(parts) + "\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "windows_gen.cuh")
    assert math.comb(8, 4) == len(members(8, 4))
