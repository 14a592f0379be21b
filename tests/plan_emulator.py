"""NumPy emulation of the sector kernel's stage program (test helper).

Applies a plan serialized by ``ffgb_debug_plan`` to one sector vector with the
same addressing the CUDA kernel uses (group bases from the half-sector rank
tables, member order, cross-half partner ranks and fermionic signs), so the
host factorization and the index arithmetic can be checked on the CPU.
"""

from __future__ import annotations

import itertools
import math

import numpy as np


def _members(b, k):
    return sorted(sum(1 << i for i in c) for c in itertools.combinations(range(b), k))


def _triangle(b):
    return [col - 1 for r in range(b - 1) for col in range(b - 1, r, -1)]


def _brick(b):
    """Window networks: b layers alternating the pairs (0,1),(2,3),... and (1,2),(3,4),..."""
    return [l for t in range(b) for l in range(t % 2, b - 1, 2)]


def _rank_shifted(s, base, m0):
    r, t = 0, m0
    p = 0
    while s:
        if s & 1:
            t += 1
            r += math.comb(base + p, t)
        s >>= 1
        p += 1
    return r


def parse(buf):
    it = iter(buf)
    kind = int(next(it))
    h = int(next(it))
    err = float(next(it))

    def giv():
        n = int(next(it))
        return [(next(it), complex(next(it), next(it))) for _ in range(n)]

    tri, b1, b2, a1, a2 = giv(), giv(), giv(), giv(), giv()
    ncs = int(next(it))
    cs = []
    for _ in range(ncs):
        i, j = int(next(it)), int(next(it))
        g = [complex(next(it), next(it)) for _ in range(4)]
        cs.append((i, j, g))
    nd = int(next(it))
    diag = np.array([complex(next(it), next(it)) for _ in range(nd)])
    ops = []
    for _ in range(int(next(it))):
        typ, lo, b = int(next(it)), int(next(it)), int(next(it))
        net = giv()
        pairs = []
        for _ in range(int(next(it))):
            i, j = int(next(it)), int(next(it))
            pairs.append((i, j, [complex(next(it), next(it)) for _ in range(4)]))
        ops.append(dict(type=typ, lo=lo, b=b, net=net, pairs=pairs))
    nd = int(next(it))
    ops_diag = np.array([complex(next(it), next(it)) for _ in range(nd)])
    return dict(kind=kind, h=h, err=err, tri=tri, b1=b1, b2=b2, a1=a1, a2=a2, cs=cs, diag=diag, ops=ops,
                ops_diag=ops_diag)


def apply_ops(plan, vec, norb, nocc):
    """The stage sequence of a cosine-sine plan applied string by string:
    window networks on orbitals (lo + l, lo + l + 1) and cross-half rotations
    on (i, j) with the fermionic sign of the occupied orbitals between them,
    then the final orbital phases."""
    v = np.array(vec, dtype=complex)
    strings = sorted(sum(1 << i for i in c) for c in itertools.combinations(range(norb), nocc))
    addr = {s: a for a, s in enumerate(strings)}
    for op in plan["ops"]:
        if op["type"] == 0:
            for (c, s), l in zip(op["net"], _brick(op["b"])):
                a = op["lo"] + l
                for st in strings:
                    if (st >> a) & 1 and not (st >> (a + 1)) & 1:
                        _rot(v, addr[st], addr[st ^ (3 << a)], c, s)
        else:
            for pi, pj, g in op["pairs"]:
                between = ((1 << pj) - 1) & ~((1 << (pi + 1)) - 1)
                for st in strings:
                    if (st >> pi) & 1 and not (st >> pj) & 1:
                        x, y = addr[st], addr[st ^ (1 << pi) ^ (1 << pj)]
                        sgn = -1.0 if bin(st & between).count("1") & 1 else 1.0
                        vx, vy = v[x], v[y]
                        v[x] = g[0] * vx + g[1] * sgn * vy
                        v[y] = g[2] * sgn * vx + g[3] * vy
    d = plan["ops_diag"]
    for a, st in enumerate(strings):
        ph = 1.0 + 0j
        for i in range(norb):
            if (st >> i) & 1:
                ph *= d[i]
        v[a] *= ph
    return v


def _rot(v, x, y, c, s):
    vx, vy = v[x], v[y]
    v[x] = c * vx + s * vy
    v[y] = -np.conj(s) * vx + c * vy


def _win(v, b, gp):
    """triangle network on a member array (members of one group)."""
    return v  # placeholder (replaced below)


def apply_plan(plan, vec, norb, nocc):
    v = np.array(vec, dtype=complex)
    kind = plan["kind"]
    strings = sorted(sum(1 << i for i in c) for c in itertools.combinations(range(norb), nocc))
    addr = {s: a for a, s in enumerate(strings)}
    if kind in (1, 2):  # TRIANGLE or FULL: adjacent rotations over the whole sector
        for (c, s), l in zip(plan["tri"], _triangle(norb) if kind == 1 else _brick(norb)):
            for st in strings:
                if (st >> l) & 1 and not (st >> (l + 1)) & 1:
                    _rot(v, addr[st], addr[st ^ (3 << l)], c, s)
    elif kind == 3:
        H = plan["h"]
        Q = norb - H

        def window_low(gp):
            for k in range(max(0, nocc - Q), min(H, nocc) + 1):
                m = nocc - k
                mem = _members(H, k)
                for s2 in _members(Q, m):
                    base = _rank_shifted(s2, H, k)
                    idx = [base + j for j in range(len(mem))]
                    grp = v[idx].copy()
                    local = {w: j for j, w in enumerate(mem)}
                    for (c, s), l in zip(gp, _brick(H)):
                        for w in mem:
                            if (w >> l) & 1 and not (w >> (l + 1)) & 1:
                                _rot(grp, local[w], local[w ^ (3 << l)], c, s)
                    v[idx] = grp

        def window_high(gp):
            for k in range(max(0, nocc - H), min(Q, nocc) + 1):
                mem = _members(Q, k)
                offs = [_rank_shifted(w, H, nocc - k) for w in mem]
                for g in range(math.comb(H, nocc - k)):
                    idx = [g + o for o in offs]
                    grp = v[idx].copy()
                    local = {w: j for j, w in enumerate(mem)}
                    for (c, s), l in zip(gp, _brick(Q)):
                        for w in mem:
                            if (w >> l) & 1 and not (w >> (l + 1)) & 1:
                                _rot(grp, local[w], local[w ^ (3 << l)], c, s)
                    v[idx] = grp

        window_low(plan["b1"])
        window_high(plan["b2"])
        for i, (pi, pj, g) in enumerate(plan["cs"]):
            assert pi == i and pj == H + i
            for k in range(max(1, nocc - Q), min(H, nocc) + 1):
                m = nocc - k
                mem = _members(H, k)
                prev = {w: j for j, w in enumerate(_members(H, k - 1))}
                for s2 in _members(Q, m):
                    if (s2 >> i) & 1:
                        continue
                    bx = _rank_shifted(s2, H, k)
                    by = _rank_shifted(s2 | (1 << i), H, k - 1)
                    sg0 = bin(s2 & ((1 << i) - 1)).count("1") & 1
                    for j, w in enumerate(mem):
                        if not (w >> i) & 1:
                            continue
                        jp = prev[w ^ (1 << i)]
                        par = bin(w >> (i + 1)).count("1") & 1
                        sgn = -1.0 if (par ^ sg0) else 1.0
                        x, y = v[bx + j], v[by + jp]
                        v[bx + j] = g[0] * x + g[1] * sgn * y
                        v[by + jp] = g[2] * sgn * x + g[3] * y
        window_low(plan["a1"])
        window_high(plan["a2"])
    # final orbital phases
    d = plan["diag"]
    if len(d):
        for a, st in enumerate(strings):
            ph = 1.0 + 0j
            for i in range(norb):
                if (st >> i) & 1:
                    ph *= d[i]
            v[a] *= ph
    return v
