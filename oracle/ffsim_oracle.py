"""FP64 CPU oracle for the ffsim statevector gate path.

TEST INFRASTRUCTURE ONLY.  This module is the checker that the CUDA path is
compared against.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.
The product package ``ffsim_gb300`` never imports, calls or falls back to it.

It restates, in NumPy complex128, the algorithm of the reference (ffsim)
for every function on the hot path.  Each function cites the reference file
and lines it follows (paths are relative to the ffsim project root):

* string tables          python/ffsim/_cistring.py:21-30 (pyscf cistring order:
                         ascending integer bitstrings, pinned by
                         tests/python/states/bitstring_test.py:24-60)
* pair / occupied subsets python/ffsim/gates/orbital_rotation.py:202-236
* Givens decomposition   src/linalg/givens.rs:20-149
* Givens row rotation    src/gates/orbital_rotation.rs:18-104
* phase shift            src/gates/phase_shift.rs:17-30
* orbital rotation       python/ffsim/gates/orbital_rotation.py:44-174
* diag-Coulomb evolution python/ffsim/gates/diag_coulomb.py:68-275,
                         src/gates/diag_coulomb.rs:19-190
* num-op-sum evolution   python/ffsim/gates/num_op_sum.py:62-236,
                         src/gates/num_op_sum.rs:18-36
* contractions           python/ffsim/contract/diag_coulomb.py:41-192,
                         src/contract/diag_coulomb.rs:22-174,
                         python/ffsim/contract/num_op_sum.py:27-72,
                         src/contract/num_op_sum.rs:20-39
* linear operators       python/ffsim/contract/diag_coulomb.py:195-272,
                         python/ffsim/contract/num_op_sum.py:75-131,
                         python/ffsim/hamiltonians/double_factorized_hamiltonian.py:244-275
* UCJ apply_unitary      python/ffsim/variational/ucj_spin_balanced.py:657-696,
                         ucj_spin_unbalanced.py, ucj_spinless.py
* parameter maps         python/ffsim/linalg/util.py:93-124,212-232
* one-body operators,    python/ffsim/contract/one_body.py:24-90,
  1- and 2-RDMs          python/ffsim/states/rdm.py:73-274
* molecular Hamiltonian  python/ffsim/hamiltonians/molecular_hamiltonian.py:24-173
* Trotter evolution      python/ffsim/trotter/double_factorized.py:25-127,
                         python/ffsim/trotter/_util.py:18-60,
                         python/ffsim/trotter/diagonal_coulomb_split_op.py:25-122
* diagonal Coulomb       python/ffsim/hamiltonians/diagonal_coulomb_hamiltonian.py:67-97,208-238
  Hamiltonian
* random inputs          python/ffsim/random/random.py:24-47,84-106,549-560,563-665

Parity pins: tests/golden/make_golden.py runs the reference's own Python
orchestration (with its pure-Python kernel restatements from
python/ffsim/_slow/) and records golden vectors that tests/test_oracle.py
checks this module against, together with the reference's closed-form
known-answer tests.
"""

from __future__ import annotations

import itertools
import math
from functools import lru_cache

import numpy as np
import scipy.linalg

# ---------------------------------------------------------------------------
# string indexing (python/ffsim/_cistring.py:21-30)
# ---------------------------------------------------------------------------


@lru_cache(maxsize=None)
def make_strings(norb: int, nocc: int) -> np.ndarray:
    """Bitstrings with ``nocc`` set bits among ``norb``, in address order.

    Address order is ascending integer order (pyscf cistring order, pinned by
    the reference's bitstring KATs: norb=3, nocc=2 -> [0b011, 0b101, 0b110]).
    """
    if nocc < 0 or nocc > norb:
        return np.zeros(0, dtype=np.int64)
    out = [sum(1 << i for i in c) for c in itertools.combinations(range(norb), nocc)]
    out.sort()
    return np.asarray(out, dtype=np.int64)


@lru_cache(maxsize=None)
def gen_occslst(norb: int, nocc: int) -> np.ndarray:
    """Occupied-orbital lists, ascending within each string, in address order."""
    strings = make_strings(norb, nocc)
    occ = np.zeros((len(strings), nocc), dtype=np.int64)
    for a, s in enumerate(strings):
        occ[a] = [i for i in range(norb) if (int(s) >> i) & 1]
    return occ


def _occ_mask(norb: int, nocc: int) -> np.ndarray:
    """Boolean occupation matrix [dim, norb]."""
    strings = make_strings(norb, nocc)
    return ((strings[:, None] >> np.arange(norb)[None, :]) & 1).astype(bool)


@lru_cache(maxsize=None)
def zero_one_subspace_indices(norb: int, nocc: int, target_orbs: tuple) -> np.ndarray:
    """Addresses where (i, j) are 10 followed by their 01 partners.

    Follows python/ffsim/gates/orbital_rotation.py:202-212 and :228-236: the
    target orbitals are relabelled to the two highest bits, strings sorted by
    the relabelled value; the slice [n00, len - n11) holds first the strings
    with i occupied / j empty and then, in the same order of the remaining
    bits, the strings with j occupied / i empty.
    """
    i, j = target_orbs
    strings = make_strings(norb, nocc)
    relabel = _shifted_orbitals(norb, target_orbs)
    relabelled = np.zeros_like(strings)
    for p in range(norb):
        relabelled |= ((strings >> p) & 1) << int(relabel[p])
    indices = np.argsort(relabelled, kind="stable")
    n00 = math.comb(norb - 2, nocc)
    n11 = math.comb(norb - 2, nocc - 2) if nocc >= 2 else 0
    return indices[n00 : len(indices) - n11]


@lru_cache(maxsize=None)
def one_subspace_indices(norb: int, nocc: int, target_orbs: tuple) -> np.ndarray:
    """Addresses where every target orbital is occupied (orbital_rotation.py:215-225)."""
    strings = make_strings(norb, nocc)
    relabel = _shifted_orbitals(norb, target_orbs)
    relabelled = np.zeros_like(strings)
    for p in range(norb):
        relabelled |= ((strings >> p) & 1) << int(relabel[p])
    indices = np.argsort(relabelled, kind="stable")
    n0 = math.comb(norb, nocc)
    if nocc >= len(target_orbs):
        n0 -= math.comb(norb - len(target_orbs), nocc - len(target_orbs))
    return indices[n0:]


def _shifted_orbitals(norb: int, target_orbs: tuple) -> np.ndarray:
    """Orbital relabelling with the targets moved to the top (orbital_rotation.py:228-236)."""
    k = len(target_orbs)
    orbitals = list(range(norb - k))
    for index, val in sorted(zip(target_orbs, range(norb - k, norb))):
        orbitals.insert(index, val)
    return np.asarray(orbitals)


def dim(norb: int, nelec) -> int:
    if isinstance(nelec, int):
        return math.comb(norb, nelec)
    return math.comb(norb, nelec[0]) * math.comb(norb, nelec[1])


# ---------------------------------------------------------------------------
# Givens decomposition (src/linalg/givens.rs:20-149)
# ---------------------------------------------------------------------------


def _zrotg_safe(a: complex, b: complex, tol: float):
    """givens.rs:20-34."""
    abs_a = abs(a)
    abs_b = abs(b)
    if abs_b <= tol:
        return 1.0, 0j
    if abs_a <= tol:
        return 0.0, 1 + 0j
    r = math.hypot(abs_a, abs_b)
    c = abs_a / r
    s = (a / abs_a) * b.conjugate() / r
    return min(max(c, -1.0), 1.0), s


def _rotate_columns(mat, x, y, c, s):
    """givens.rs:36-50."""
    xo = mat[:, x].copy()
    yo = mat[:, y].copy()
    mat[:, x] = c * xo + s * yo
    mat[:, y] = c * yo - s.conjugate() * xo


def _rotate_rows(mat, x, y, c, s):
    """givens.rs:52-66."""
    xo = mat[x, :].copy()
    yo = mat[y, :].copy()
    mat[x, :] = c * xo + s * yo
    mat[y, :] = c * yo - s.conjugate() * xo


def givens_decomposition(mat: np.ndarray, tol: float = 1e-12):
    """Clements-style decomposition ``U = D G_L^* ... G_1^*`` (givens.rs:68-149).

    Returns (list of (c, s, i, j), diagonal ndarray).
    """
    mat = np.asarray(mat, dtype=complex)
    if mat.ndim != 2 or mat.shape[0] != mat.shape[1]:
        raise ValueError("mat must be a square matrix")
    n = mat.shape[0]
    cur = mat.copy()
    left = []
    right = []
    for i in range(max(n - 1, 0)):
        if i % 2 == 0:
            for j in range(i + 1):
                target = i - j
                row = n - j - 1
                if abs(cur[row, target]) > tol:
                    c, s = _zrotg_safe(cur[row, target + 1], cur[row, target], tol)
                    right.append((c, s, target + 1, target))
                    _rotate_columns(cur, target + 1, target, c, s)
        else:
            for j in range(i + 1):
                target = n - i + j - 1
                col = j
                if abs(cur[target, col]) > tol:
                    c, s = _zrotg_safe(cur[target - 1, col], cur[target, col], tol)
                    left.append((c, s, target - 1, target))
                    _rotate_rows(cur, target - 1, target, c, s)
    for c_left, s_left, i, j in reversed(left):
        c, s = _zrotg_safe(c_left * cur[j, j], s_left.conjugate() * cur[i, i], tol)
        right.append((c, -s.conjugate(), i, j))
        di = cur[i, i]
        dj = cur[j, j]
        g00 = c * di
        g01 = -s * dj
        g10 = s.conjugate() * di
        g11 = c * dj
        c_new, s_new = _zrotg_safe(g11, g10, tol)
        cur[i, i] = g00 * c_new + g01 * (-s_new.conjugate())
        cur[j, j] = g10 * s_new + g11 * c_new
    return right, np.diagonal(cur).copy()


# ---------------------------------------------------------------------------
# elementary kernels (src/gates/*.rs)
# ---------------------------------------------------------------------------


def apply_givens_rotation_in_place(vec2d, c, s, slice1, slice2):
    """orbital_rotation.rs:86-104 applied to every pair (rows)."""
    if len(slice1) == 0:
        return
    r1 = vec2d[slice1].copy()
    r2 = vec2d[slice2].copy()
    vec2d[slice1] = c * r1 + s * r2
    vec2d[slice2] = c * r2 - np.conj(s) * r1


def apply_phase_shift_in_place(vec2d, phase, indices):
    """phase_shift.rs:17-30."""
    vec2d[indices] *= phase


def _apply_adjacent(vec2d, c, s, target_orbs, norb, nocc):
    """orbital_rotation.py:177-199."""
    i, j = target_orbs
    assert i == j + 1 or i == j - 1, "Target orbitals must be adjacent."
    idx = zero_one_subspace_indices(norb, nocc, (i, j))
    half = len(idx) // 2
    apply_givens_rotation_in_place(vec2d, c, s, idx[:half], idx[half:])


def _apply_decomp(vec2d, decomp, norb, nocc):
    rotations, phases = decomp
    for c, s, i, j in rotations:
        _apply_adjacent(vec2d, c, s.conjugate(), (i, j), norb, nocc)
    for i, ph in enumerate(phases):
        apply_phase_shift_in_place(vec2d, ph, one_subspace_indices(norb, nocc, (i,)))


def _get_givens(mat):
    """orbital_rotation.py:157-174."""
    if isinstance(mat, np.ndarray) and mat.ndim == 2:
        d = givens_decomposition(mat)
        return d, d
    mat_a, mat_b = mat
    da = givens_decomposition(mat_a) if mat_a is not None else None
    db = givens_decomposition(mat_b) if mat_b is not None else None
    return da, db


def apply_orbital_rotation(vec, mat, norb, nelec, *, copy=True):
    """orbital_rotation.py:44-154."""
    vec = np.array(vec, dtype=complex, copy=True) if copy else np.asarray(vec, dtype=complex)
    if isinstance(nelec, int):
        decomp = givens_decomposition(mat)
        v = np.ascontiguousarray(vec.reshape((-1, 1)))
        _apply_decomp(v, decomp, norb, nelec)
        return v.reshape(-1)
    da, db = _get_givens(mat)
    n_alpha, n_beta = nelec
    dim_a = math.comb(norb, n_alpha)
    dim_b = math.comb(norb, n_beta)
    v = np.ascontiguousarray(vec.reshape((dim_a, dim_b)))
    if da is not None:
        _apply_decomp(v, da, norb, n_alpha)
    if db is not None:
        v = np.ascontiguousarray(v.T)
        _apply_decomp(v, db, norb, n_beta)
        v = v.T
    return np.ascontiguousarray(v).reshape(-1)


def _conj_rotation(orbital_rotation):
    """contract/diag_coulomb.py:28-38."""
    if isinstance(orbital_rotation, np.ndarray) and orbital_rotation.ndim == 2:
        return orbital_rotation.T.conj()
    a, b = orbital_rotation
    return (a.T.conj() if a is not None else None, b.T.conj() if b is not None else None)


# ---------------------------------------------------------------------------
# diagonal Coulomb evolution (gates/diag_coulomb.py:156-275, diag_coulomb.rs)
# ---------------------------------------------------------------------------


def get_mat_exp(mat, time, norb, z_representation):
    """diag_coulomb.py:223-275."""
    if isinstance(mat, np.ndarray) and mat.ndim == 2:
        aa, ab = mat.astype(float).copy(), mat.astype(float).copy()
        aa[np.diag_indices(norb)] *= 0.5
        if z_representation:
            aa *= 0.25
            ab *= 0.25
        ea = np.exp(-1j * time * aa)
        return ea, np.exp(-1j * time * ab), ea
    aa, ab, bb = mat
    if aa is None:
        ea = np.ones((norb, norb), dtype=complex)
    else:
        aa = np.array(aa, dtype=float)
        aa[np.diag_indices(norb)] *= 0.5
        if z_representation:
            aa *= 0.25
        ea = np.exp(-1j * time * aa)
    if bb is None:
        eb = np.ones((norb, norb), dtype=complex)
    else:
        bb = np.array(bb, dtype=float)
        bb[np.diag_indices(norb)] *= 0.5
        if z_representation:
            bb *= 0.25
        eb = np.exp(-1j * time * bb)
    if ab is None:
        eab = np.ones((norb, norb), dtype=complex)
    else:
        ab = np.array(ab, dtype=float)
        if z_representation:
            ab = ab * 0.25
        eab = np.exp(-1j * time * ab)
    return ea, eab, eb


def diag_coulomb_evolution_num_rep_in_place(vec2d, eaa, eab, ebb, norb, na, nb):
    """diag_coulomb.rs:19-90 (three-phase product of exponential tables)."""
    occ_a = gen_occslst(norb, na)
    occ_b = gen_occslst(norb, nb)
    dim_a, dim_b = vec2d.shape
    beta_ph = np.ones(dim_b, dtype=complex)
    for j in range(nb):
        for k in range(j, nb):
            beta_ph *= ebb[occ_b[:, j], occ_b[:, k]]
    alpha_ph = np.ones(dim_a, dtype=complex)
    phase_map = np.ones((dim_a, norb), dtype=complex)
    for j in range(na):
        phase_map *= eab[occ_a[:, j], :]
        for k in range(j, na):
            alpha_ph *= eaa[occ_a[:, j], occ_a[:, k]]
    ph = alpha_ph[:, None] * beta_ph[None, :]
    for j in range(nb):
        ph *= phase_map[:, occ_b[:, j]]
    vec2d *= ph


def diag_coulomb_evolution_z_rep_in_place(vec2d, eaa, eab, ebb, norb, na, nb):
    """diag_coulomb.rs:92-190."""
    sa = make_strings(norb, na)
    sb = make_strings(norb, nb)
    dim_a, dim_b = vec2d.shape
    eaa_c, eab_c, ebb_c = eaa.conj(), eab.conj(), ebb.conj()
    beta_ph = np.ones(dim_b, dtype=complex)
    for j in range(norb):
        bj = (sb >> j) & 1
        for k in range(j + 1, norb):
            bk = (sb >> k) & 1
            beta_ph *= np.where(bj ^ bk, ebb_c[j, k], ebb[j, k])
    alpha_ph = np.ones(dim_a, dtype=complex)
    phase_map = np.ones((dim_a, norb), dtype=complex)
    for j in range(norb):
        aj = (sa >> j) & 1
        phase_map *= np.where(aj[:, None] == 1, eab_c[j][None, :], eab[j][None, :])
        for k in range(j + 1, norb):
            ak = (sa >> k) & 1
            alpha_ph *= np.where(aj ^ ak, eaa_c[j, k], eaa[j, k])
    ph = alpha_ph[:, None] * beta_ph[None, :]
    for j in range(norb):
        bj = ((sb >> j) & 1).astype(bool)
        ph *= np.where(bj[None, :], phase_map[:, j : j + 1].conj(), phase_map[:, j : j + 1])
    vec2d *= ph


def apply_diag_coulomb_evolution(
    vec, mat, time, norb, nelec, *, orbital_rotation=None, z_representation=False, copy=True
):
    """diag_coulomb.py:68-220."""
    vec = np.array(vec, dtype=complex, copy=True) if copy else np.asarray(vec, dtype=complex)
    if isinstance(nelec, int):
        if z_representation:
            raise NotImplementedError
        nelec = (nelec, 0)
    eaa, eab, ebb = get_mat_exp(mat, time, norb, z_representation)
    na, nb = nelec
    dim_a, dim_b = math.comb(norb, na), math.comb(norb, nb)
    if orbital_rotation is not None:
        vec = apply_orbital_rotation(vec, _conj_rotation(orbital_rotation), norb, nelec, copy=False)
    v = vec.reshape((dim_a, dim_b))
    if z_representation:
        diag_coulomb_evolution_z_rep_in_place(v, eaa, eab, ebb, norb, na, nb)
    else:
        diag_coulomb_evolution_num_rep_in_place(v, eaa, eab, ebb, norb, na, nb)
    vec = v.reshape(-1)
    if orbital_rotation is not None:
        vec = apply_orbital_rotation(vec, orbital_rotation, norb, nelec, copy=False)
    return vec


# ---------------------------------------------------------------------------
# num-op-sum evolution (gates/num_op_sum.py:62-236, num_op_sum.rs:18-36)
# ---------------------------------------------------------------------------


def num_op_sum_evolution_in_place(vec2d, phases, occupations):
    """num_op_sum.rs:18-36 (rows)."""
    ph = np.ones(vec2d.shape[0], dtype=complex)
    for j in range(occupations.shape[1]):
        ph *= phases[occupations[:, j]]
    vec2d *= ph[:, None]


def apply_num_op_sum_evolution(vec, coeffs, time, norb, nelec, *, orbital_rotation=None, copy=True):
    """num_op_sum.py:62-219."""
    vec = np.array(vec, dtype=complex, copy=True) if copy else np.asarray(vec, dtype=complex)
    if isinstance(nelec, int):
        phases = np.exp(-1j * time * np.asarray(coeffs))
        if orbital_rotation is not None:
            vec = apply_orbital_rotation(vec, orbital_rotation.T.conj(), norb, nelec, copy=False)
        v = vec.reshape((-1, 1))
        num_op_sum_evolution_in_place(v, phases, gen_occslst(norb, nelec))
        vec = v.reshape(-1)
        if orbital_rotation is not None:
            vec = apply_orbital_rotation(vec, orbital_rotation, norb, nelec, copy=False)
        return vec
    if isinstance(coeffs, np.ndarray):
        pa = pb = np.exp(-1j * time * coeffs)
    else:
        ca, cb = coeffs
        pa = np.exp(-1j * time * ca) if ca is not None else None
        pb = np.exp(-1j * time * cb) if cb is not None else None
    na, nb = nelec
    dim_a, dim_b = math.comb(norb, na), math.comb(norb, nb)
    if orbital_rotation is not None:
        vec = apply_orbital_rotation(vec, _conj_rotation(orbital_rotation), norb, nelec, copy=False)
    v = vec.reshape((dim_a, dim_b))
    if pa is not None:
        num_op_sum_evolution_in_place(v, pa, gen_occslst(norb, na))
    if pb is not None:
        vt = v.T
        num_op_sum_evolution_in_place(vt, pb, gen_occslst(norb, nb))
    vec = v.reshape(-1)
    if orbital_rotation is not None:
        vec = apply_orbital_rotation(vec, orbital_rotation, norb, nelec, copy=False)
    return vec


# ---------------------------------------------------------------------------
# contractions (contract/diag_coulomb.py, contract/num_op_sum.py)
# ---------------------------------------------------------------------------


def get_mats(mat, norb, z_representation):
    """contract/diag_coulomb.py:102-130."""
    if isinstance(mat, np.ndarray):
        aa, ab = mat.astype(float), mat.astype(float)
        if not z_representation:
            aa = aa.copy()
            aa[np.diag_indices(norb)] *= 0.5
        return aa, ab, aa
    aa, ab, bb = mat
    if aa is None:
        aa = np.zeros((norb, norb))
    elif not z_representation:
        aa = np.array(aa, dtype=float)
        aa[np.diag_indices(norb)] *= 0.5
    if bb is None:
        bb = np.zeros((norb, norb))
    elif not z_representation:
        bb = np.array(bb, dtype=float)
        bb[np.diag_indices(norb)] *= 0.5
    if ab is None:
        ab = np.zeros((norb, norb))
    return np.asarray(aa, float), np.asarray(ab, float), np.asarray(bb, float)


def diag_coulomb_coeffs(mat_aa, mat_ab, mat_bb, norb, nelec, z_representation):
    """Per-amplitude real coefficient of the contraction (contract/diag_coulomb.rs:22-174)."""
    na, nb = nelec
    if not z_representation:
        occ_a = gen_occslst(norb, na)
        occ_b = gen_occslst(norb, nb)
        beta = np.zeros(len(occ_b))
        for j in range(nb):
            for k in range(j, nb):
                beta += mat_bb[occ_b[:, j], occ_b[:, k]]
        alpha = np.zeros(len(occ_a))
        cmap = np.zeros((len(occ_a), norb))
        for j in range(na):
            cmap += mat_ab[occ_a[:, j], :]
            for k in range(j, na):
                alpha += mat_aa[occ_a[:, j], occ_a[:, k]]
        coeff = alpha[:, None] + beta[None, :]
        for j in range(nb):
            coeff = coeff + cmap[:, occ_b[:, j]]
        return coeff
    sa = make_strings(norb, na)
    sb = make_strings(norb, nb)
    za = 1 - 2 * ((sa[:, None] >> np.arange(norb)[None, :]) & 1)
    zb = 1 - 2 * ((sb[:, None] >> np.arange(norb)[None, :]) & 1)
    beta = np.zeros(len(sb))
    alpha = np.zeros(len(sa))
    for j in range(norb):
        for k in range(j + 1, norb):
            beta += zb[:, j] * zb[:, k] * mat_bb[j, k]
            alpha += za[:, j] * za[:, k] * mat_aa[j, k]
    cmap = za.astype(float) @ mat_ab
    coeff = alpha[:, None] + beta[None, :] + cmap @ zb.T.astype(float)
    return 0.25 * coeff


def contract_diag_coulomb(vec, mat, norb, nelec, *, z_representation=False):
    """contract/diag_coulomb.py:41-192."""
    aa, ab, bb = get_mats(mat, norb, z_representation)
    vec = np.asarray(vec, dtype=complex)
    na, nb = nelec
    dim_a, dim_b = math.comb(norb, na), math.comb(norb, nb)
    coeff = diag_coulomb_coeffs(aa, ab, bb, norb, nelec, z_representation)
    return (coeff * vec.reshape((dim_a, dim_b))).reshape(-1)


def contract_num_op_sum(vec, coeffs, norb, nelec):
    """contract/num_op_sum.py:27-72 and num_op_sum.rs:20-39."""
    vec = np.asarray(vec, dtype=complex)
    na, nb = nelec
    occ_a = gen_occslst(norb, na)
    occ_b = gen_occslst(norb, nb)
    dim_a, dim_b = len(occ_a), len(occ_b)
    ca = coeffs[occ_a].sum(axis=1) if na else np.zeros(dim_a)
    cb = coeffs[occ_b].sum(axis=1) if nb else np.zeros(dim_b)
    v = vec.reshape((dim_a, dim_b))
    return ((ca[:, None] + cb[None, :]) * v).reshape(-1)


def diag_coulomb_linop_matvec(mat, norb, nelec, *, orbital_rotation=None, z_representation=False):
    """contract/diag_coulomb.py:195-272; returns the matvec closure."""

    def matvec(vec):
        if orbital_rotation is not None:
            vec = apply_orbital_rotation(vec, _conj_rotation(orbital_rotation), norb, nelec)
        vec = contract_diag_coulomb(vec, mat, norb, nelec, z_representation=z_representation)
        if orbital_rotation is not None:
            vec = apply_orbital_rotation(vec, orbital_rotation, norb, nelec, copy=False)
        return vec

    return matvec


def num_op_sum_linop_matvec(coeffs, norb, nelec, *, orbital_rotation=None):
    """contract/num_op_sum.py:75-131."""

    def matvec(vec):
        if orbital_rotation is not None:
            vec = apply_orbital_rotation(vec, orbital_rotation.T.conj(), norb, nelec)
        vec = contract_num_op_sum(vec, coeffs, norb, nelec)
        if orbital_rotation is not None:
            vec = apply_orbital_rotation(vec, orbital_rotation, norb, nelec, copy=False)
        return vec

    return matvec


def df_hamiltonian_matvec(one_body_tensor, diag_coulomb_mats, orbital_rotations, constant,
                          norb, nelec, z_representation=False):
    """double_factorized_hamiltonian.py:244-275 (matvec = rmatvec)."""
    eigs, vecs = scipy.linalg.eigh(one_body_tensor)
    num_mv = num_op_sum_linop_matvec(eigs, norb, nelec, orbital_rotation=vecs)
    dc_mvs = [
        diag_coulomb_linop_matvec(m, norb, nelec, orbital_rotation=u, z_representation=z_representation)
        for m, u in zip(diag_coulomb_mats, orbital_rotations)
    ]

    def matvec(vec):
        vec = np.asarray(vec, dtype=complex)
        result = constant * vec
        result = result + num_mv(vec)
        for mv in dc_mvs:
            result = result + mv(vec)
        return result

    return matvec


def df_energy(vec, one_body_tensor, diag_coulomb_mats, orbital_rotations, constant, norb, nelec,
              z_representation=False):
    """``np.vdot(vec, H @ vec).real`` (tests/python/variational/ucj_spin_balanced_test.py:152-158)."""
    mv = df_hamiltonian_matvec(one_body_tensor, diag_coulomb_mats, orbital_rotations, constant,
                               norb, nelec, z_representation)
    return float(np.vdot(vec, mv(vec)).real)


# ---------------------------------------------------------------------------
# One-body operators and 1-RDMs from their definition (contract/one_body.py:24-90,
# states/rdm.py:73-170; the reference's tests/python/states/rdm_test.py:147-176
# evaluate <a+_p a_q> the same way)
# ---------------------------------------------------------------------------


def _excitation_lists(norb, nocc, p, q):
    """Source and target addresses and signs of a+_p a_q on one sector's
    strings (colex addresses, Jordan-Wigner order within the sector)."""
    strings = make_strings(norb, nocc)
    addr = {int(s): i for i, s in enumerate(strings)}
    src, dst, sgn = [], [], []
    for i, s in enumerate(strings):
        s = int(s)
        if not (s >> q) & 1:
            continue
        t = s & ~(1 << q)
        if p != q and (t >> p) & 1:
            continue
        sign = (-1) ** (bin(s & ((1 << q) - 1)).count("1") + bin(t & ((1 << p) - 1)).count("1"))
        src.append(i)
        dst.append(addr[t | (1 << p)])
        sgn.append(sign)
    return np.array(src, dtype=np.int64), np.array(dst, dtype=np.int64), np.array(sgn, dtype=float)


def _apply_excitation(v2, norb, nelec, p, q, spin):
    na, nb = nelec
    out = np.zeros_like(v2)
    src, dst, sgn = _excitation_lists(norb, na if spin == 0 else nb, p, q)
    if spin == 0:
        np.add.at(out, dst, sgn[:, None] * v2[src])
    else:
        np.add.at(out.T, dst, sgn[:, None] * v2.T[src])
    return out


def spin_square(vec, norb, nelec):
    """<psi|S^2|psi> (unnormalised, python/ffsim/states/states.py:52-59) from
    S^2 = S_- S_+ + S_z (S_z + 1), with <psi|S_- S_+|psi> = |S_+ psi|^2 and
    S_+ = sum_p a+_{p alpha} a_{p beta} applied string by string into the
    (n_alpha + 1, n_beta - 1) sector.  States are a+_alpha... a+_beta... |0>,
    so a_{p beta} passes all n_alpha alpha operators and the beta ones below
    p, and a+_{p alpha} the alpha ones below p."""
    na, nb = nelec
    v2 = np.asarray(vec, dtype=complex).reshape(math.comb(norb, na), math.comb(norb, nb))
    sz = 0.5 * (na - nb)
    norm2 = float(np.vdot(v2, v2).real)
    if nb == 0 or na == norb:
        return sz * (sz + 1) * norm2
    sa, sb = make_strings(norb, na), make_strings(norb, nb)
    ta, tb = make_strings(norb, na + 1), make_strings(norb, nb - 1)
    ia = {int(x): k for k, x in enumerate(ta)}
    ib = {int(x): k for k, x in enumerate(tb)}
    out = np.zeros((len(ta), len(tb)), dtype=complex)
    for i, a in enumerate(sa):
        a = int(a)
        for j, b in enumerate(sb):
            b = int(b)
            for orb in range(norb):
                if not (b >> orb) & 1 or (a >> orb) & 1:
                    continue
                below = (1 << orb) - 1
                sign = (-1) ** (na + bin(b & below).count("1") + bin(a & below).count("1"))
                out[ia[a | (1 << orb)], ib[b & ~(1 << orb)]] += sign * v2[i, j]
    return float(np.vdot(out, out).real) + sz * (sz + 1) * norm2


def one_body_action(vec, mat, norb, nelec):
    """sum_{pq} M_pq (a+_{p alpha} a_{q alpha} + a+_{p beta} a_{q beta}) vec."""
    na, nb = nelec
    v2 = np.asarray(vec, dtype=complex).reshape(math.comb(norb, na), math.comb(norb, nb))
    out = np.zeros_like(v2)
    for p in range(norb):
        for q in range(norb):
            if mat[p, q] != 0:
                for spin in (0, 1):
                    out += mat[p, q] * _apply_excitation(v2, norb, nelec, p, q, spin)
    return out.reshape(-1)


def rdm2s(vec, norb, nelec, reorder=True):
    """[aa, ab, bb] 2-RDMs from the definition (states/rdm.py:73-120):
    reorder=True: rdm2[p, q, r, s] = <a+_p a+_r a_s a_q>; reorder=False:
    rdm2[p, q, r, s] = <a+_p a_q a+_r a_s>; first index pair on the first spin."""
    na, nb = nelec
    v2 = np.asarray(vec, dtype=complex).reshape(math.comb(norb, na), math.comb(norb, nb))
    out = np.zeros((3, norb, norb, norb, norb), dtype=complex)
    for blk, (t, sg) in enumerate([(0, 0), (0, 1), (1, 1)]):
        for r in range(norb):
            for s in range(norb):
                phi = _apply_excitation(v2, norb, nelec, r, s, sg)
                for p in range(norb):
                    for q in range(norb):
                        val = np.vdot(v2, _apply_excitation(phi, norb, nelec, p, q, t))
                        if reorder and t == sg and q == r:
                            val -= np.vdot(v2, _apply_excitation(v2, norb, nelec, p, s, t))
                        out[blk, p, q, r, s] = val
    return out


def molecular_hamiltonian_action(vec, one_body_tensor, two_body_tensor, constant, norb, nelec):
    """H vec for H = sum h_pq E_pq + 1/2 sum h_pqrs a+_ps a+_rt a_st a_qs + constant
    (hamiltonians/molecular_hamiltonian.py:24-60) from the definition, with
    a+_ps a+_rt a_st a_qs = E^s_pq E^t_rs - delta_qr delta_st E^s_ps."""
    na, nb = nelec
    v2 = np.asarray(vec, dtype=complex).reshape(math.comb(norb, na), math.comb(norb, nb))

    def e(x, p, q):
        return _apply_excitation(x, norb, nelec, p, q, 0) + _apply_excitation(x, norb, nelec, p, q, 1)

    out = constant * v2
    for p in range(norb):
        for q in range(norb):
            coef = one_body_tensor[p, q] - 0.5 * sum(two_body_tensor[p, r, r, q] for r in range(norb))
            if coef != 0:
                out = out + coef * e(v2, p, q)
    for r in range(norb):
        for s in range(norb):
            phi = e(v2, r, s)
            for p in range(norb):
                for q in range(norb):
                    if two_body_tensor[p, q, r, s] != 0:
                        out = out + 0.5 * two_body_tensor[p, q, r, s] * e(phi, p, q)
    return out.reshape(-1)


def random_two_body_tensor(norb, *, seed=None):
    """sum_k M_k (x) M_k over norb**2 random Hermitian M_k (random/random.py:211-237):
    the symmetries of molecular integrals, h_pqrs = h_rspq = conj(h_qpsr)."""
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((norb * norb, norb, norb)) + 1j * rng.standard_normal((norb * norb, norb, norb))
    m = m + m.transpose(0, 2, 1).conj()
    return np.tensordot(m, m, axes=(0, 0))


def rdm1s(vec, norb, nelec):
    """[alpha, beta] 1-RDMs, rdm[p, q] = <vec| a+_p a_q |vec>."""
    na, nb = nelec
    v2 = np.asarray(vec, dtype=complex).reshape(math.comb(norb, na), math.comb(norb, nb))
    out = np.zeros((2, norb, norb), dtype=complex)
    for spin in (0, 1):
        for p in range(norb):
            for q in range(norb):
                out[spin, p, q] = np.vdot(v2, _apply_excitation(v2, norb, nelec, p, q, spin))
    return out


# ---------------------------------------------------------------------------
# Trotter-Suzuki evolution of a double-factorized Hamiltonian
# (trotter/double_factorized.py:25-127, trotter/_util.py:18-60)
# ---------------------------------------------------------------------------


def trotter_step_terms(n_terms, time, order=0):
    """(term index, time) sequence of one Trotter step (trotter/_util.py:18-60):
    order 0 is the plain product; order k >= 1 is Suzuki's symmetric fractal
    (J. Math. Phys. 32, 400 (1991)): order 1 sweeps the terms at half time up
    to the last one at full time and back, and order k nests five order-(k-1)
    steps with times p, p, 1 - 4p, p, p, p = 1 / (4 - 4^(1/(2k-1)))."""
    if order == 0:
        return [(i, time) for i in range(n_terms)]
    if order == 1:
        seq = [(i, time / 2) for i in range(n_terms - 1)] + [(n_terms - 1, time)]
        return seq + [(i, time / 2) for i in reversed(range(n_terms - 1))]
    p = time / (4 - 4 ** (1 / (2 * order - 1)))
    inner = trotter_step_terms(n_terms, p, order - 1)
    return inner * 2 + trotter_step_terms(n_terms, time - 4 * p, order - 1) + inner * 2


def simulate_trotter_double_factorized(vec, one_body_tensor, diag_coulomb_mats, orbital_rotations, constant,
                                       time, norb, nelec, n_steps=1, order=0, z_representation=False):
    """double_factorized.py:25-127: term 0 (one-body) multiplies the running
    orbital basis by exp(-i t h); term k >= 1 rotates the state into
    U_k's basis and applies exp(-i t J_k n n); the last basis and the global
    phase exp(-i T constant) close the evolution."""
    if order < 0 or n_steps < 0:
        raise ValueError("order and n_steps must be non-negative")
    vec = np.array(vec, dtype=complex, copy=True)
    if n_steps == 0:
        return vec
    step = time / n_steps
    basis = np.eye(norb, dtype=complex)
    for _ in range(n_steps):
        for k, t in trotter_step_terms(1 + len(diag_coulomb_mats), step, order):
            if k == 0:
                basis = scipy.linalg.expm(-1j * t * one_body_tensor) @ basis
            else:
                u = orbital_rotations[k - 1]
                vec = apply_orbital_rotation(vec, u.T.conj() @ basis, norb, nelec, copy=False)
                vec = apply_diag_coulomb_evolution(vec, diag_coulomb_mats[k - 1], t, norb, nelec,
                                                   z_representation=z_representation, copy=False)
                basis = u
    vec = apply_orbital_rotation(vec, basis, norb, nelec, copy=False)
    if constant:
        vec = vec * np.exp(-1j * time * constant)
    return vec


# ---------------------------------------------------------------------------
# Diagonal Coulomb Hamiltonian (hamiltonians/diagonal_coulomb_hamiltonian.py:27-252)
# and its split-operator Trotter evolution (trotter/diagonal_coulomb_split_op.py:25-122)
# ---------------------------------------------------------------------------


def diag_coulomb_hamiltonian_action(vec, one_body_tensor, diag_coulomb_mats, constant, norb, nelec):
    """H |vec> for H = sum h_pq a+_ps a_qs + 1/2 sum J^{st}_pq n_ps n_qt + constant,
    J^{aa} = J^{bb} = mats[0], J^{ab} = J^{ba} = mats[1]
    (diagonal_coulomb_hamiltonian.py:67-97): the one-body part in the
    eigenbasis of h, the Coulomb part diagonal in the occupation basis."""
    vec = np.asarray(vec, dtype=complex)
    eigs, vecs = scipy.linalg.eigh(one_body_tensor)
    aa, ab = diag_coulomb_mats
    out = constant * vec
    out = out + num_op_sum_linop_matvec(eigs, norb, nelec, orbital_rotation=vecs)(vec)
    return out + contract_diag_coulomb(vec, (aa, ab, aa), norb, nelec)


def diag_coulomb_hamiltonian_diag(one_body_tensor, diag_coulomb_mats, constant, norb, nelec):
    """Diagonal of H in the occupation basis (diagonal_coulomb_hamiltonian.py:208-238):
    the one-body diagonal summed over occupied orbitals plus the Coulomb
    energy of each (alpha, beta) pair of strings."""
    na, nb = nelec
    occ_a = np.zeros((math.comb(norb, na), norb))
    occ_b = np.zeros((math.comb(norb, nb), norb))
    for k, occ in enumerate(gen_occslst(norb, na)):
        occ_a[k, occ] = 1.0
    for k, occ in enumerate(gen_occslst(norb, nb)):
        occ_b[k, occ] = 1.0
    aa, ab = (np.asarray(m, dtype=float) for m in diag_coulomb_mats)
    h = np.diag(one_body_tensor).real
    ea = occ_a @ h + 0.5 * np.einsum("ip,pq,iq->i", occ_a, aa, occ_a)
    eb = occ_b @ h + 0.5 * np.einsum("ip,pq,iq->i", occ_b, aa, occ_b)
    return (ea[:, None] + eb[None, :] + occ_a @ ab @ occ_b.T + constant).reshape(-1)


def simulate_trotter_diag_coulomb_split_op(vec, one_body_tensor, diag_coulomb_mats, constant, time,
                                           norb, nelec, n_steps=1, order=0):
    """diagonal_coulomb_split_op.py:25-122: a two-term step sequence; term 0
    multiplies the running basis by exp(-i t h), term 1 rotates the state by
    the running basis, applies exp(-i t J n n) with (J_aa, J_ab, J_aa) and
    resets the basis to the identity."""
    if order < 0 or n_steps < 0:
        raise ValueError("order and n_steps must be non-negative")
    vec = np.array(vec, dtype=complex, copy=True)
    if n_steps == 0:
        return vec
    aa, ab = diag_coulomb_mats
    step = time / n_steps
    basis = np.eye(norb, dtype=complex)
    for _ in range(n_steps):
        for k, t in trotter_step_terms(2, step, order):
            if k == 0:
                basis = scipy.linalg.expm(-1j * t * one_body_tensor) @ basis
            else:
                vec = apply_orbital_rotation(vec, basis, norb, nelec, copy=False)
                vec = apply_diag_coulomb_evolution(vec, (aa, ab, aa), t, norb, nelec, copy=False)
                basis = np.eye(norb, dtype=complex)
    vec = apply_orbital_rotation(vec, basis, norb, nelec, copy=False)
    if constant:
        vec = vec * np.exp(-1j * time * constant)
    return vec


# ---------------------------------------------------------------------------
# UCJ (variational/ucj_spin_balanced.py:657-696) and parameter maps
# ---------------------------------------------------------------------------


def ucj_spin_balanced_apply(vec, diag_coulomb_mats, orbital_rotations, final_orbital_rotation,
                            norb, nelec, copy=True):
    """ucj_spin_balanced.py:657-696."""
    vec = np.array(vec, dtype=complex, copy=True) if copy else np.asarray(vec, dtype=complex)
    current = np.eye(norb)
    for (jaa, jab), u in zip(diag_coulomb_mats, orbital_rotations):
        vec = apply_orbital_rotation(vec, u.T.conj() @ current, norb, nelec, copy=False)
        vec = apply_diag_coulomb_evolution(vec, (jaa, jab, jaa), -1.0, norb, nelec, copy=False)
        current = u
    if final_orbital_rotation is None:
        vec = apply_orbital_rotation(vec, current, norb, nelec, copy=False)
    else:
        vec = apply_orbital_rotation(vec, final_orbital_rotation @ current, norb, nelec, copy=False)
    return vec


def ucj_spin_unbalanced_apply(vec, diag_coulomb_mats, orbital_rotations, final_orbital_rotation, norb, nelec):
    """ucj_spin_unbalanced.py:705-745: per rep the (alpha, beta) rotations
    U_k^dag U_{k-1} and exp(+i J_k) with [aa, ab, bb], then the final rotation."""
    vec = np.array(vec, dtype=complex, copy=True)
    basis = [np.eye(norb), np.eye(norb)]
    for mats, rot in zip(diag_coulomb_mats, orbital_rotations):
        vec = apply_orbital_rotation(vec, (rot[0].T.conj() @ basis[0], rot[1].T.conj() @ basis[1]), norb, nelec,
                                     copy=False)
        vec = apply_diag_coulomb_evolution(vec, (mats[0], mats[1], mats[2]), -1.0, norb, nelec, copy=False)
        basis = [rot[0], rot[1]]
    if final_orbital_rotation is not None:
        basis = [final_orbital_rotation[0] @ basis[0], final_orbital_rotation[1] @ basis[1]]
    return apply_orbital_rotation(vec, tuple(basis), norb, nelec, copy=False)


def ucj_spinless_apply(vec, diag_coulomb_mats, orbital_rotations, final_orbital_rotation, norb, nelec):
    """ucj_spinless.py:456-515: one rotation and one matrix per rep; on spinful
    states the matrix acts within each spin, (J, 0, J)."""
    vec = np.array(vec, dtype=complex, copy=True)
    basis = np.eye(norb)
    zero = np.zeros((norb, norb))
    for mat, rot in zip(diag_coulomb_mats, orbital_rotations):
        vec = apply_orbital_rotation(vec, rot.T.conj() @ basis, norb, nelec, copy=False)
        m = mat if isinstance(nelec, int) else (mat, zero, mat)
        vec = apply_diag_coulomb_evolution(vec, m, -1.0, norb, nelec, copy=False)
        basis = rot
    if final_orbital_rotation is not None:
        basis = final_orbital_rotation @ basis
    return apply_orbital_rotation(vec, basis, norb, nelec, copy=False)


def antihermitians_from_parameters(params, dim_, n_mats):
    """linalg/util.py:93-124 (complex case)."""
    per = dim_**2
    params = np.asarray(params, float).reshape(n_mats, per)
    mats = np.zeros((n_mats, dim_, dim_), dtype=complex)
    n_triu = dim_ * (dim_ - 1) // 2
    rows, cols = np.triu_indices(dim_)
    vals = 1j * params[:, n_triu:]
    mats[:, rows, cols] = vals
    mats[:, cols, rows] = vals
    vals = params[:, :n_triu]
    rows, cols = np.triu_indices(dim_, k=1)
    mats[:, rows, cols] += vals
    mats[:, cols, rows] -= vals
    return mats


def unitary_from_parameters(params, dim_):
    """linalg/util.py:189-232."""
    return scipy.linalg.expm(antihermitians_from_parameters(params, dim_, 1)[0])


def ucj_from_parameters(params, norb, n_reps, with_final_orbital_rotation=False):
    """ucj_spin_balanced.py:197-293 without interaction pairs."""
    triu = list(itertools.combinations_with_replacement(range(norb), 2))
    dcm = np.zeros((n_reps, 2, norb, norb))
    rots = np.zeros((n_reps, norb, norb), dtype=complex)
    index = 0
    for r in range(n_reps):
        rots[r] = unitary_from_parameters(params[index : index + norb**2], norb)
        index += norb**2
        for t in range(2):
            rows, cols = zip(*triu)
            vals = params[index : index + len(triu)]
            dcm[r, t][cols, rows] = vals
            dcm[r, t][rows, cols] = vals
            index += len(triu)
    final = None
    if with_final_orbital_rotation:
        final = unitary_from_parameters(params[index:], norb)
    return dcm, rots, final


def hartree_fock_state(norb, nelec):
    """states/slater.py:122-138: one-hot at address 0."""
    v = np.zeros(dim(norb, nelec), dtype=complex)
    v[0] = 1
    return v


# ---------------------------------------------------------------------------
# random inputs (random/random.py) -- same draws for the same seed
# ---------------------------------------------------------------------------


def random_state_vector(dim_, *, seed=None):
    """random.py:24-47."""
    rng = np.random.default_rng(seed)
    vec = rng.standard_normal(dim_).astype(complex)
    vec += 1j * rng.standard_normal(dim_)
    vec /= np.linalg.norm(vec)
    return vec


def random_unitary(dim_, *, seed=None):
    """random.py:84-106."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((dim_, dim_)).astype(complex)
    z += 1j * rng.standard_normal((dim_, dim_))
    q, r = np.linalg.qr(z)
    d = np.diagonal(r)
    return q * (d / np.abs(d))


def random_symmetric_normal(dim_, *, mean=0.0, scale=1.0, seed=None):
    """random.py:549-560."""
    rng = np.random.default_rng(seed)
    vals = rng.normal(loc=mean, scale=scale, size=dim_ * (dim_ + 1) // 2)
    mat = np.zeros((dim_, dim_))
    rows, cols = np.triu_indices(dim_)
    mat[rows, cols] = vals
    mat[cols, rows] = vals
    return mat


# ---------------------------------------------------------------------------
# independent cross-checks (not from the reference; used to pin the above)
# ---------------------------------------------------------------------------


def slater_rotation_amplitudes(mat, norb, nocc, src_occ):
    """<I| W(U) |J> = det U[occ(I), occ(J)] for one spin sector."""
    strings = make_strings(norb, nocc)
    out = np.zeros(len(strings), dtype=complex)
    for a, s in enumerate(strings):
        occ = [i for i in range(norb) if (int(s) >> i) & 1]
        out[a] = np.linalg.det(mat[np.ix_(occ, list(src_occ))]) if nocc else 1.0
    return out
