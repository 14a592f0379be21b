"""Two-orbital fermionic gates, the GPU counterparts of
python/ffsim/gates/basic_gates.py and python/ffsim/gates/quad_ham.py.

Each gate is the reference's composition over this library's entry points:
Givens, FSWAP and quadratic-Hamiltonian gates are orbital rotations by an
explicit matrix (``ffgb_apply_orbital_rotation``); a number interaction is a
number-operator-sum evolution with one coefficient; a product of two number
operators is a diagonal Coulomb evolution with one matrix entry
(``ffgb_apply_diag_coulomb_evolution``: exp(-i t sum J n n / 2) with t = -1);
larger products of number operators multiply the projector onto their
configurations, built from n_p = a+_p a_p excitations (``ffgb_apply_excitation``).
"""

from __future__ import annotations

import cmath
import math
from enum import Flag, auto

import numpy as np
import scipy.linalg
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import prepare, split_nelec, stream_ptr
from ffsim_gb300.gates import apply_diag_coulomb_evolution, apply_num_op_sum_evolution, apply_orbital_rotation


class Spin(Flag):
    """Spin sector(s) a gate acts on (python/ffsim/states/spin.py:19-31)."""

    ALPHA = auto()
    BETA = auto()
    ALPHA_AND_BETA = ALPHA | BETA


def pair_for_spin(obj, spin: Spin):
    """(obj, obj), (obj, None) or (None, obj) for both spins, alpha or beta
    (python/ffsim/states/spin.py:35-46)."""
    if spin is Spin.ALPHA:
        return obj, None
    if spin is Spin.BETA:
        return None, obj
    return obj, obj


def _distinct(target_orbs, what: str) -> None:
    if len(set(target_orbs)) == 1:
        raise ValueError(f"The orbitals to {what} must be distinct. Got {target_orbs}.")


def _two_orbital_matrix(norb: int, target_orbs, block) -> np.ndarray:
    mat = np.eye(norb, dtype=complex)
    mat[np.ix_(target_orbs, target_orbs)] = block
    return mat


def apply_givens_rotation(vec, theta: float, target_orbs: tuple[int, int], norb: int, nelec,
                          spin: Spin = Spin.ALPHA_AND_BETA, *, phi: float = 0.0, copy: bool = True):
    r"""G(theta, phi) on orbitals (p, q): the orbital rotation that is the
    identity except for [[c, s], [-conj(s), c]] on (p, q), c = cos theta,
    s = e^{i phi} sin theta (basic_gates.py:54-123)."""
    _distinct(target_orbs, "rotate")
    c = math.cos(theta)
    s = cmath.exp(1j * phi) * math.sin(theta)
    mat = _two_orbital_matrix(norb, target_orbs, [[c, s], [-s.conjugate(), c]])
    if isinstance(nelec, (int, np.integer)):
        return apply_orbital_rotation(vec, mat, norb, nelec, copy=copy)
    return apply_orbital_rotation(vec, pair_for_spin(mat, spin), norb, nelec, copy=copy)


def apply_num_interaction(vec, theta: float, target_orb: int, norb: int, nelec,
                          spin: Spin = Spin.ALPHA_AND_BETA, *, copy: bool = True):
    r"""exp(i theta n_p) in the selected sectors (basic_gates.py:195-246)."""
    coeffs = np.zeros(norb)
    coeffs[target_orb] = 1.0
    if isinstance(nelec, (int, np.integer)):
        return apply_num_op_sum_evolution(vec, coeffs, -theta, norb, nelec, copy=copy)
    return apply_num_op_sum_evolution(vec, pair_for_spin(coeffs, spin), -theta, norb, nelec, copy=copy)


def apply_tunneling_interaction(vec, theta: float, target_orbs: tuple[int, int], norb: int, nelec,
                                spin: Spin = Spin.ALPHA_AND_BETA, *, copy: bool = True):
    r"""A Givens rotation conjugated by exp(-/+ i pi/2 n_p) (basic_gates.py:126-192)."""
    _distinct(target_orbs, "rotate")
    vec = apply_num_interaction(vec, -math.pi / 2, target_orbs[0], norb, nelec, spin, copy=copy)
    vec = apply_givens_rotation(vec, theta, target_orbs, norb, nelec, spin, copy=False)
    return apply_num_interaction(vec, math.pi / 2, target_orbs[0], norb, nelec, spin, copy=False)


def _pair_matrix(norb: int, p: int, q: int, theta: float) -> np.ndarray:
    mat = np.zeros((norb, norb))
    mat[p, q] += theta
    mat[q, p] += theta
    return mat


def apply_num_num_interaction(vec, theta: float, target_orbs: tuple[int, int], norb: int, nelec,
                              spin: Spin = Spin.ALPHA_AND_BETA, *, copy: bool = True):
    r"""exp(i theta n_p n_q) in each selected sector (basic_gates.py:249-325):
    one diagonal Coulomb evolution with J_pq = J_qp = theta in the selected
    same-spin matrices and time -1."""
    _distinct(target_orbs, "interact")
    p, q = target_orbs
    mat = _pair_matrix(norb, p, q, theta)
    if isinstance(nelec, (int, np.integer)):
        return apply_diag_coulomb_evolution(vec, mat, -1.0, norb, nelec, copy=copy)
    aa = mat if spin & Spin.ALPHA else None
    bb = mat if spin & Spin.BETA else None
    return apply_diag_coulomb_evolution(vec, (aa, None, bb), -1.0, norb, nelec, copy=copy)


def apply_on_site_interaction(vec, theta: float, target_orb: int, norb: int, nelec: tuple[int, int], *,
                              copy: bool = True):
    r"""exp(i theta n_{p alpha} n_{p beta}) (basic_gates.py:328-372): the
    alpha-beta matrix with J_pp = theta, time -1."""
    ab = np.zeros((norb, norb))
    ab[target_orb, target_orb] = theta
    return apply_diag_coulomb_evolution(vec, (None, ab, None), -1.0, norb, nelec, copy=copy)


def _project_occupied(t: torch.Tensor, alpha_orbs, beta_orbs, norb: int, nelec) -> torch.Tensor:
    """prod n_{p alpha} prod n_{q beta} t, one n_p = a+_p a_p excitation per orbital."""
    n_alpha, n_beta = split_nelec(nelec)
    code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
    cur = t
    for spin, orbs in ((0, alpha_orbs), (1, beta_orbs)):
        for orb in orbs:
            out = torch.empty_like(t)
            _lib.call("ffgb_apply_excitation", cur.data_ptr(), out.data_ptr(), code, norb, n_alpha, n_beta, spin,
                      int(orb), int(orb), stream_ptr(t))
            cur = out
    return cur


def apply_num_op_prod_interaction(vec, theta: float, target_orbs, norb: int, nelec: tuple[int, int], *,
                                  copy: bool = True):
    r"""exp(i theta prod_{p in S_a} n_{p alpha} prod_{q in S_b} n_{q beta})
    (basic_gates.py:375-424): configurations with every target occupied pick
    up e^{i theta}.  Up to two number operators this is one diagonal Coulomb
    (or number-operator-sum) evolution; more use the projector P onto those
    configurations, vec + (e^{i theta} - 1) P vec."""
    alpha, beta = (sorted(set(int(x) for x in orbs)) for orbs in target_orbs)
    if not alpha and not beta:
        p = prepare(vec, norb, nelec, copy=copy)
        p.tensor.mul_(cmath.exp(1j * theta))
        return p.finish()
    if len(alpha) + len(beta) == 1:
        orb, spin = (alpha[0], Spin.ALPHA) if alpha else (beta[0], Spin.BETA)
        return apply_num_interaction(vec, theta, orb, norb, nelec, spin, copy=copy)
    if len(alpha) == 2 and not beta:
        return apply_diag_coulomb_evolution(vec, (_pair_matrix(norb, *alpha, theta), None, None), -1.0, norb, nelec,
                                            copy=copy)
    if len(beta) == 2 and not alpha:
        return apply_diag_coulomb_evolution(vec, (None, None, _pair_matrix(norb, *beta, theta)), -1.0, norb, nelec,
                                            copy=copy)
    if len(alpha) == 1 and len(beta) == 1:
        ab = np.zeros((norb, norb))
        ab[alpha[0], beta[0]] = theta
        return apply_diag_coulomb_evolution(vec, (None, ab, None), -1.0, norb, nelec, copy=copy)
    p = prepare(vec, norb, nelec, copy=copy)
    proj = _project_occupied(p.tensor.reshape(-1), alpha, beta, norb, nelec)
    p.tensor.reshape(-1).add_(proj, alpha=cmath.exp(1j * theta) - 1)
    return p.finish()


def apply_hop_gate(vec, theta: float, target_orbs: tuple[int, int], norb: int, nelec,
                   spin: Spin = Spin.ALPHA_AND_BETA, *, copy: bool = True):
    r"""A Givens rotation followed by exp(i pi n_p n_q) (basic_gates.py:427-497)."""
    vec = apply_givens_rotation(vec, theta, target_orbs, norb, nelec, spin, copy=copy)
    return apply_num_num_interaction(vec, math.pi, target_orbs, norb, nelec, spin, copy=False)


def apply_fsim_gate(vec, theta: float, phi: float, target_orbs: tuple[int, int], norb: int, nelec,
                    spin: Spin = Spin.ALPHA_AND_BETA, *, copy: bool = True):
    r"""A tunneling interaction by -theta followed by exp(-i phi n_p n_q)
    (basic_gates.py:500-572)."""
    vec = apply_tunneling_interaction(vec, -theta, target_orbs, norb, nelec, spin, copy=copy)
    return apply_num_num_interaction(vec, -phi, target_orbs, norb, nelec, spin, copy=False)


def apply_fswap_gate(vec, target_orbs: tuple[int, int], norb: int, nelec, spin: Spin = Spin.ALPHA_AND_BETA, *,
                     copy: bool = True):
    r"""The orbital rotation that swaps orbitals p and q (basic_gates.py:575-629)."""
    mat = _two_orbital_matrix(norb, target_orbs, [[0, 1], [1, 0]])
    if isinstance(nelec, (int, np.integer)):
        return apply_orbital_rotation(vec, mat, norb, nelec, copy=copy)
    return apply_orbital_rotation(vec, pair_for_spin(mat, spin), norb, nelec, copy=copy)


def apply_quad_ham_evolution(vec, mat, time: float, norb: int, nelec, *, copy: bool = True):
    r"""exp(-i t sum M_pq a+_p a_q): the orbital rotation exp(-i t M), one matrix
    for both sectors or one per sector, ``None`` for none
    (python/ffsim/gates/quad_ham.py:43-108)."""
    if isinstance(nelec, (int, np.integer)) or (isinstance(mat, np.ndarray) and mat.ndim == 2):
        return apply_orbital_rotation(vec, scipy.linalg.expm(-1j * time * np.asarray(mat)), norb, nelec, copy=copy)
    mat_a, mat_b = mat
    rot_a = None if mat_a is None else scipy.linalg.expm(-1j * time * np.asarray(mat_a))
    rot_b = None if mat_b is None else scipy.linalg.expm(-1j * time * np.asarray(mat_b))
    return apply_orbital_rotation(vec, (rot_a, rot_b), norb, nelec, copy=copy)
