"""State helpers: dimensions, string tables (host), Hartree-Fock state, inner products."""

from __future__ import annotations

import itertools
import math
from functools import lru_cache

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import dim, dims, prepare, split_nelec, stream_ptr

__all__ = ["dim", "dims", "make_strings", "init_cache", "hartree_fock_state", "vdot",
           "slater_determinant", "slater_determinant_rdms", "slater_determinant_amplitudes", "spin_square",
           "spinful_to_spinless_vec", "spinful_to_spinless_rdm1", "spinful_to_spinless_rdm2"]


@lru_cache(maxsize=None)
def make_strings(norb: int, nocc: int) -> np.ndarray:
    """Occupation bitstrings in address order (ascending integers with ``nocc``
    set bits); the string order of python/ffsim/_cistring.py:21-24."""
    if nocc < 0 or nocc > norb:
        return np.zeros(0, dtype=np.int64)
    out = np.fromiter(
        (sum(1 << i for i in c) for c in itertools.combinations(range(norb), nocc)),
        dtype=np.int64, count=math.comb(norb, nocc))
    out.sort()
    return out


def init_cache(norb: int, nelec: tuple[int, int]) -> None:
    """Build the host string tables of both sectors ahead of timing
    (python/ffsim/init_cache.py:25-41).  The kernels rank strings in registers
    and the library builds its device tables on first use, so only the host
    tables used by the bitstring and Slater-determinant helpers are made here."""
    for nocc in nelec:
        make_strings(norb, int(nocc))


def hartree_fock_state(norb: int, nelec, *, dtype=torch.complex128, device="cuda") -> torch.Tensor:
    """The Hartree-Fock state: one-hot at address 0 (python/ffsim/states/slater.py:122-138)."""
    n = dim(norb, nelec)
    t = torch.empty(n, dtype=dtype, device=device)
    code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
    _lib.call("ffgb_hartree_fock", t.data_ptr(), code, n, stream_ptr(t))
    return t


def vdot(x: torch.Tensor, y: torch.Tensor) -> complex:
    """sum conj(x) y accumulated in FP64 on the device."""
    if x.dtype != y.dtype or x.numel() != y.numel():
        raise ValueError("vdot needs two vectors of the same dtype and size")
    if not (x.is_cuda and y.is_cuda) or x.dtype not in (torch.complex64, torch.complex128):
        raise ValueError("vdot needs complex CUDA tensors")
    x = x.contiguous()
    y = y.contiguous()
    out = np.zeros(2)
    code = _lib.FFGB_C64 if x.dtype == torch.complex64 else _lib.FFGB_C128
    _lib.call("ffgb_vdot", x.data_ptr(), y.data_ptr(), code, x.numel(), _lib.dptr(out), stream_ptr(x))
    return complex(out[0], out[1])



def _spinless(occupied_orbitals) -> bool:
    return not occupied_orbitals or isinstance(occupied_orbitals[0], (int, np.integer))


def _permutation_parity(orbitals) -> int:
    """+1 or -1: the sign of sorting ``orbitals`` (the number of inversions)."""
    orbs = list(orbitals)
    inv = sum(1 for i in range(len(orbs)) for j in range(i + 1, len(orbs)) if orbs[i] > orbs[j])
    return -1 if inv % 2 else 1


def _address(norb: int, orbitals) -> int:
    bits = sum(1 << int(i) for i in orbitals)
    return int(np.searchsorted(make_strings(norb, len(orbitals)), bits))


def slater_determinant(norb: int, occupied_orbitals, orbital_rotation=None, *, dtype=torch.complex128,
                       device="cuda") -> torch.Tensor:
    r""":math:`\mathcal{U} |x\rangle` for the configuration x of
    ``occupied_orbitals`` (a list, spinless, or an (alpha, beta) pair of lists),
    as a device tensor (python/ffsim/states/slater.py:32-103).  The one-hot
    vector is signed by the parity of the listed orbital order and rotated by
    ``orbital_rotation`` (one matrix, or a pair with ``None`` entries) on the GPU."""
    from ffsim_gb300.gates import apply_orbital_rotation

    if norb == 0:
        return torch.ones(1, dtype=dtype, device=device)
    if _spinless(occupied_orbitals):
        orbs = list(occupied_orbitals)
        nelec = len(orbs)
        index = _address(norb, orbs)
        sign = _permutation_parity(orbs)
    else:
        alpha, beta = (list(x) for x in occupied_orbitals)
        nelec = (len(alpha), len(beta))
        index = _address(norb, alpha) * math.comb(norb, len(beta)) + _address(norb, beta)
        sign = _permutation_parity(alpha) * _permutation_parity(beta)
    vec = torch.zeros(dim(norb, nelec), dtype=dtype, device=device)
    vec[index] = sign
    if orbital_rotation is not None:
        vec = apply_orbital_rotation(vec, orbital_rotation, norb, nelec, copy=False)
    return vec


def _rdm1_rotated(norb, orbitals, rot):
    rdm = np.zeros((norb, norb))
    if orbitals:
        rdm[orbitals, orbitals] = 1
    if rot is not None:
        rot = np.asarray(rot)
        rdm = rot.conj() @ rdm @ rot.T
    return rdm


def _rdm2_same(rdm, reorder, norb):
    out = np.einsum("pq,rs->pqrs", rdm, rdm) - np.einsum("ps,rq->pqrs", rdm, rdm)
    if not reorder:
        out = out + np.einsum("ps,qr->pqrs", rdm, np.eye(norb))
    return out


def slater_determinant_rdms(norb: int, occupied_orbitals, orbital_rotation=None, *, rank: int = 1,
                            reorder: bool = True):
    """Closed-form 1- and 2-RDMs of a Slater determinant (python/ffsim/states/slater.py:141-300):
    rdm1 = conj(U) P U^T with P the occupied projector; rdm2 from Wick's
    theorem (direct minus exchange, plus rdm1 (x) 1 when ``reorder`` is
    False).  Spinful results are stacked (a, b) and (aa, ab, bb)."""
    if rank not in (1, 2):
        raise NotImplementedError(f"Returning the rank {rank} reduced density matrix is currently not supported.")
    if _spinless(occupied_orbitals):
        rdm1 = _rdm1_rotated(norb, list(occupied_orbitals), orbital_rotation)
        return rdm1 if rank == 1 else (rdm1, _rdm2_same(rdm1, reorder, norb))
    if isinstance(orbital_rotation, np.ndarray) and orbital_rotation.ndim == 2:
        rot_a = rot_b = orbital_rotation
    else:
        rot_a, rot_b = orbital_rotation if orbital_rotation is not None else (None, None)
    alpha, beta = (list(x) for x in occupied_orbitals)
    rdm_a = _rdm1_rotated(norb, alpha, rot_a)
    rdm_b = _rdm1_rotated(norb, beta, rot_b)
    rdm1 = np.stack([rdm_a, rdm_b])
    if rank == 1:
        return rdm1
    rdm2 = np.stack([_rdm2_same(rdm_a, reorder, norb), np.einsum("pq,rs->pqrs", rdm_a, rdm_b),
                     _rdm2_same(rdm_b, reorder, norb)])
    return rdm1, rdm2


def slater_determinant_amplitudes(bitstrings, norb: int, occupied_orbitals, orbital_rotation) -> np.ndarray:
    """Amplitudes of given bitstrings in a Slater determinant: determinants of
    the rotation's occupied columns restricted to the bitstring's rows
    (python/ffsim/states/slater.py:303-350); spinful amplitudes are the
    products of the two sectors'."""
    import scipy.linalg

    def sector(strings, orbs, rot):
        cols = np.asarray(rot)[:, list(orbs)]
        return np.array([scipy.linalg.det(cols[[i for i in range(norb) if (int(b) >> i) & 1]]) for b in strings])

    if _spinless(occupied_orbitals):
        return sector(bitstrings, occupied_orbitals, orbital_rotation)
    strings_a, strings_b = bitstrings
    orbs_a, orbs_b = occupied_orbitals
    if isinstance(orbital_rotation, np.ndarray) and orbital_rotation.ndim == 2:
        rot_a = rot_b = orbital_rotation
    else:
        rot_a, rot_b = orbital_rotation
    return sector(strings_a, orbs_a, rot_a) * sector(strings_b, orbs_b, rot_b)


def spin_square(fcivec, norb: int, nelec: tuple[int, int]) -> float:
    r""":math:`\langle\psi|S^2|\psi\rangle` of an unnormalised state
    (python/ffsim/states/states.py:52-59).

    :math:`S^2 = S_- S_+ + S_z(S_z + 1)` and :math:`S_- S_+ = N_\beta - \sum_{pq}
    E^\alpha_{qp} E^\beta_{pq}`, so :math:`\langle S^2\rangle = (S_z(S_z+1) + N_\beta)
    \langle\psi|\psi\rangle - \sum_{pq} \langle E^\alpha_{pq}\psi | E^\beta_{pq}\psi\rangle`:
    per orbital pair two single-excitation launches (``ffgb_apply_excitation``)
    and one FP64 inner product (``ffgb_vdot``) on the device."""
    n_alpha, n_beta = split_nelec(nelec)
    if n_beta < 0:
        raise ValueError("spin_square needs the electron numbers of both spin sectors")
    p = prepare(fcivec, norb, (n_alpha, n_beta), copy=False)
    t = p.tensor.reshape(-1)
    code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
    xa, xb = torch.empty_like(t), torch.empty_like(t)
    cross = 0.0
    if n_alpha and n_beta:
        for orb_p in range(norb):
            for orb_q in range(norb):
                for spin, x in ((0, xa), (1, xb)):
                    _lib.call("ffgb_apply_excitation", t.data_ptr(), x.data_ptr(), code, norb, n_alpha, n_beta,
                              spin, orb_p, orb_q, stream_ptr(t))
                cross += vdot(xa, xb).real
    sz = 0.5 * (n_alpha - n_beta)
    return (sz * (sz + 1) + n_beta) * vdot(t, t).real - cross


def spinful_to_spinless_vec(vec, norb: int, nelec: tuple[int, int]):
    """The same state on 2 norb spinless orbitals, alpha orbitals first
    (python/ffsim/states/states.py): the amplitude of (alpha string a, beta
    string b) moves to the spinless string (b << norb) | a.  numpy in, numpy
    out; a torch tensor stays on its device."""
    from ffsim_gb300.bitstring import addresses_to_strings, strings_to_addresses

    n_old = dim(norb, nelec)
    strings = addresses_to_strings(range(n_old), norb, nelec)
    addrs = strings_to_addresses(strings, 2 * norb, sum(nelec))
    n_new = dim(2 * norb, sum(nelec))
    if isinstance(vec, torch.Tensor):
        out = torch.zeros(n_new, dtype=vec.dtype, device=vec.device)
        out[torch.from_numpy(addrs).to(vec.device)] = vec.reshape(-1)
        return out
    vec = np.asarray(vec)
    out = np.zeros(n_new, dtype=vec.dtype)
    out[addrs] = vec.reshape(-1)
    return out


def spinful_to_spinless_rdm1(mat_a: np.ndarray, mat_b: np.ndarray) -> np.ndarray:
    """The spinless 1-RDM: the two spin blocks on the diagonal (states/states.py)."""
    n = mat_a.shape[0]
    out = np.zeros((2 * n, 2 * n), dtype=np.result_type(mat_a, mat_b))
    out[:n, :n], out[n:, n:] = mat_a, mat_b
    return out


def spinful_to_spinless_rdm2(mat_aa: np.ndarray, mat_ab: np.ndarray, mat_bb: np.ndarray) -> np.ndarray:
    """The spinless 2-RDM, G[p, q, r, s] = <a+_p a+_r a_s a_q> over 2 norb
    orbitals (alpha first), from the spin blocks (states/states.py).  The
    alpha-beta block fills (a a | b b) directly, (b b | a a) with its pairs
    swapped, and the two exchange-ordered blocks (a b | b a), (b a | a b)
    with a minus sign from reordering the operators."""
    n = mat_aa.shape[0]
    a, b = slice(0, n), slice(n, 2 * n)
    out = np.zeros((2 * n,) * 4, dtype=np.result_type(mat_aa, mat_ab, mat_bb))
    out[a, a, a, a] = mat_aa
    out[b, b, b, b] = mat_bb
    out[a, a, b, b] = mat_ab
    out[b, b, a, a] = np.einsum("pqrs->rspq", mat_ab)
    out[a, b, b, a] = -np.einsum("psrq->pqrs", mat_ab)
    out[b, a, a, b] = -np.einsum("rqps->pqrs", mat_ab)
    return out
