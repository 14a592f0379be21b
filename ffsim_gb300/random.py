"""Seeded random inputs.  Draws match python/ffsim/random/random.py for the same
seed, so the same inputs can be fed to this library and to the reference."""

from __future__ import annotations

import math

import numpy as np

from ffsim_gb300.hamiltonians import DiagonalCoulombHamiltonian, DoubleFactorizedHamiltonian, MolecularHamiltonian
from ffsim_gb300.variational import (
    UCJOpSpinBalanced,
    UCJOpSpinless,
    UCJOpSpinUnbalanced,
    validate_interaction_pairs,
)


def random_state_vector(dim: int, *, seed=None, dtype=complex) -> np.ndarray:
    """Normalised complex Gaussian vector (random.py:24-47)."""
    if dim < 1:
        raise ValueError("Dimension must be at least one.")
    rng = np.random.default_rng(seed)
    vec = rng.standard_normal(dim).astype(dtype, copy=False)
    if np.issubdtype(dtype, np.complexfloating):
        vec += 1j * rng.standard_normal(dim).astype(dtype, copy=False)
    vec /= np.linalg.norm(vec)
    return vec


def random_unitary(dim: int, *, seed=None, dtype=complex) -> np.ndarray:
    """Haar unitary via QR with phase fix (random.py:84-106)."""
    rng = np.random.default_rng(seed)
    z = rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    z += 1j * rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    q, r = np.linalg.qr(z)
    d = np.diagonal(r)
    return q * (d / np.abs(d))


def random_density_matrix(dim: int, *, seed=None, dtype=complex) -> np.ndarray:
    """G G^dag / tr, G Gaussian: the Hilbert-Schmidt measure (random.py:50-81)."""
    if dim < 1:
        raise ValueError("Dimension must be at least one.")
    rng = np.random.default_rng(seed)
    mat = rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    if np.issubdtype(dtype, np.complexfloating):
        mat += 1j * rng.standard_normal((dim, dim))
    mat = mat @ mat.T.conj()
    return mat / np.trace(mat)


def random_orthogonal(dim: int, seed=None, dtype=float) -> np.ndarray:
    """Haar orthogonal matrix via QR with sign fix (random.py:109-130)."""
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    q, r = np.linalg.qr(m)
    d = np.diagonal(r)
    return q * (d / np.abs(d))


def random_special_orthogonal(dim: int, seed=None, dtype=float) -> np.ndarray:
    """Haar orthogonal matrix with its first row negated when the determinant is -1 (random.py:133-148)."""
    mat = random_orthogonal(dim, seed=seed, dtype=dtype)
    if np.linalg.det(mat) < 0:
        mat[0] *= -1
    return mat


def random_hermitian(dim: int, *, seed=None, dtype=complex) -> np.ndarray:
    """G + G^dag for a complex Gaussian G (random.py:151-167)."""
    rng = np.random.default_rng(seed)
    mat = rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    mat += 1j * rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    return mat + mat.T.conj()


def random_antihermitian(dim: int, *, seed=None, dtype=complex) -> np.ndarray:
    """G - G^dag for a complex Gaussian G (random.py:192-208)."""
    rng = np.random.default_rng(seed)
    mat = rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    mat += 1j * rng.standard_normal((dim, dim)).astype(dtype, copy=False)
    return mat - mat.T.conj()


def random_two_body_tensor(dim: int, *, rank: int | None = None, seed=None, dtype=complex) -> np.ndarray:
    """sum_k M_k (x) M_k over Hermitian (real symmetric for real dtype) M_k: a
    two-body tensor with the symmetries of molecular integrals (random.py:212-237)."""
    rng = np.random.default_rng(seed)
    is_complex = np.issubdtype(dtype, np.complexfloating)
    if rank is None:
        rank = dim**2 if is_complex else dim * (dim + 1) // 2
    mats = rng.standard_normal((rank, dim, dim)).astype(dtype, copy=False)
    if is_complex:
        mats += 1j * rng.standard_normal((rank, dim, dim))
    mats += mats.transpose(0, 2, 1).conj()
    return np.tensordot(mats, mats, axes=(0, 0))


def random_t2_amplitudes(norb: int, nocc: int, *, seed=None, dtype=complex) -> np.ndarray:
    """t2[i, j, a, b] = t2[j, i, b, a], one normal draw per unordered pair of
    (occupied, virtual) pairs; complex amplitudes are then rotated by a Haar
    unitary in the full orbital space (random.py:240-276)."""
    import itertools

    rng = np.random.default_rng(seed)
    nvrt = norb - nocc
    t2 = np.zeros((nocc, nocc, nvrt, nvrt), dtype=dtype)
    pairs = list(itertools.product(range(nocc), range(nocc, norb)))
    for (i, a), (j, b) in itertools.combinations_with_replacement(pairs, 2):
        val = rng.standard_normal()
        t2[i, j, a - nocc, b - nocc] = val
        t2[j, i, b - nocc, a - nocc] = val
    if np.issubdtype(dtype, np.complexfloating):
        big = np.zeros((norb, norb, norb, norb), dtype=dtype)
        big[:nocc, :nocc, nocc:, nocc:] = t2
        u = random_unitary(norb, seed=rng)
        big = np.einsum("ijab,iI,jJ,aA,bB->IJAB", big, u.conj(), u.conj(), u, u, optimize=True)
        t2 = big[:nocc, :nocc, nocc:, nocc:]
    return t2


def random_molecular_hamiltonian(norb: int, seed=None, dtype=complex) -> MolecularHamiltonian:
    """Random molecular Hamiltonian (random.py:279-305)."""
    rng = np.random.default_rng(seed)
    if np.issubdtype(dtype, np.complexfloating):
        one_body = random_hermitian(norb, seed=rng, dtype=dtype)
    else:
        one_body = random_real_symmetric_matrix(norb, seed=rng, dtype=dtype)
    two_body = random_two_body_tensor(norb, seed=rng, dtype=dtype)
    constant = rng.standard_normal()
    return MolecularHamiltonian(one_body, two_body, constant=constant)


def random_diagonal_coulomb_hamiltonian(norb: int, *, real: bool = False, seed=None) -> DiagonalCoulombHamiltonian:
    """Random diagonal Coulomb Hamiltonian (random.py:883-908)."""
    rng = np.random.default_rng(seed)
    if real:
        one_body = random_real_symmetric_matrix(norb, seed=rng)
    else:
        one_body = random_hermitian(norb, seed=rng)
    mat_aa = random_real_symmetric_matrix(norb, seed=rng)
    mat_ab = random_real_symmetric_matrix(norb, seed=rng)
    constant = rng.standard_normal()
    return DiagonalCoulombHamiltonian(one_body, np.stack([mat_aa, mat_ab]), constant=constant)


def random_double_factorized_hamiltonian(norb: int, *, rank: int | None = None, z_representation: bool = False,
                                         real: bool = False, seed=None) -> DoubleFactorizedHamiltonian:
    """Random double-factorized Hamiltonian (random.py:911-956): rank terms
    (default norb(norb+1)/2) with Haar rotations (orthogonal when ``real``) and
    M M^T Coulomb matrices."""
    if rank is None:
        rank = norb * (norb + 1) // 2
    rng = np.random.default_rng(seed)
    if real:
        one_body = random_real_symmetric_matrix(norb, seed=rng)
        rots = np.stack([random_orthogonal(norb, seed=rng) for _ in range(rank)])
    else:
        one_body = random_hermitian(norb, seed=rng)
        rots = np.stack([random_unitary(norb, seed=rng) for _ in range(rank)])
    dcm = np.stack([random_real_symmetric_matrix(norb, seed=rng) for _ in range(rank)])
    constant = rng.standard_normal()
    return DoubleFactorizedHamiltonian(one_body, dcm, rots, constant=constant, z_representation=z_representation)


def random_real_symmetric_matrix(dim: int, *, rank: int | None = None, seed=None,
                                 dtype=float) -> np.ndarray:
    """M M^T with M a (dim, rank) Gaussian matrix (random.py:170-189)."""
    rng = np.random.default_rng(seed)
    if rank is None:
        rank = dim
    mat = rng.standard_normal((dim, rank)).astype(dtype, copy=False)
    return mat @ mat.T


def random_symmetric_matrix_normal(dim: int, *, mean: float = 0.0, scale: float = 1.0,
                                   seed=None) -> np.ndarray:
    """Upper triangle i.i.d. normal(mean, scale), mirrored (random.py:549-560)."""
    rng = np.random.default_rng(seed)
    vals = rng.normal(loc=mean, scale=scale, size=dim * (dim + 1) // 2)
    mat = np.zeros((dim, dim))
    rows, cols = np.triu_indices(dim)
    mat[rows, cols] = vals
    mat[cols, rows] = vals
    return mat


def _random_symmetric_matrix_uniform(dim: int, *, mean: float, scale: float, seed=None) -> np.ndarray:
    rng = np.random.default_rng(seed)
    vals = mean + rng.uniform(-0.5 * scale, 0.5 * scale, size=dim * (dim + 1) // 2)
    mat = np.zeros((dim, dim))
    rows, cols = np.triu_indices(dim)
    mat[rows, cols] = vals
    mat[cols, rows] = vals
    return mat


def _pair_mask(norb: int, pairs, symmetric: bool) -> np.ndarray:
    mask = np.zeros((norb, norb), dtype=bool)
    if pairs:
        rows, cols = zip(*pairs)
        mask[rows, cols] = True
        if symmetric:
            mask[cols, rows] = True
    return mask


def _dc_generator(normal: bool):
    return random_symmetric_matrix_normal if normal else _random_symmetric_matrix_uniform


def random_ucj_op_spin_balanced(norb: int, *, n_reps: int = 1, interaction_pairs=None,
                                with_final_orbital_rotation: bool = False, diag_coulomb_mean: float = 0.0,
                                diag_coulomb_scale: float = 2 * math.pi, diag_coulomb_normal: bool = False,
                                seed=None) -> UCJOpSpinBalanced:
    """Random spin-balanced UCJ operator (random.py:563-665): per layer an
    alpha-alpha and an alpha-beta symmetric matrix, then the layer rotations
    and the optional final rotation; entries outside the interaction pairs
    are zeroed after the draws."""
    pairs_aa, pairs_ab = (None, None) if interaction_pairs is None else interaction_pairs
    validate_interaction_pairs(pairs_aa, ordered=False)
    validate_interaction_pairs(pairs_ab, ordered=False)
    rng = np.random.default_rng(seed)
    gen = _dc_generator(diag_coulomb_normal)
    dcm = np.stack([
        np.stack([gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng),
                  gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng)])
        for _ in range(n_reps)
    ])
    rots = np.stack([random_unitary(norb, seed=rng) for _ in range(n_reps)])
    final = random_unitary(norb, seed=rng) if with_final_orbital_rotation else None
    if pairs_aa is not None:
        dcm[:, 0] *= _pair_mask(norb, pairs_aa, True)
    if pairs_ab is not None:
        dcm[:, 1] *= _pair_mask(norb, pairs_ab, True)
    return UCJOpSpinBalanced(dcm, rots, final)


def random_ucj_op_spin_unbalanced(norb: int, *, n_reps: int = 1, interaction_pairs=None,
                                  with_final_orbital_rotation: bool = False, diag_coulomb_mean: float = 0.0,
                                  diag_coulomb_scale: float = 2 * math.pi, diag_coulomb_normal: bool = False,
                                  seed=None) -> UCJOpSpinUnbalanced:
    """Random spin-unbalanced UCJ operator (random.py:668-799): per layer a
    symmetric alpha-alpha matrix, a general alpha-beta matrix and a symmetric
    beta-beta matrix, then a pair of rotations per layer and the optional
    final pair.  Alpha-beta pairs mask one entry each (the matrix is not
    symmetric); like the reference, only the same-spin pairs are validated."""
    pairs_aa, pairs_ab, pairs_bb = (None, None, None) if interaction_pairs is None else interaction_pairs
    validate_interaction_pairs(pairs_aa, ordered=False)
    validate_interaction_pairs(pairs_bb, ordered=False)
    rng = np.random.default_rng(seed)
    gen = _dc_generator(diag_coulomb_normal)

    def general(n):
        if diag_coulomb_normal:
            return rng.normal(loc=diag_coulomb_mean, scale=diag_coulomb_scale, size=(n, n))
        return diag_coulomb_mean + rng.uniform(-0.5 * diag_coulomb_scale, 0.5 * diag_coulomb_scale, size=(n, n))

    dcm = np.stack([
        np.stack([gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng),
                  general(norb),
                  gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng)])
        for _ in range(n_reps)
    ])
    rots = np.stack([np.stack([random_unitary(norb, seed=rng), random_unitary(norb, seed=rng)])
                     for _ in range(n_reps)])
    final = None
    if with_final_orbital_rotation:
        final = np.stack([random_unitary(norb, seed=rng), random_unitary(norb, seed=rng)])
    if pairs_aa is not None:
        dcm[:, 0] *= _pair_mask(norb, pairs_aa, True)
    if pairs_ab is not None:
        dcm[:, 1] *= _pair_mask(norb, pairs_ab, False)
    if pairs_bb is not None:
        dcm[:, 2] *= _pair_mask(norb, pairs_bb, True)
    return UCJOpSpinUnbalanced(dcm, rots, final)


def random_ucj_op_spinless(norb: int, *, n_reps: int = 1, interaction_pairs=None,
                           with_final_orbital_rotation: bool = False, diag_coulomb_mean: float = 0.0,
                           diag_coulomb_scale: float = 2 * math.pi, diag_coulomb_normal: bool = False,
                           seed=None) -> UCJOpSpinless:
    """Random spinless UCJ operator (random.py:802-880)."""
    validate_interaction_pairs(interaction_pairs, ordered=False)
    rng = np.random.default_rng(seed)
    gen = _dc_generator(diag_coulomb_normal)
    dcm = np.stack([gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng) for _ in range(n_reps)])
    rots = np.stack([random_unitary(norb, seed=rng) for _ in range(n_reps)])
    final = random_unitary(norb, seed=rng) if with_final_orbital_rotation else None
    if interaction_pairs is not None:
        dcm *= _pair_mask(norb, interaction_pairs, True)
    return UCJOpSpinless(dcm, rots, final)


def random_df_hamiltonian_normal(norb: int, *, rank: int, one_body_scale: float = 1.0 / 16,
                                 diag_coulomb_scale: float = 0.05, constant: float = -100.0,
                                 seed=None) -> DoubleFactorizedHamiltonian:
    """Synthetic double-factorized Hamiltonian of the LUCJ energy workload:
    Hermitian one-body matrix with entries N(0,1)*one_body_scale ((G + G^H)/2),
    ``rank`` Haar orbital rotations and real symmetric diagonal Coulomb
    matrices with upper triangles N(0, diag_coulomb_scale), number representation."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))
    one_body = 0.5 * (g + g.conj().T) * one_body_scale
    dcm = np.stack([random_symmetric_matrix_normal(norb, scale=diag_coulomb_scale, seed=rng)
                    for _ in range(rank)])
    rots = np.stack([random_unitary(norb, seed=rng) for _ in range(rank)])
    return DoubleFactorizedHamiltonian(one_body, dcm, rots, constant=constant)
