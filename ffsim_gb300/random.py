"""Seeded random inputs.  Draws match python/ffsim/random/random.py for the same
seed, so the same inputs can be fed to this library and to the reference."""

from __future__ import annotations

import math

import numpy as np

from ffsim_gb300.hamiltonians import DoubleFactorizedHamiltonian
from ffsim_gb300.variational import UCJOpSpinBalanced


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


def random_real_symmetric_matrix(dim: int, *, rank: int | None = None, seed=None,
                                 dtype=float) -> np.ndarray:
    """M M^T with M a (dim, rank) Gaussian matrix (random.py:163-189)."""
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


def random_ucj_op_spin_balanced(norb: int, *, n_reps: int = 1, with_final_orbital_rotation: bool = False,
                                diag_coulomb_mean: float = 0.0, diag_coulomb_scale: float = 2 * math.pi,
                                diag_coulomb_normal: bool = False, seed=None) -> UCJOpSpinBalanced:
    """Random spin-balanced UCJ operator (random.py:563-665, no interaction pairs)."""
    rng = np.random.default_rng(seed)
    gen = random_symmetric_matrix_normal if diag_coulomb_normal else _random_symmetric_matrix_uniform
    dcm = np.stack([
        np.stack([gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng),
                  gen(norb, mean=diag_coulomb_mean, scale=diag_coulomb_scale, seed=rng)])
        for _ in range(n_reps)
    ])
    rots = np.stack([random_unitary(norb, seed=rng) for _ in range(n_reps)])
    final = random_unitary(norb, seed=rng) if with_final_orbital_rotation else None
    return UCJOpSpinBalanced(dcm, rots, final)


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
