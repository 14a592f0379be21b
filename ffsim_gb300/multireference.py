"""Multireference states: the Hamiltonian projected onto ansatz-rotated
reference determinants (python/ffsim/variational/multireference.py:28-76,
python/ffsim/linalg/linalg.py:50-69)."""

from __future__ import annotations

import numpy as np
import scipy.linalg
import torch

from ffsim_gb300.protocols import LinearOperator, apply_unitary, linear_operator
from ffsim_gb300.states import slater_determinant, vdot


def _inner(a, b) -> complex:
    if isinstance(a, torch.Tensor):
        return vdot(a.reshape(-1), b.reshape(-1))
    return complex(np.vdot(a, b))


def reduced_matrix(mat, vecs) -> np.ndarray:
    """M[i, j] = <v_i| mat |v_j> over the given vectors (linalg.py:50-69).
    ``mat`` is one of this library's linear operators (CUDA tensors or numpy
    arrays), or any object with ``@`` on the vectors' type; the inner products
    of CUDA tensors are FP64 sums on the device."""
    n = len(vecs)
    out = np.zeros((n, n), dtype=complex)
    for j, vj in enumerate(vecs):
        hv = mat @ vj
        for i, vi in enumerate(vecs):
            out[i, j] = _inner(vi, hv)
    return out


def multireference_state(hamiltonian, ansatz_operator, reference_occupations, norb: int, nelec: tuple[int, int],
                         root: int = 0, *, dtype=torch.complex128):
    """Energy and state of the ``root``-th eigenvector of the Hamiltonian in
    the span of the ansatz applied to each reference determinant
    (multireference.py:28-76).  As in the reference the energy is
    Re sum_ij c_i c_j M_ij with the eigenvector c of M.  The states are
    built and rotated on the GPU (``slater_determinant``, ``apply_unitary``)
    and the state returned is a CUDA tensor."""
    lin = hamiltonian if isinstance(hamiltonian, LinearOperator) or not hasattr(hamiltonian, "_linear_operator_") \
        else linear_operator(hamiltonian, norb, nelec)
    basis = [apply_unitary(slater_determinant(norb, occ, dtype=dtype), ansatz_operator, norb, nelec, copy=False)
             for occ in reference_occupations]
    mat = reduced_matrix(lin, basis)
    _, vecs = scipy.linalg.eigh(mat)
    coeffs = vecs[:, root]
    energy = float(np.real(np.sum(np.outer(coeffs, coeffs) * mat)))
    state = sum(complex(c) * v for c, v in zip(coeffs, basis))
    return energy, state
