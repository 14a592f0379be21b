"""Host linear algebra on the path (FP64): Givens decomposition, Hermitian
eigendecomposition and the UCJ parameter maps."""

from __future__ import annotations

import numpy as np
import scipy.linalg

from ffsim_gb300 import _lib


def givens_decomposition(mat: np.ndarray, tol: float = 1e-12):
    r"""Exact Givens decomposition :math:`U = D G_L^* \cdots G_1^*`.

    Same output as ``ffsim.linalg.givens_decomposition`` without compression
    (python/ffsim/linalg/givens.py:59-156 -> src/linalg/givens.rs:68-149): a list
    of ``(c, s, i, j)`` with ``|i - j| = 1`` and the diagonal of ``D``.
    """
    mat = np.asarray(mat)
    if mat.ndim != 2 or mat.shape[0] != mat.shape[1]:
        raise ValueError("mat must be a square matrix")
    n = mat.shape[0]
    m = _lib.cmat(mat)
    nmax = max(n * (n - 1) // 2, 1)
    cs = np.zeros(3 * nmax)
    ij = np.zeros(2 * nmax, dtype=np.int32)
    nrot = np.zeros(1, dtype=np.int32)
    diag = np.zeros(2 * max(n, 1))
    _lib.call("ffgb_givens_decomposition", _lib.dptr(m), n, float(tol), _lib.dptr(cs),
              ij.ctypes.data_as(_lib._ip), nrot.ctypes.data_as(_lib._ip), _lib.dptr(diag))
    rots = [(float(cs[3 * k]), complex(cs[3 * k + 1], cs[3 * k + 2]), int(ij[2 * k]), int(ij[2 * k + 1]))
            for k in range(int(nrot[0]))]
    return rots, diag[: 2 * n].view(np.complex128).copy()


def eigh(mat: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Hermitian eigendecomposition (ascending), computed by the library on the host."""
    mat = _lib.cmat(mat)
    n = mat.shape[0]
    w = np.zeros(n)
    v = np.zeros((n, n), dtype=np.complex128)
    _lib.call("ffgb_eigh", _lib.dptr(mat), n, _lib.dptr(w), v.ctypes.data_as(_lib._dp))
    return w, v


def antihermitians_from_parameters(params: np.ndarray, dim: int, n_mats: int) -> np.ndarray:
    """Batch of antihermitian matrices from real parameters (python/ffsim/linalg/util.py:93-124)."""
    params = np.asarray(params, dtype=float).reshape(n_mats, dim * dim)
    mats = np.zeros((n_mats, dim, dim), dtype=complex)
    n_triu = dim * (dim - 1) // 2
    rows, cols = np.triu_indices(dim)
    vals = 1j * params[:, n_triu:]
    mats[:, rows, cols] = vals
    mats[:, cols, rows] = vals
    rows, cols = np.triu_indices(dim, k=1)
    vals = params[:, :n_triu]
    mats[:, rows, cols] += vals
    mats[:, cols, rows] -= vals
    return mats


def antihermitians_to_parameters(mats: np.ndarray) -> np.ndarray:
    """Inverse of :func:`antihermitians_from_parameters` (python/ffsim/linalg/util.py:64-90)."""
    mats = np.asarray(mats)
    n_mats, dim, _ = mats.shape
    n_triu = dim * (dim - 1) // 2
    params = np.zeros((n_mats, dim * dim))
    rows, cols = np.triu_indices(dim, k=1)
    params[:, :n_triu] = mats[:, rows, cols].real
    rows, cols = np.triu_indices(dim)
    params[:, n_triu:] = mats[:, rows, cols].imag
    return params.reshape(-1)


def unitary_from_parameters(params: np.ndarray, dim: int) -> np.ndarray:
    """exp of the antihermitian matrix of the parameters (python/ffsim/linalg/util.py:189-232)."""
    return scipy.linalg.expm(antihermitians_from_parameters(params, dim, 1)[0])


def unitary_to_parameters(mat: np.ndarray) -> np.ndarray:
    """Parameters of the matrix logarithm (python/ffsim/linalg/util.py:160-186)."""
    return antihermitians_to_parameters(scipy.linalg.logm(np.asarray(mat))[None, :, :])


def is_unitary(mat: np.ndarray, *, rtol: float = 1e-5, atol: float = 1e-8) -> bool:
    mat = np.asarray(mat)
    return mat.ndim == 2 and mat.shape[0] == mat.shape[1] and np.allclose(
        mat @ mat.T.conj(), np.eye(mat.shape[0]), rtol=rtol, atol=atol)


def is_real_symmetric(mat: np.ndarray, *, rtol: float = 1e-5, atol: float = 1e-8) -> bool:
    mat = np.asarray(mat)
    return bool(np.all(np.isreal(mat)) and np.allclose(mat, mat.T, rtol=rtol, atol=atol))
