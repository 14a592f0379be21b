"""Host linear algebra on the path (FP64): Givens decomposition, Hermitian
eigendecomposition, the UCJ parameter maps, the double factorization of a
two-body tensor and tensor rotations."""

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


def modified_cholesky(mat: np.ndarray, *, tol: float = 1e-8, max_vecs: int | None = None) -> np.ndarray:
    r"""Pivoted ("modified") Cholesky factorization :math:`M \approx \sum_i v_i v_i^\dagger`
    of a positive semidefinite matrix (python/ffsim/linalg/double_factorized_decomposition.py:70-131;
    Motta and Zhang, arXiv:1711.02242).

    Each step pivots on the largest remaining diagonal error, takes that column
    of M minus the part the earlier vectors already explain, and scales it by
    the error's square root.  It stops when the largest error falls below
    ``tol`` or after ``max_vecs`` vectors; the vectors are the returned columns.
    """
    mat = np.asarray(mat)
    n = mat.shape[0]
    if not n:
        return np.empty((0, 0))
    if max_vecs is None:
        max_vecs = n
    vecs = np.zeros((n, max_vecs), dtype=mat.dtype)
    err = np.real(np.diagonal(mat)).copy()
    k = 0
    while k < max_vecs:
        piv = int(np.argmax(err))
        e = err[piv]
        if e < tol:
            break
        col = mat[:, piv].copy()
        if k:
            col -= vecs[:, :k] @ vecs[piv, :k].conj()
        vecs[:, k] = col / np.sqrt(e)
        err -= np.abs(vecs[:, k]) ** 2
        k += 1
    return vecs[:, :k]


def double_factorized(two_body_tensor: np.ndarray, *, tol: float = 1e-8, max_vecs: int | None = None,
                      optimize: bool = False, method: str = "L-BFGS-B", callback=None, options: dict | None = None,
                      diag_coulomb_indices=None, return_optimize_result: bool = False, cholesky: bool = True):
    r"""Double factorization :math:`h_{pqrs} = \sum_t \sum_{ij} U^t_{pi} U^{t*}_{qi} J^t_{ij} U^t_{rj} U^{t*}_{sj}`
    of a real two-body tensor (python/ffsim/linalg/double_factorized_decomposition.py:145-309).

    The (norb², norb²) matrix h[(p,q),(r,s)] is factored as a sum of outer
    products of vectors L_t (pivoted Cholesky, or its truncated
    eigendecomposition with ``cholesky=False``).  Each L_t, reshaped to a
    norb × norb matrix, is diagonalised, L_t = U_t diag(μ) U_t^dag, giving
    J_t = μ μ^T (times the eigenvalue on the eigendecomposition path).
    ``tol`` bounds the largest element error (Cholesky) or the discarded
    eigenvalue weight; ``max_vecs`` (default norb(norb+1)/2) caps the terms.
    Returns (diag_coulomb_mats, orbital_rotations).  The compressed form
    (``optimize=True``) fits the factors by gradient descent on a JAX loss in
    the reference and is not available here.
    """
    two_body_tensor = np.asarray(two_body_tensor)
    if np.iscomplexobj(two_body_tensor):
        raise ValueError("Double factorization of complex two-body tensors is not supported.")
    norb = two_body_tensor.shape[0]
    if not norb:
        return np.empty((0, 0, 0)), np.empty((0, 0, 0))
    if max_vecs is None:
        max_vecs = norb * (norb + 1) // 2
    if optimize:
        raise NotImplementedError("the compressed (optimize=True) double factorization is not available")
    flat = two_body_tensor.reshape(norb * norb, norb * norb)
    if cholesky:
        vecs = modified_cholesky(flat, tol=tol, max_vecs=max_vecs)
        mats = vecs.T.reshape(-1, norb, norb)
        mu, rots = np.linalg.eigh(mats)
        return mu[:, :, None] * mu[:, None, :], rots
    w, v = scipy.linalg.eigh(flat)
    order = np.argsort(np.abs(w))[::-1]
    w, v = w[order], v[:, order]
    n_drop = int(np.searchsorted(np.cumsum(np.abs(w[::-1])), tol))
    keep = min(max_vecs, len(w) - n_drop)
    w, v = w[:keep], v[:, :keep]
    mu, rots = np.linalg.eigh(v.T.reshape(-1, norb, norb))
    return w[:, None, None] * mu[:, :, None] * mu[:, None, :], rots


def rotate_one_body_tensor(tensor: np.ndarray, orbital_rotation: np.ndarray | None) -> np.ndarray:
    r""":math:`\sum_{ab} U_{Aa} \overline{U_{Bb}} t_{ab}`, the one-body tensor of
    :math:`\mathcal{U} H \mathcal{U}^\dagger` (python/ffsim/linalg/util.py:743-803)."""
    if orbital_rotation is None:
        return tensor
    u = np.asarray(orbital_rotation)
    return u @ np.asarray(tensor) @ u.conj().T


def rotate_two_body_tensor(tensor: np.ndarray, orbital_rotation_1: np.ndarray | None,
                           orbital_rotation_2: np.ndarray | None) -> np.ndarray:
    r""":math:`\sum_{abcd} U_{Aa} \overline{U_{Bb}} V_{Cc} \overline{V_{Dd}} t_{abcd}`
    (python/ffsim/linalg/util.py:813-900); ``None`` is the identity."""
    t = np.asarray(tensor)
    if orbital_rotation_1 is not None:
        u = np.asarray(orbital_rotation_1)
        t = np.einsum("abcd,Aa,Bb->ABcd", t, u, u.conj(), optimize=True)
    if orbital_rotation_2 is not None:
        v = np.asarray(orbital_rotation_2)
        t = np.einsum("abcd,Cc,Dd->abCD", t, v, v.conj(), optimize=True)
    return t


def double_factorized_t2(t2_amplitudes: np.ndarray, *, tol: float = 1e-8, max_terms: int | None = None,
                         optimize: bool = False, method: str = "L-BFGS-B", callback=None, options: dict | None = None,
                         diag_coulomb_indices=None, regularization: float = 0, multi_stage_start: int | None = None,
                         multi_stage_step: int | None = None, return_optimize_result: bool = False):
    r"""Double factorization of t2 amplitudes into diagonal Coulomb terms
    (python/ffsim/linalg/double_factorized_decomposition.py:467-659).

    The matrix T[(i, a), (j, b)] = t2[i, j, a, b] is diagonalised and
    truncated (largest |eigenvalues| first; the dropped tail's total |weight|
    stays below ``tol``).  Each eigenvector becomes the norb x norb matrix K
    with K[nocc + a, i] = v[(i, a)], and K splits into the two Hermitian
    quadratures Q_s = (1 - i s)(K + i s K^dag) / 2, s = +1, -1.  With
    Q_s = U diag(mu) U^dag the term is J = s lambda mu mu^T with rotation U.
    The terms (each eigenvector's + then -) are cut to ``max_terms``.  As in
    the reference, K is real: complex eigenvectors keep their real part.
    Returns (diag_coulomb_mats, orbital_rotations).  The compressed form
    (``optimize=True``) is fitted with a JAX gradient in the reference and is
    not available here.
    """
    if max_terms is not None and max_terms < 1:
        raise ValueError(f"max_terms must be at least 1. Got {max_terms}.")
    if optimize:
        raise NotImplementedError("the compressed (optimize=True) t2 factorization is not available")
    t2 = np.asarray(t2_amplitudes)
    nocc, _, nvrt, _ = t2.shape
    norb = nocc + nvrt
    w, v = scipy.linalg.eigh(t2.transpose(0, 2, 1, 3).reshape(nocc * nvrt, nocc * nvrt))
    order = np.argsort(np.abs(w))[::-1]
    w, v = w[order], v[:, order]
    keep = len(w) - int(np.searchsorted(np.cumsum(np.abs(w[::-1])), tol))
    w, v = w[:keep], v[:, :keep]
    occ = np.repeat(np.arange(nocc), nvrt)
    vrt = np.tile(np.arange(nocc, norb), nocc)
    quads = np.zeros((keep, 2, norb, norb), dtype=complex)
    for t in range(keep):
        k = np.zeros((norb, norb))
        k[vrt, occ] = v[:, t].real
        for m, sgn in enumerate((1, -1)):
            quads[t, m] = 0.5 * (1 - sgn * 1j) * (k + sgn * 1j * k.conj().T)
    mu, rots = np.linalg.eigh(quads)
    coeff = np.array([1, -1]) * w[:, None]
    mats = coeff[:, :, None, None] * mu[:, :, :, None] * mu[:, :, None, :]
    return mats.reshape(-1, norb, norb)[:max_terms], rots.reshape(-1, norb, norb)[:max_terms]


def reduced_matrix(mat, vecs) -> np.ndarray:
    """M[i, j] = <v_i| mat |v_j> (python/ffsim/linalg/linalg.py:50-69)."""
    from ffsim_gb300.multireference import reduced_matrix as _reduced

    return _reduced(mat, vecs)
