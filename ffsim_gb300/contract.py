"""Contractions and linear operators: the GPU counterparts of
python/ffsim/contract/{diag_coulomb,num_op_sum,one_body}.py."""

from __future__ import annotations

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import dim as _dim
from ffsim_gb300._state import prepare, scratch, stream_ptr
from ffsim_gb300.gates import _dagger, _split_pair, apply_orbital_rotation
from ffsim_gb300.linalg import eigh
from ffsim_gb300.protocols import LinearOperator


def _mats(mat):
    """(aa, ab, bb) from a single matrix or a triple (python/ffsim/contract/diag_coulomb.py:102-130)."""
    if isinstance(mat, np.ndarray) and mat.ndim == 2:
        return mat, mat, mat
    aa, ab, bb = mat
    return aa, ab, bb


def contract_diag_coulomb(vec, mat, norb: int, nelec: tuple[int, int], *, z_representation: bool = False):
    r"""Return :math:`\sum Z^{(\sigma\tau)}_{ij} n_{i\sigma} n_{j\tau}/2 \, |vec\rangle`
    (python/ffsim/contract/diag_coulomb.py:41-99)."""
    p = prepare(vec, norb, nelec, copy=False)
    out = torch.empty_like(p.tensor)
    aa, ab, bb = (_lib.rmat(m, (norb, norb), "diagonal Coulomb matrix") for m in _mats(mat))
    n_alpha, n_beta = nelec
    _lib.call("ffgb_contract_diag_coulomb", p.ptr(), out.data_ptr(), p.dtype_code, norb, n_alpha, n_beta,
              _lib.dptr(aa), _lib.dptr(ab), _lib.dptr(bb), int(bool(z_representation)), 0,
              stream_ptr(p.tensor))
    return p.finish(out)


def contract_num_op_sum(vec, coeffs, norb: int, nelec: tuple[int, int]):
    r"""Return :math:`\sum_{i\sigma} \lambda_i n_{i\sigma} |vec\rangle`
    (python/ffsim/contract/num_op_sum.py:27-72)."""
    p = prepare(vec, norb, nelec, copy=False)
    out = torch.empty_like(p.tensor)
    c = _lib.rmat(coeffs, (norb,), "coefficients")
    n_alpha, n_beta = nelec
    _lib.call("ffgb_contract_num_op_sum", p.ptr(), out.data_ptr(), p.dtype_code, norb, n_alpha, n_beta,
              _lib.dptr(c), 0, stream_ptr(p.tensor))
    return p.finish(out)


def _rotated_matvec(vec: torch.Tensor, norb, nelec, one_body, mat, z_rep, rot):
    n_alpha, n_beta = nelec
    t = vec if vec.is_contiguous() else vec.contiguous()
    out = torch.empty_like(t)
    code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
    buf, nbytes = scratch(t, 1, norb, n_alpha, n_beta)
    ob = _lib.rmat(one_body, (norb,), "coefficients")
    m = _lib.rmat(mat, (norb, norb), "diagonal Coulomb matrix")
    r = _lib.cmat(rot, (norb, norb), "orbital rotation")
    _lib.call("ffgb_rotated_diag_matvec", t.data_ptr(), out.data_ptr(), code, norb, n_alpha, n_beta,
              _lib.dptr(ob), _lib.dptr(m), int(bool(z_rep)), _lib.dptr(r), 0, buf.data_ptr(), nbytes,
              stream_ptr(t))
    return out


def diag_coulomb_linop(mat, norb: int, nelec: tuple[int, int], *, orbital_rotation=None,
                       z_representation: bool = False) -> LinearOperator:
    r"""Linear operator :math:`\mathcal{U} Z \mathcal{U}^\dagger`
    (python/ffsim/contract/diag_coulomb.py:195-272); matvec = rmatvec."""
    d = _dim(norb, nelec)
    single_mat = isinstance(mat, np.ndarray) and mat.ndim == 2
    single_rot = orbital_rotation is None or (
        isinstance(orbital_rotation, np.ndarray) and orbital_rotation.ndim == 2
    )

    def matvec(vec: torch.Tensor) -> torch.Tensor:
        if single_mat and single_rot:
            return _rotated_matvec(vec, norb, nelec, None, mat, z_representation, orbital_rotation)
        v = vec
        if orbital_rotation is not None:
            ra, rb = _split_pair(orbital_rotation)
            v = apply_orbital_rotation(v, (_dagger(ra), _dagger(rb)), norb, nelec)
        v = contract_diag_coulomb(v, mat, norb, nelec, z_representation=z_representation)
        if orbital_rotation is not None:
            v = apply_orbital_rotation(v, orbital_rotation, norb, nelec, copy=False)
        return v

    return LinearOperator((d, d), matvec)


def num_op_sum_linop(coeffs, norb: int, nelec: tuple[int, int], *, orbital_rotation=None) -> LinearOperator:
    r"""Linear operator :math:`\mathcal{U} (\sum \lambda_i n_{i\sigma}) \mathcal{U}^\dagger`
    (python/ffsim/contract/num_op_sum.py:75-131)."""
    d = _dim(norb, nelec)

    def matvec(vec: torch.Tensor) -> torch.Tensor:
        return _rotated_matvec(vec, norb, nelec, coeffs, None, False, orbital_rotation)

    return LinearOperator((d, d), matvec)


def _hermitian_parts(mat):
    """M = A + i B with A = (M + M^H) / 2, B = (M - M^H) / (2i), both Hermitian."""
    m = np.asarray(mat, dtype=complex)
    return (m + m.conj().T) / 2, (m - m.conj().T) / 2j


def contract_one_body(vec, mat, norb: int, nelec: tuple[int, int]):
    r""":math:`\sum_{pq} M_{pq} a^\dagger_{p\sigma} a_{q\sigma}` applied to ``vec``
    (python/ffsim/contract/one_body.py:24-58) for any complex matrix M.

    Each Hermitian part of M is diagonal in its eigenbasis, so its action is one
    rotated number-operator matvec ``W(V) (sum_i w_i n_i) W(V)^dag``
    (``ffgb_rotated_diag_matvec``); the anti-Hermitian part adds a second one.
    """
    a, b = _hermitian_parts(mat)
    wa, va = eigh(a)
    out = num_op_sum_linop(wa, norb, nelec, orbital_rotation=va) @ vec
    if np.abs(b).max() > 0.0:
        wb, vb = eigh(b)
        out = out + 1j * (num_op_sum_linop(wb, norb, nelec, orbital_rotation=vb) @ vec)
    return out


def one_body_linop(mat, norb: int, nelec: tuple[int, int]) -> LinearOperator:
    """Linear operator of a one-body tensor (python/ffsim/contract/one_body.py:61-90);
    rmatvec applies M^H."""
    d = _dim(norb, nelec)
    m = np.asarray(mat, dtype=complex)
    return LinearOperator((d, d), lambda v: contract_one_body(v, m, norb, nelec),
                          lambda v: contract_one_body(v, m.conj().T, norb, nelec))
