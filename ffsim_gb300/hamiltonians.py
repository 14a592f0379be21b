"""Double-factorized Hamiltonian with a GPU linear operator
(python/ffsim/hamiltonians/double_factorized_hamiltonian.py)."""

from __future__ import annotations

import dataclasses

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import dim as _dim
from ffsim_gb300._state import scratch, stream_ptr
from ffsim_gb300.protocols import LinearOperator


@dataclasses.dataclass(frozen=True)
class DoubleFactorizedHamiltonian:
    r""":math:`H = \sum \kappa_{pq} a^\dagger_{p\sigma} a_{q\sigma} + \frac12 \sum_t \sum J^{(t)}_{ij}
    n^{(t)}_{i\sigma} n^{(t)}_{j\tau} + \text{constant}` with
    :math:`n^{(t)}_{i\sigma} = \sum_{pq} U^{(t)}_{pi} a^\dagger_{p\sigma} a_{q\sigma} U^{(t)*}_{qi}`.

    Same fields as the reference dataclass (double_factorized_hamiltonian.py:28-105).
    """

    one_body_tensor: np.ndarray
    diag_coulomb_mats: np.ndarray
    orbital_rotations: np.ndarray
    constant: float = 0.0
    z_representation: bool = False

    @property
    def norb(self) -> int:
        return self.one_body_tensor.shape[0]

    def _arrays(self):
        return (
            _lib.cmat(self.one_body_tensor),
            _lib.rmat(self.diag_coulomb_mats).reshape(-1, self.norb, self.norb),
            _lib.cmat(self.orbital_rotations).reshape(-1, self.norb, self.norb),
        )

    def to_z_representation(self) -> "DoubleFactorizedHamiltonian":
        if self.z_representation:
            return self
        ob, c = _df_z_representation(self.diag_coulomb_mats, self.orbital_rotations)
        return DoubleFactorizedHamiltonian(self.one_body_tensor + ob, self.diag_coulomb_mats,
                                           self.orbital_rotations, self.constant + c, True)

    def to_number_representation(self) -> "DoubleFactorizedHamiltonian":
        if not self.z_representation:
            return self
        ob, c = _df_z_representation(self.diag_coulomb_mats, self.orbital_rotations)
        return DoubleFactorizedHamiltonian(self.one_body_tensor - ob, self.diag_coulomb_mats,
                                           self.orbital_rotations, self.constant - c, False)

    def _linear_operator_(self, norb: int, nelec) -> LinearOperator:
        """GPU counterpart of double_factorized_hamiltonian.py:244-275 (matvec = rmatvec),
        with a fused FP64 ``expectation``."""
        assert isinstance(nelec, tuple)
        d = _dim(norb, nelec)
        n_alpha, n_beta = nelec
        one_body, dcm, rots = self._arrays()
        n_terms = dcm.shape[0]

        def matvec(vec: torch.Tensor) -> torch.Tensor:
            t = vec.contiguous()
            if t.dtype not in (torch.complex64, torch.complex128):
                t = t.to(torch.complex128)
            out = torch.empty_like(t)
            code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
            buf, nbytes = scratch(t, 1, norb, n_alpha, n_beta)
            _lib.call("ffgb_df_matvec", t.data_ptr(), out.data_ptr(), code, norb, n_alpha, n_beta,
                      _lib.dptr(one_body), n_terms, _lib.dptr(dcm), rots.ctypes.data_as(_lib._dp),
                      float(self.constant), int(bool(self.z_representation)), buf.data_ptr(), nbytes,
                      stream_ptr(t))
            return out

        def expectation(vec: torch.Tensor) -> float:
            t = vec.contiguous()
            code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
            buf, nbytes = scratch(t, 2, norb, n_alpha, n_beta)
            e = np.zeros(1)
            _lib.call("ffgb_df_expectation", t.data_ptr(), code, norb, n_alpha, n_beta,
                      _lib.dptr(one_body), n_terms, _lib.dptr(dcm), rots.ctypes.data_as(_lib._dp),
                      float(self.constant), int(bool(self.z_representation)), None, _lib.dptr(e),
                      buf.data_ptr(), nbytes, stream_ptr(t))
            return float(e[0])

        return LinearOperator((d, d), matvec, matvec, expectation)


def _df_z_representation(diag_coulomb_mats, orbital_rotations):
    """One-body and constant corrections between representations
    (double_factorized_hamiltonian.py:306-328)."""
    one_body = 0.5 * (
        np.einsum("tij,tpi,tqi->pq", diag_coulomb_mats, orbital_rotations, orbital_rotations.conj())
        + np.einsum("tij,tpj,tqj->pq", diag_coulomb_mats, orbital_rotations, orbital_rotations.conj())
    )
    constant = 0.25 * np.einsum("ijj->", diag_coulomb_mats) - 0.5 * np.sum(diag_coulomb_mats)
    return one_body, float(constant)
