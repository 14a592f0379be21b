"""Spin-balanced unitary cluster Jastrow operator
(python/ffsim/variational/ucj_spin_balanced.py) with a GPU ``_apply_unitary_``."""

from __future__ import annotations

import itertools
from dataclasses import InitVar, dataclass

import numpy as np

from ffsim_gb300 import _lib, linalg
from ffsim_gb300._state import prepare, scratch, split_nelec, stream_ptr


@dataclass(frozen=True)
class UCJOpSpinBalanced:
    r""":math:`\prod_{k=1}^L \mathcal{U}_k e^{i \mathcal{J}_k} \mathcal{U}_k^\dagger`, optionally
    followed by a final orbital rotation.  Fields and validation as in
    ucj_spin_balanced.py:31-141."""

    diag_coulomb_mats: np.ndarray  # (n_reps, 2, norb, norb): [aa, ab]
    orbital_rotations: np.ndarray  # (n_reps, norb, norb)
    final_orbital_rotation: np.ndarray | None = None
    validate: InitVar[bool] = True
    rtol: InitVar[float] = 1e-5
    atol: InitVar[float] = 1e-8

    def __post_init__(self, validate: bool, rtol: float, atol: float):
        if not validate:
            return
        if self.diag_coulomb_mats.ndim != 4 or self.diag_coulomb_mats.shape[1] != 2:
            raise ValueError(
                "diag_coulomb_mats should have shape (n_reps, 2, norb, norb). "
                f"Got shape {self.diag_coulomb_mats.shape}.")
        if self.orbital_rotations.ndim != 3:
            raise ValueError(
                "orbital_rotations should have shape (n_reps, norb, norb). "
                f"Got shape {self.orbital_rotations.shape}.")
        if self.final_orbital_rotation is not None and self.final_orbital_rotation.ndim != 2:
            raise ValueError(
                "final_orbital_rotation should have shape (norb, norb). "
                f"Got shape {self.final_orbital_rotation.shape}.")
        if self.diag_coulomb_mats.shape[0] != self.orbital_rotations.shape[0]:
            raise ValueError(
                "diag_coulomb_mats and orbital_rotations should have the same first dimension. "
                f"Got {self.diag_coulomb_mats.shape[0]} and {self.orbital_rotations.shape[0]}.")
        if not all(linalg.is_real_symmetric(m[0], rtol=rtol, atol=atol)
                   and linalg.is_real_symmetric(m[1], rtol=rtol, atol=atol)
                   for m in self.diag_coulomb_mats):
            raise ValueError("Diagonal Coulomb matrices were not all real symmetric.")
        if not all(linalg.is_unitary(u, rtol=rtol, atol=atol) for u in self.orbital_rotations):
            raise ValueError("Orbital rotations were not all unitary.")
        if self.final_orbital_rotation is not None and not linalg.is_unitary(
                self.final_orbital_rotation, rtol=rtol, atol=atol):
            raise ValueError("Final orbital rotation was not unitary.")

    @property
    def norb(self) -> int:
        return self.diag_coulomb_mats.shape[-1]

    @property
    def n_reps(self) -> int:
        return self.diag_coulomb_mats.shape[0]

    @staticmethod
    def n_params(norb: int, n_reps: int, *, with_final_orbital_rotation: bool = False) -> int:
        """ucj_spin_balanced.py:149-195 without interaction pairs."""
        n_triu = norb * (norb + 1) // 2
        return n_reps * (2 * n_triu + norb**2) + with_final_orbital_rotation * norb**2

    @staticmethod
    def from_parameters(params: np.ndarray, *, norb: int, n_reps: int,
                        with_final_orbital_rotation: bool = False) -> "UCJOpSpinBalanced":
        """ucj_spin_balanced.py:197-293 without interaction pairs: per rep, the
        orbital rotation's norb**2 parameters, then the aa and ab upper triangles."""
        params = np.asarray(params, dtype=float)
        n = UCJOpSpinBalanced.n_params(norb, n_reps, with_final_orbital_rotation=with_final_orbital_rotation)
        if len(params) != n:
            raise ValueError(
                "The number of parameters passed did not match the number expected based on the "
                f"function inputs. Expected {n} but got {len(params)}.")
        triu = list(itertools.combinations_with_replacement(range(norb), 2))
        rows, cols = zip(*triu)
        dcm = np.zeros((n_reps, 2, norb, norb))
        rots = np.zeros((n_reps, norb, norb), dtype=complex)
        index = 0
        for r in range(n_reps):
            rots[r] = linalg.unitary_from_parameters(params[index: index + norb**2], norb)
            index += norb**2
            for t in range(2):
                vals = params[index: index + len(triu)]
                dcm[r, t][cols, rows] = vals
                dcm[r, t][rows, cols] = vals
                index += len(triu)
        final = None
        if with_final_orbital_rotation:
            final = linalg.unitary_from_parameters(params[index:], norb)
        return UCJOpSpinBalanced(dcm, rots, final)

    def to_parameters(self) -> np.ndarray:
        """ucj_spin_balanced.py:295-374 without interaction pairs."""
        n_reps, _, norb, _ = self.diag_coulomb_mats.shape
        triu = list(itertools.combinations_with_replacement(range(norb), 2))
        idx = tuple(zip(*triu))
        out = []
        for u, mats in zip(self.orbital_rotations, self.diag_coulomb_mats):
            out.append(linalg.unitary_to_parameters(u))
            out.append(mats[0][idx])
            out.append(mats[1][idx])
        if self.final_orbital_rotation is not None:
            out.append(linalg.unitary_to_parameters(self.final_orbital_rotation))
        return np.concatenate(out)

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        """GPU counterpart of ucj_spin_balanced.py:657-696: for each rep, the
        merged rotation U_k^dag U_{k-1} then exp(-i(-1) J_k), then the final rotation."""
        if isinstance(nelec, (int, np.integer)):
            return NotImplemented
        n_alpha, n_beta = split_nelec(nelec)
        p = prepare(vec, norb, nelec, copy=copy)
        dcm = _lib.rmat(self.diag_coulomb_mats)
        rots = _lib.cmat(self.orbital_rotations)
        final = _lib.cmat(self.final_orbital_rotation)
        buf, nbytes = scratch(p.tensor, 0, norb, n_alpha, n_beta)
        _lib.call("ffgb_ucj_spin_balanced_apply", p.ptr(), p.dtype_code, norb, n_alpha, n_beta,
                  self.n_reps, _lib.dptr(dcm), rots.ctypes.data_as(_lib._dp), _lib.dptr(final),
                  buf.data_ptr(), nbytes, stream_ptr(p.tensor))
        return p.finish()

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, UCJOpSpinBalanced):
            return NotImplemented
        if not np.allclose(self.diag_coulomb_mats, other.diag_coulomb_mats, rtol=rtol, atol=atol):
            return False
        if not np.allclose(self.orbital_rotations, other.orbital_rotations, rtol=rtol, atol=atol):
            return False
        if (self.final_orbital_rotation is None) != (other.final_orbital_rotation is None):
            return False
        if self.final_orbital_rotation is not None:
            return bool(np.allclose(self.final_orbital_rotation, other.final_orbital_rotation,
                                    rtol=rtol, atol=atol))
        return True
