"""Double-factorized and molecular Hamiltonians with GPU linear operators
(python/ffsim/hamiltonians/double_factorized_hamiltonian.py, molecular_hamiltonian.py)."""

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
        n = self.norb
        dcm = _lib.rmat(self.diag_coulomb_mats)
        rots = _lib.cmat(self.orbital_rotations)
        if dcm.ndim == 2:  # one term given as a single matrix
            dcm = dcm[None]
        if rots.ndim == 2:
            rots = rots[None]
        n_terms = dcm.shape[0] if dcm.ndim == 3 else -1
        return (
            _lib.cmat(self.one_body_tensor, (n, n), "one_body_tensor"),
            _lib.rmat(dcm, (n_terms, n, n), "diag_coulomb_mats"),
            _lib.cmat(rots, (n_terms, n, n), "orbital_rotations"),
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

    @staticmethod
    def from_molecular_hamiltonian(hamiltonian: "MolecularHamiltonian", *, z_representation: bool = False,
                                   tol: float = 1e-8, max_vecs: int | None = None, optimize: bool = False,
                                   method: str = "L-BFGS-B", callback=None, options: dict | None = None,
                                   diag_coulomb_indices=None, cholesky: bool = True) -> "DoubleFactorizedHamiltonian":
        """Double-factorize a molecular Hamiltonian (double_factorized_hamiltonian.py:140-222):
        normal ordering moves -1/2 sum_r h_prrq into the one-body tensor, and
        the two-body tensor is factored by ``linalg.double_factorized``."""
        from ffsim_gb300.linalg import double_factorized

        one_body = hamiltonian.one_body_tensor - 0.5 * np.einsum("prrq", hamiltonian.two_body_tensor)
        mats, rots = double_factorized(hamiltonian.two_body_tensor, tol=tol, max_vecs=max_vecs, optimize=optimize,
                                       method=method, callback=callback, options=options,
                                       diag_coulomb_indices=diag_coulomb_indices, cholesky=cholesky)
        df = DoubleFactorizedHamiltonian(one_body, mats, rots, constant=hamiltonian.constant)
        return df.to_z_representation() if z_representation else df

    def to_molecular_hamiltonian(self) -> "MolecularHamiltonian":
        """The molecular Hamiltonian with the same operator
        (double_factorized_hamiltonian.py:224-242)."""
        df = self.to_number_representation()
        u = np.asarray(df.orbital_rotations)
        two_body = np.einsum("kij,kpi,kqi,krj,ksj->pqrs", df.diag_coulomb_mats, u, u.conj(), u, u.conj(),
                             optimize=True)
        one_body = df.one_body_tensor + 0.5 * np.einsum("prrq", two_body)
        return MolecularHamiltonian(one_body, two_body, constant=df.constant)

    def _diag_(self, norb: int, nelec) -> np.ndarray:
        """Diagonal entries, through the molecular form (double_factorized_hamiltonian.py:277-280)."""
        return self.to_molecular_hamiltonian()._diag_(norb, nelec)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, DoubleFactorizedHamiltonian):
            return NotImplemented
        return (self.z_representation == other.z_representation
                and bool(np.isclose(self.constant, other.constant, rtol=rtol, atol=atol))
                and all(bool(np.allclose(a, b, rtol=rtol, atol=atol)) for a, b in [
                    (self.one_body_tensor, other.one_body_tensor),
                    (self.diag_coulomb_mats, other.diag_coulomb_mats),
                    (self.orbital_rotations, other.orbital_rotations)]))

    def _linear_operator_(self, norb: int, nelec) -> LinearOperator:
        """GPU counterpart of double_factorized_hamiltonian.py:244-275 (matvec = rmatvec),
        with a fused FP64 ``expectation``."""
        assert isinstance(nelec, tuple)
        if norb != self.norb:
            raise ValueError(f"the Hamiltonian acts on {self.norb} orbitals, but norb={norb} was given")
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

        def matmat(rows: torch.Tensor) -> torch.Tensor:
            """H on every row of a contiguous (k, dim) tensor: each term once
            over all k states (ffgb_batch_df_matvec)."""
            t = rows.contiguous()
            if t.dtype not in (torch.complex64, torch.complex128):
                t = t.to(torch.complex128)
            out = torch.empty_like(t)
            code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
            k = t.shape[0]
            nbytes = _lib.load().ffgb_batch_scratch_bytes(1, code, norb, n_alpha, n_beta, k)
            buf = torch.empty(nbytes, dtype=torch.uint8, device=t.device)
            _lib.call("ffgb_batch_df_matvec", t.data_ptr(), out.data_ptr(), k, code, norb, n_alpha, n_beta,
                      _lib.dptr(one_body), n_terms, _lib.dptr(dcm), rots.ctypes.data_as(_lib._dp),
                      float(self.constant), int(bool(self.z_representation)), buf.data_ptr(), nbytes, None,
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

        return LinearOperator((d, d), matvec, None, expectation, matmat=matmat)


def _df_z_representation(diag_coulomb_mats, orbital_rotations):
    """One-body and constant corrections between representations
    (double_factorized_hamiltonian.py:306-328)."""
    one_body = 0.5 * (
        np.einsum("tij,tpi,tqi->pq", diag_coulomb_mats, orbital_rotations, orbital_rotations.conj())
        + np.einsum("tij,tpj,tqj->pq", diag_coulomb_mats, orbital_rotations, orbital_rotations.conj())
    )
    constant = 0.25 * np.einsum("ijj->", diag_coulomb_mats) - 0.5 * np.sum(diag_coulomb_mats)
    return one_body, float(constant)


def _exact_double_factorization(one_body, two_body, tol: float = 1e-12):
    r"""An exact double-factorized form of
    :math:`\sum h_{pq} E_{pq} + \frac12 \sum h_{pqrs} a^\dagger_{p\sigma} a^\dagger_{r\tau} a_{s\tau} a_{q\sigma}`
    (:math:`E_{pq} = \sum_\sigma a^\dagger_{p\sigma} a_{q\sigma}`), for two-body
    tensors with the symmetries of molecular integrals, h_pqrs = h_rspq =
    conj(h_qpsr).

    Normal ordering gives sum_pqrs h_pqrs E_pq E_rs / 2 plus the one-body term
    -sum_r h_prrq / 2.  The matrix A[(p, q), (s, r)] = h_pqrs is Hermitian, so
    h_pqrs = sum_t lambda_t L_t[p, q] conj(L_t[s, r]) and
    sum h_pqrs E_pq E_rs = sum_t lambda_t X_t X_t^dag with X_t = sum L_t[p, q] E_pq.
    With L_t = H1 + i H2 (H1, H2 Hermitian) and A_k = sum (H_k)_pq E_pq,
    X X^dag = A_1^2 + A_2^2 + i [A_2, A_1], the commutator a one-body operator
    with matrix i [H2, H1].  Each A_k^2 is (sum_i mu_i n_i)^2 in the eigenbasis U
    of H_k: a diagonal Coulomb term J = lambda mu mu^T with rotation U.
    Returns (one-body tensor, J terms, rotations)."""
    n = one_body.shape[0]
    h = np.asarray(two_body, dtype=complex)
    kappa = np.asarray(one_body, dtype=complex) - 0.5 * np.einsum("prrq->pq", h)
    amat = h.transpose(0, 1, 3, 2).reshape(n * n, n * n)
    amat = (amat + amat.conj().T) / 2
    lam, vecs = np.linalg.eigh(amat)
    scale = max(np.abs(lam).max(), 1.0) if lam.size else 1.0
    mats, rots = [], []
    for t in range(lam.size):
        if abs(lam[t]) <= tol * scale:
            continue
        l_t = vecs[:, t].reshape(n, n)
        h1 = (l_t + l_t.conj().T) / 2
        h2 = (l_t - l_t.conj().T) / 2j
        for hk in (h1, h2):
            if np.abs(hk).max() <= tol:
                continue
            mu, u = np.linalg.eigh(hk)
            mats.append(lam[t] * np.outer(mu, mu))
            rots.append(u)
        kappa = kappa + 0.5 * lam[t] * 1j * (h2 @ h1 - h1 @ h2)
    if not mats:
        return kappa, np.zeros((0, n, n)), np.zeros((0, n, n), dtype=complex)
    return kappa, np.stack(mats), np.stack(rots)


@dataclasses.dataclass(frozen=True)
class MolecularHamiltonian:
    r""":math:`H = \sum h_{pq} a^\dagger_{p\sigma} a_{q\sigma} + \frac12 \sum h_{pqrs}
    a^\dagger_{p\sigma} a^\dagger_{r\tau} a_{s\tau} a_{q\sigma} + \text{constant}`
    (python/ffsim/hamiltonians/molecular_hamiltonian.py:24-60).

    The linear operator (matvec and a fused FP64 ``expectation``) runs the
    exact double-factorized form of the Hamiltonian on the GPU: at most
    2 norb^2 rotated diagonal Coulomb terms.  The reference contracts the
    two-body tensor with double-excitation string links on the CPU
    (contract/two_body.py); the operator is the same."""

    one_body_tensor: np.ndarray
    two_body_tensor: np.ndarray
    constant: float = 0.0

    @property
    def norb(self) -> int:
        return self.one_body_tensor.shape[0]

    def to_double_factorized(self) -> DoubleFactorizedHamiltonian:
        kappa, mats, rots = _exact_double_factorization(self.one_body_tensor, self.two_body_tensor)
        return DoubleFactorizedHamiltonian(kappa, mats, rots, constant=float(self.constant))

    def _linear_operator_(self, norb: int, nelec) -> LinearOperator:
        assert isinstance(nelec, tuple)
        return self.to_double_factorized()._linear_operator_(norb, nelec)

    def rotated(self, orbital_rotation: np.ndarray) -> "MolecularHamiltonian":
        """U H U^dag as a molecular Hamiltonian (molecular_hamiltonian.py:119-144)."""
        from ffsim_gb300.linalg import rotate_one_body_tensor, rotate_two_body_tensor

        return MolecularHamiltonian(rotate_one_body_tensor(self.one_body_tensor, orbital_rotation),
                                    rotate_two_body_tensor(self.two_body_tensor, orbital_rotation, orbital_rotation),
                                    constant=self.constant)

    def _diag_(self, norb: int, nelec) -> np.ndarray:
        """Diagonal entries for real tensors (molecular_hamiltonian.py:175-188).

        In the occupation basis only the Coulomb integrals J_pr = h_pprr and,
        within a spin, the exchange integrals K_pr = h_prrp survive, so the
        diagonal is that of the diagonal Coulomb Hamiltonian with
        J^aa = J - K and J^ab = J, computed on the GPU."""
        if np.iscomplexobj(self.two_body_tensor) or np.iscomplexobj(self.one_body_tensor):
            raise NotImplementedError("Computing diagonal of complex molecular Hamiltonian is not yet supported.")
        h = np.asarray(self.two_body_tensor, dtype=float)
        coulomb = np.einsum("pprr->pr", h)
        exchange = np.einsum("prrp->pr", h)
        dch = DiagonalCoulombHamiltonian(self.one_body_tensor, np.stack([coulomb - exchange, coulomb]),
                                         constant=self.constant)
        return dch._diag_(norb, nelec)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, MolecularHamiltonian):
            return NotImplemented
        return (bool(np.isclose(self.constant, other.constant, rtol=rtol, atol=atol))
                and bool(np.allclose(self.one_body_tensor, other.one_body_tensor, rtol=rtol, atol=atol))
                and bool(np.allclose(self.two_body_tensor, other.two_body_tensor, rtol=rtol, atol=atol)))


@dataclasses.dataclass(frozen=True)
class DiagonalCoulombHamiltonian:
    r""":math:`H = \sum h_{pq} a^\dagger_{p\sigma} a_{q\sigma} + \frac12 \sum
    J^{\sigma\tau}_{pq} n_{p\sigma} n_{q\tau} + \text{constant}` with
    :math:`J^{\alpha\alpha} = J^{\beta\beta}` = ``diag_coulomb_mats[0]`` and
    :math:`J^{\alpha\beta} = J^{\beta\alpha}` = ``diag_coulomb_mats[1]``
    (python/ffsim/hamiltonians/diagonal_coulomb_hamiltonian.py:27-66).

    The linear operator is one rotated number-operator matvec in the eigenbasis
    of h (``ffgb_rotated_diag_matvec``) plus one diagonal Coulomb contraction
    in the occupation basis (``ffgb_contract_diag_coulomb``); the diagonal is
    the same two contractions applied to the all-ones vector."""

    one_body_tensor: np.ndarray
    diag_coulomb_mats: np.ndarray
    constant: float = 0.0

    @property
    def norb(self) -> int:
        return self.one_body_tensor.shape[0]

    def _coulomb_mats(self):
        aa, ab = np.asarray(self.diag_coulomb_mats, dtype=float)
        return aa, ab, aa

    def _linear_operator_(self, norb: int, nelec) -> LinearOperator:
        """GPU counterpart of diagonal_coulomb_hamiltonian.py:67-97 (matvec = rmatvec)."""
        from ffsim_gb300.contract import contract_diag_coulomb, num_op_sum_linop
        from ffsim_gb300.linalg import eigh

        assert isinstance(nelec, tuple)
        d = _dim(norb, nelec)
        eigs, vecs = eigh(np.asarray(self.one_body_tensor, dtype=complex))
        num_linop = num_op_sum_linop(eigs, norb, nelec, orbital_rotation=vecs)
        mats = self._coulomb_mats()
        constant = float(self.constant)

        def matvec(vec: torch.Tensor) -> torch.Tensor:
            t = vec.contiguous()
            if t.dtype not in (torch.complex64, torch.complex128):
                t = t.to(torch.complex128)
            out = num_linop @ t
            out += contract_diag_coulomb(t, mats, norb, nelec)
            if constant:
                out += constant * t
            return out

        return LinearOperator((d, d), matvec, matvec)

    def _diag_(self, norb: int, nelec) -> np.ndarray:
        """Diagonal entries (diagonal_coulomb_hamiltonian.py:208-238), as a host
        FP64 array like the reference's."""
        from ffsim_gb300.contract import contract_diag_coulomb, contract_num_op_sum

        assert isinstance(nelec, tuple)
        ones = torch.ones(_dim(norb, nelec), dtype=torch.complex128, device="cuda")
        h = np.real(np.diag(np.asarray(self.one_body_tensor))).astype(float)
        out = contract_num_op_sum(ones, h, norb, nelec)
        out += contract_diag_coulomb(ones, self._coulomb_mats(), norb, nelec)
        return out.real.cpu().numpy() + float(self.constant)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, DiagonalCoulombHamiltonian):
            return NotImplemented
        return (bool(np.isclose(self.constant, other.constant, rtol=rtol, atol=atol))
                and bool(np.allclose(self.one_body_tensor, other.one_body_tensor, rtol=rtol, atol=atol))
                and bool(np.allclose(self.diag_coulomb_mats, other.diag_coulomb_mats, rtol=rtol, atol=atol)))
