"""Spin-balanced unitary cluster Jastrow operator
(python/ffsim/variational/ucj_spin_balanced.py) with a GPU ``_apply_unitary_``."""

from __future__ import annotations

import itertools
from dataclasses import InitVar, dataclass

import numpy as np

from ffsim_gb300 import _lib, linalg
from ffsim_gb300._state import prepare, scratch, split_nelec, stream_ptr


def validate_interaction_pairs(interaction_pairs, ordered: bool) -> None:
    """No duplicates; unordered (same-spin or spinless) pairs must be upper
    triangular (python/ffsim/variational/util.py:19-35)."""
    if interaction_pairs is None:
        return
    if len(set(interaction_pairs)) != len(interaction_pairs):
        raise ValueError(f"Duplicate interaction pairs encountered: {interaction_pairs}.")
    if not ordered:
        for i, j in interaction_pairs:
            if i > j:
                raise ValueError(
                    "When specifying spinless, alpha-alpha or beta-beta interaction pairs, you must provide "
                    f"only upper triangular pairs. Got {(i, j)}, which is a lower triangular pair.")


def _check_norb(own: int, norb: int) -> None:
    if own != norb:
        raise ValueError(f"the operator acts on {own} orbitals, but norb={norb} was given")


def orbital_rotation_from_t1_amplitudes(t1: np.ndarray) -> np.ndarray:
    """exp(t1 - t1^dag) embedded in the occupied-virtual block
    (python/ffsim/variational/util.py:38-54)."""
    import scipy.linalg

    t1 = np.asarray(t1)
    nocc, nvrt = t1.shape
    norb = nocc + nvrt
    gen = np.zeros((norb, norb), dtype=t1.dtype)
    gen[:nocc, nocc:] = -t1.conj()
    gen[nocc:, :nocc] = t1.T
    return scipy.linalg.expm(gen)


def interaction_pairs_spin_balanced(connectivity: str, norb: int):
    """Alpha-alpha and alpha-beta interaction pairs of a qubit layout
    (python/ffsim/variational/util.py:57-75): all-to-all (no restriction),
    square (a chain plus every ab on-site pair), hex (on-site every second
    orbital), heavy-hex (every fourth)."""
    if connectivity == "all-to-all":
        return None, None
    chain = [(p, p + 1) for p in range(norb - 1)]
    stride = {"square": 1, "hex": 2, "heavy-hex": 4}.get(connectivity)
    if stride is None:
        raise ValueError(f"Invalid connectivity: {connectivity}")
    return chain, [(p, p) for p in range(0, norb, stride)]


def _triu(norb: int) -> list:
    return list(itertools.combinations_with_replacement(range(norb), 2))


def _put(mat, pairs, vals, symmetric: bool) -> None:
    """Write vals at the pairs (and their mirror when symmetric)."""
    if not pairs:
        return
    rows, cols = zip(*pairs)
    if symmetric:
        mat[cols, rows] = vals
    mat[rows, cols] = vals


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
    def n_params(norb: int, n_reps: int, *, interaction_pairs=None,
                 with_final_orbital_rotation: bool = False) -> int:
        """ucj_spin_balanced.py:149-195.  ``interaction_pairs`` = (aa pairs, ab
        pairs), each upper triangular or None (all pairs)."""
        pairs_aa, pairs_ab = interaction_pairs if interaction_pairs is not None else (None, None)
        validate_interaction_pairs(pairs_aa, ordered=False)
        validate_interaction_pairs(pairs_ab, ordered=False)
        n_triu = norb * (norb + 1) // 2
        n_aa = n_triu if pairs_aa is None else len(pairs_aa)
        n_ab = n_triu if pairs_ab is None else len(pairs_ab)
        return n_reps * (n_aa + n_ab + norb**2) + with_final_orbital_rotation * norb**2

    @staticmethod
    def from_parameters(params: np.ndarray, *, norb: int, n_reps: int, interaction_pairs=None,
                        with_final_orbital_rotation: bool = False) -> "UCJOpSpinBalanced":
        """ucj_spin_balanced.py:197-293: per rep, the orbital rotation's norb**2
        parameters, then the aa and the ab entries at their pairs (both matrices
        symmetric); then the final rotation."""
        params = _check_params(params, UCJOpSpinBalanced.n_params(
            norb, n_reps, interaction_pairs=interaction_pairs,
            with_final_orbital_rotation=with_final_orbital_rotation))
        pairs_aa, pairs_ab = interaction_pairs if interaction_pairs is not None else (None, None)
        pairs = [_triu(norb) if pairs_aa is None else pairs_aa, _triu(norb) if pairs_ab is None else pairs_ab]
        dcm = np.zeros((n_reps, 2, norb, norb))
        rots = np.zeros((n_reps, norb, norb), dtype=complex)
        index = 0
        for r in range(n_reps):
            rots[r] = linalg.unitary_from_parameters(params[index: index + norb**2], norb)
            index += norb**2
            for t in range(2):
                _put(dcm[r, t], pairs[t], params[index: index + len(pairs[t])], True)
                index += len(pairs[t])
        final = None
        if with_final_orbital_rotation:
            final = linalg.unitary_from_parameters(params[index:], norb)
        return UCJOpSpinBalanced(dcm, rots, final)

    @staticmethod
    def from_t_amplitudes(t2: np.ndarray, *, t1: np.ndarray | None = None, n_reps: int | None = None,
                          interaction_pairs=None, tol: float = 1e-8, optimize: bool = False,
                          method: str = "L-BFGS-B", callback=None, options: dict | None = None,
                          regularization: float = 0, multi_stage_start: int | None = None,
                          multi_stage_step: int | None = None) -> "UCJOpSpinBalanced":
        """UCJ operator from (CCSD) t2 and optional t1 amplitudes
        (ucj_spin_balanced.py:377-532): the t2 double factorization gives one
        layer per term (the same matrix for aa and ab), padded with identity
        layers up to ``n_reps``; t1 gives the final rotation exp(t1 - t1^dag);
        entries outside the interaction pairs are zeroed."""
        if isinstance(n_reps, int) and n_reps <= 0:
            raise ValueError(f"n_reps must be at least 1. Got {n_reps}.")
        pairs_aa, pairs_ab = (None, None) if interaction_pairs is None else interaction_pairs
        validate_interaction_pairs(pairs_aa, ordered=False)
        validate_interaction_pairs(pairs_ab, ordered=False)
        nocc, _, nvrt, _ = np.asarray(t2).shape
        norb = nocc + nvrt
        indices = None
        if pairs_aa is not None or pairs_ab is not None:
            indices = list(set((pairs_aa or []) + (pairs_ab or [])))
        mats, rots = linalg.double_factorized_t2(
            t2, tol=tol, max_terms=n_reps, optimize=optimize, method=method, callback=callback, options=options,
            diag_coulomb_indices=indices, regularization=regularization, multi_stage_start=multi_stage_start,
            multi_stage_step=multi_stage_step)
        dcm = np.stack([mats, mats], axis=1)
        if n_reps is not None and dcm.shape[0] < n_reps:
            pad = n_reps - dcm.shape[0]
            dcm = np.concatenate([dcm, np.zeros((pad, 2, norb, norb))])
            rots = np.concatenate([rots, np.stack([np.eye(norb)] * pad)])
        final = orbital_rotation_from_t1_amplitudes(t1) if t1 is not None else None
        for t, pairs in enumerate((pairs_aa, pairs_ab)):
            if pairs is not None:
                mask = np.zeros((norb, norb), dtype=bool)
                if pairs:
                    rows, cols = zip(*pairs)
                    mask[rows, cols] = True
                    mask[cols, rows] = True
                dcm[:, t] *= mask
        return UCJOpSpinBalanced(dcm, rots, final)

    def to_parameters(self, *, interaction_pairs=None) -> np.ndarray:
        """ucj_spin_balanced.py:295-374."""
        norb = self.norb
        pairs_aa, pairs_ab = interaction_pairs if interaction_pairs is not None else (None, None)
        validate_interaction_pairs(pairs_aa, ordered=False)
        validate_interaction_pairs(pairs_ab, ordered=False)
        pairs = [_triu(norb) if pairs_aa is None else pairs_aa, _triu(norb) if pairs_ab is None else pairs_ab]
        out = []
        for u, mats in zip(self.orbital_rotations, self.diag_coulomb_mats):
            out.append(linalg.unitary_to_parameters(u))
            for t in range(2):
                if pairs[t]:
                    out.append(mats[t][tuple(zip(*pairs[t]))])
        if self.final_orbital_rotation is not None:
            out.append(linalg.unitary_to_parameters(self.final_orbital_rotation))
        return np.concatenate(out)

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        """GPU counterpart of ucj_spin_balanced.py:657-696: for each rep, the
        merged rotation U_k^dag U_{k-1} then exp(-i(-1) J_k), then the final rotation."""
        if isinstance(nelec, (int, np.integer)):
            return NotImplemented
        _check_norb(self.norb, norb)
        n_alpha, n_beta = split_nelec(nelec)
        p = prepare(vec, norb, nelec, copy=copy)
        dcm = _lib.rmat(self.diag_coulomb_mats, (self.n_reps, 2, norb, norb), "diag_coulomb_mats")
        rots = _lib.cmat(self.orbital_rotations, (self.n_reps, norb, norb), "orbital_rotations")
        final = _lib.cmat(self.final_orbital_rotation, (norb, norb), "final_orbital_rotation")
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


def _check_params(params, n: int) -> np.ndarray:
    params = np.asarray(params, dtype=float)
    if len(params) != n:
        raise ValueError(
            "The number of parameters passed did not match the number expected based on the "
            f"function inputs. Expected {n} but got {len(params)}.")
    return params


def _allclose_or_none(a, b, rtol, atol) -> bool:
    if (a is None) != (b is None):
        return False
    return a is None or bool(np.allclose(a, b, rtol=rtol, atol=atol))


@dataclass(frozen=True)
class UCJOpSpinUnbalanced:
    r"""Spin-unbalanced UCJ operator: per repetition an orbital rotation for each
    spin and diagonal Coulomb matrices [aa, ab, bb] (ucj_spin_unbalanced.py:28-141).
    ``_apply_unitary_`` composes the GPU gates as the reference does
    (ucj_spin_unbalanced.py:705-745)."""

    diag_coulomb_mats: np.ndarray  # (n_reps, 3, norb, norb): [aa, ab, bb]
    orbital_rotations: np.ndarray  # (n_reps, 2, norb, norb): [alpha, beta]
    final_orbital_rotation: np.ndarray | None = None  # (2, norb, norb)
    validate: InitVar[bool] = True
    rtol: InitVar[float] = 1e-5
    atol: InitVar[float] = 1e-8

    def __post_init__(self, validate: bool, rtol: float, atol: float):
        if not validate:
            return
        if self.diag_coulomb_mats.ndim != 4 or self.diag_coulomb_mats.shape[1] != 3:
            raise ValueError(
                "diag_coulomb_mats should have shape (n_reps, 3, norb, norb). "
                f"Got shape {self.diag_coulomb_mats.shape}.")
        if self.orbital_rotations.ndim != 4 or self.orbital_rotations.shape[1] != 2:
            raise ValueError(
                "orbital_rotations should have shape (n_reps, 2, norb, norb). "
                f"Got shape {self.orbital_rotations.shape}.")
        if self.final_orbital_rotation is not None and self.final_orbital_rotation.ndim != 3:
            raise ValueError(
                "final_orbital_rotation should have shape (2, norb, norb). "
                f"Got shape {self.final_orbital_rotation.shape}.")
        if self.diag_coulomb_mats.shape[0] != self.orbital_rotations.shape[0]:
            raise ValueError(
                "diag_coulomb_mats and orbital_rotations should have the same first dimension. "
                f"Got {self.diag_coulomb_mats.shape[0]} and {self.orbital_rotations.shape[0]}.")
        if not all(linalg.is_real_symmetric(m[0], rtol=rtol, atol=atol)
                   and linalg.is_real_symmetric(m[2], rtol=rtol, atol=atol) for m in self.diag_coulomb_mats):
            raise ValueError("alpha-alpha and beta-beta diagonal Coulomb matrices were not all real symmetric.")
        if not all(linalg.is_unitary(u[0], rtol=rtol, atol=atol) and linalg.is_unitary(u[1], rtol=rtol, atol=atol)
                   for u in self.orbital_rotations):
            raise ValueError("Orbital rotations were not all unitary.")
        if self.final_orbital_rotation is not None and not (
                linalg.is_unitary(self.final_orbital_rotation[0], rtol=rtol, atol=atol)
                and linalg.is_unitary(self.final_orbital_rotation[1], rtol=rtol, atol=atol)):
            raise ValueError("Final orbital rotation was not unitary.")

    @property
    def norb(self) -> int:
        return self.diag_coulomb_mats.shape[-1]

    @property
    def n_reps(self) -> int:
        return self.diag_coulomb_mats.shape[0]

    @staticmethod
    def _pairs(norb: int, interaction_pairs):
        pairs_aa, pairs_ab, pairs_bb = interaction_pairs if interaction_pairs is not None else (None, None, None)
        validate_interaction_pairs(pairs_aa, ordered=False)
        validate_interaction_pairs(pairs_ab, ordered=True)
        validate_interaction_pairs(pairs_bb, ordered=False)
        full = list(itertools.product(range(norb), repeat=2))
        return [_triu(norb) if pairs_aa is None else pairs_aa, full if pairs_ab is None else pairs_ab,
                _triu(norb) if pairs_bb is None else pairs_bb]

    @staticmethod
    def n_params(norb: int, n_reps: int, *, interaction_pairs=None,
                 with_final_orbital_rotation: bool = False) -> int:
        """ucj_spin_unbalanced.py:146-206.  ``interaction_pairs`` = (aa, ab, bb);
        aa and bb upper triangular, ab ordered; None means all pairs."""
        pairs = UCJOpSpinUnbalanced._pairs(norb, interaction_pairs)
        return n_reps * (sum(len(x) for x in pairs) + 2 * norb**2) + with_final_orbital_rotation * 2 * norb**2

    @staticmethod
    def from_parameters(params: np.ndarray, *, norb: int, n_reps: int, interaction_pairs=None,
                        with_final_orbital_rotation: bool = False) -> "UCJOpSpinUnbalanced":
        """ucj_spin_unbalanced.py:208-329: per rep the alpha and beta rotations
        (norb**2 each), then the aa, ab and bb entries at their pairs (aa, bb
        symmetric); then the final rotations."""
        params = _check_params(params, UCJOpSpinUnbalanced.n_params(
            norb, n_reps, interaction_pairs=interaction_pairs,
            with_final_orbital_rotation=with_final_orbital_rotation))
        pairs = UCJOpSpinUnbalanced._pairs(norb, interaction_pairs)
        dcm = np.zeros((n_reps, 3, norb, norb))
        rots = np.zeros((n_reps, 2, norb, norb), dtype=complex)
        i = 0
        for r in range(n_reps):
            for sp in range(2):
                rots[r, sp] = linalg.unitary_from_parameters(params[i: i + norb**2], norb)
                i += norb**2
            for t in range(3):
                _put(dcm[r, t], pairs[t], params[i: i + len(pairs[t])], t != 1)
                i += len(pairs[t])
        final = None
        if with_final_orbital_rotation:
            final = np.stack([linalg.unitary_from_parameters(params[i + sp * norb**2: i + (sp + 1) * norb**2], norb)
                              for sp in range(2)])
        return UCJOpSpinUnbalanced(dcm, rots, final)

    def to_parameters(self, interaction_pairs=None) -> np.ndarray:
        """ucj_spin_unbalanced.py:331-432."""
        pairs = UCJOpSpinUnbalanced._pairs(self.norb, interaction_pairs)
        out = []
        for u, mats in zip(self.orbital_rotations, self.diag_coulomb_mats):
            out += [linalg.unitary_to_parameters(u[0]), linalg.unitary_to_parameters(u[1])]
            out += [mats[t][tuple(zip(*pairs[t]))] for t in range(3) if pairs[t]]
        if self.final_orbital_rotation is not None:
            out += [linalg.unitary_to_parameters(u) for u in self.final_orbital_rotation]
        return np.concatenate(out)

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        from ffsim_gb300.gates import apply_diag_coulomb_evolution, apply_orbital_rotation

        if isinstance(nelec, (int, np.integer)):
            return NotImplemented
        p = prepare(vec, norb, nelec, copy=copy)
        state = p.tensor.reshape(-1)
        eye = np.eye(norb, dtype=complex)
        basis = (eye, eye)
        for mats, rot in zip(self.diag_coulomb_mats, self.orbital_rotations):
            state = apply_orbital_rotation(state, (rot[0].conj().T @ basis[0], rot[1].conj().T @ basis[1]), norb,
                                           nelec, copy=False)
            state = apply_diag_coulomb_evolution(state, (mats[0], mats[1], mats[2]), -1.0, norb, nelec, copy=False)
            basis = (rot[0], rot[1])
        if self.final_orbital_rotation is not None:
            basis = (self.final_orbital_rotation[0] @ basis[0], self.final_orbital_rotation[1] @ basis[1])
        state = apply_orbital_rotation(state, basis, norb, nelec, copy=False)
        if state.data_ptr() != p.tensor.data_ptr():
            p.tensor.reshape(-1).copy_(state)
        return p.finish()

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, UCJOpSpinUnbalanced):
            return NotImplemented
        return (bool(np.allclose(self.diag_coulomb_mats, other.diag_coulomb_mats, rtol=rtol, atol=atol))
                and bool(np.allclose(self.orbital_rotations, other.orbital_rotations, rtol=rtol, atol=atol))
                and _allclose_or_none(self.final_orbital_rotation, other.final_orbital_rotation, rtol, atol))


@dataclass(frozen=True)
class UCJOpSpinless:
    r"""Spinless UCJ operator: per repetition one orbital rotation and one
    diagonal Coulomb matrix (ucj_spinless.py:28-120).  On spinful states the
    matrix acts within each spin, (J, 0, J) (ucj_spinless.py:456-515)."""

    diag_coulomb_mats: np.ndarray  # (n_reps, norb, norb)
    orbital_rotations: np.ndarray  # (n_reps, norb, norb)
    final_orbital_rotation: np.ndarray | None = None  # (norb, norb)
    validate: InitVar[bool] = True
    rtol: InitVar[float] = 1e-5
    atol: InitVar[float] = 1e-8

    def __post_init__(self, validate: bool, rtol: float, atol: float):
        if not validate:
            return
        if self.diag_coulomb_mats.ndim != 3:
            raise ValueError(
                "diag_coulomb_mats should have shape (n_reps, norb, norb). "
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
        if not all(linalg.is_real_symmetric(m, rtol=rtol, atol=atol) for m in self.diag_coulomb_mats):
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
    def n_params(norb: int, n_reps: int, *, interaction_pairs=None,
                 with_final_orbital_rotation: bool = False) -> int:
        """ucj_spinless.py:133-172 (``interaction_pairs``: upper triangular, or None for all)."""
        validate_interaction_pairs(interaction_pairs, ordered=False)
        n_pairs = norb * (norb + 1) // 2 if interaction_pairs is None else len(interaction_pairs)
        return n_reps * (n_pairs + norb**2) + with_final_orbital_rotation * norb**2

    @staticmethod
    def from_parameters(params: np.ndarray, *, norb: int, n_reps: int, interaction_pairs=None,
                        with_final_orbital_rotation: bool = False) -> "UCJOpSpinless":
        """ucj_spinless.py:174-262: per rep the rotation's norb**2 parameters,
        then the (symmetric) matrix entries at the pairs."""
        params = _check_params(params, UCJOpSpinless.n_params(
            norb, n_reps, interaction_pairs=interaction_pairs,
            with_final_orbital_rotation=with_final_orbital_rotation))
        pairs = _triu(norb) if interaction_pairs is None else interaction_pairs
        dcm = np.zeros((n_reps, norb, norb))
        rots = np.zeros((n_reps, norb, norb), dtype=complex)
        i = 0
        for r in range(n_reps):
            rots[r] = linalg.unitary_from_parameters(params[i: i + norb**2], norb)
            i += norb**2
            _put(dcm[r], pairs, params[i: i + len(pairs)], True)
            i += len(pairs)
        final = linalg.unitary_from_parameters(params[i:], norb) if with_final_orbital_rotation else None
        return UCJOpSpinless(dcm, rots, final)

    def to_parameters(self, *, interaction_pairs=None) -> np.ndarray:
        """ucj_spinless.py:264-324."""
        validate_interaction_pairs(interaction_pairs, ordered=False)
        pairs = _triu(self.norb) if interaction_pairs is None else interaction_pairs
        out = []
        for u, m in zip(self.orbital_rotations, self.diag_coulomb_mats):
            out.append(linalg.unitary_to_parameters(u))
            if pairs:
                out.append(m[tuple(zip(*pairs))])
        if self.final_orbital_rotation is not None:
            out.append(linalg.unitary_to_parameters(self.final_orbital_rotation))
        return np.concatenate(out)

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        from ffsim_gb300.gates import apply_diag_coulomb_evolution, apply_orbital_rotation

        p = prepare(vec, norb, nelec, copy=copy)
        state = p.tensor.reshape(-1)
        spinless = isinstance(nelec, (int, np.integer))
        zero = np.zeros((norb, norb))
        basis = np.eye(norb, dtype=complex)
        for mat, rot in zip(self.diag_coulomb_mats, self.orbital_rotations):
            state = apply_orbital_rotation(state, rot.conj().T @ basis, norb, nelec, copy=False)
            state = apply_diag_coulomb_evolution(state, mat if spinless else (mat, zero, mat), -1.0, norb, nelec,
                                                 copy=False)
            basis = rot
        if self.final_orbital_rotation is not None:
            basis = self.final_orbital_rotation @ basis
        state = apply_orbital_rotation(state, basis, norb, nelec, copy=False)
        if state.data_ptr() != p.tensor.data_ptr():
            p.tensor.reshape(-1).copy_(state)
        return p.finish()

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, UCJOpSpinless):
            return NotImplemented
        return (bool(np.allclose(self.diag_coulomb_mats, other.diag_coulomb_mats, rtol=rtol, atol=atol))
                and bool(np.allclose(self.orbital_rotations, other.orbital_rotations, rtol=rtol, atol=atol))
                and _allclose_or_none(self.final_orbital_rotation, other.final_orbital_rotation, rtol, atol))


def _brickwork(pairs, thetas, phis, norb):
    """Place a Givens sequence in a full brickwork of adjacent rotations
    (python/ffsim/variational/givens.py:229-300): ceil(norb/2) layers on the
    pairs (0,1),(2,3),... alternate with floor(norb/2) layers on (1,2),(3,4),...;
    each rotation goes in the earliest layer of its kind after every earlier
    rotation on its orbitals (an odd-layer slot k follows even layer k); unused
    slots keep angle 0."""
    q, r = divmod(norb, 2)
    even = [[((i, i + 1), 0.0, 0.0) for i in range(0, norb - 1, 2)] for _ in range(q + r)]
    odd = [[((i, i + 1), 0.0, 0.0) for i in range(1, norb - 1, 2)] for _ in range(q)]
    last_even, last_odd = [-1] * norb, [-1] * norb
    for (i, j), theta, phi in zip(pairs, thetas, phis):
        if i > j:
            i, j, theta, phi = j, i, -theta, -phi
        if i % 2 == 0:
            k = max(last_even[i], last_even[j], last_odd[i], last_odd[j]) + 1
            even[k][i // 2] = ((i, j), theta, phi)
            last_even[i] = last_even[j] = k
        else:
            k = max(last_odd[i] + 1, last_odd[j] + 1, last_even[i], last_even[j])
            odd[k][i // 2] = ((i, j), theta, phi)
            last_odd[i] = last_odd[j] = k
    out = [g for e, o in itertools.zip_longest(even, odd, fillvalue=()) for g in (*e, *o)]
    return [g[0] for g in out], [g[1] for g in out], [g[2] for g in out]


@dataclass(frozen=True)
class GivensAnsatzOp:
    r"""Givens rotation ansatz (python/ffsim/variational/givens.py:29-227): a
    product of Givens rotations on ``interaction_pairs`` with angles ``thetas``
    and optional phases ``phis``, after an optional layer of orbital phases.
    It is an orbital rotation, so ``_apply_unitary_`` is one
    ``ffgb_apply_orbital_rotation``."""

    norb: int
    interaction_pairs: list
    thetas: np.ndarray
    phis: np.ndarray | None
    phase_angles: np.ndarray | None

    @staticmethod
    def n_params(norb: int, interaction_pairs, with_phis: bool = True, with_phase_angles: bool = True) -> int:
        return (1 + with_phis) * len(interaction_pairs) + with_phase_angles * norb

    def to_parameters(self) -> np.ndarray:
        parts = [self.thetas] + [x for x in (self.phis, self.phase_angles) if x is not None]
        return np.concatenate(parts) if len(parts) > 1 else self.thetas

    @staticmethod
    def from_parameters(params: np.ndarray, norb: int, interaction_pairs, with_phis: bool = True,
                        with_phase_angles: bool = True) -> "GivensAnsatzOp":
        params = _check_params(params, GivensAnsatzOp.n_params(norb, interaction_pairs, with_phis,
                                                               with_phase_angles))
        n = len(interaction_pairs)
        thetas = params[:n]
        phis = params[n: 2 * n] if with_phis else None
        phase_angles = params[(2 if with_phis else 1) * n:] if with_phase_angles else None
        return GivensAnsatzOp(norb, interaction_pairs, thetas, phis, phase_angles)

    @staticmethod
    def from_orbital_rotation(orbital_rotation: np.ndarray) -> "GivensAnsatzOp":
        """From the Givens decomposition of the rotation, laid out in a brickwork
        (givens.py:154-178)."""
        norb = orbital_rotation.shape[0]
        rots, phases = linalg.givens_decomposition(orbital_rotation)
        pairs = [(i, j) for _, _, i, j in rots]
        thetas = [float(np.arctan2(abs(s), c)) for c, s, _, _ in rots]
        phis = [float(np.angle(s)) for _, s, _, _ in rots]
        pairs, thetas, phis = _brickwork(pairs, thetas, phis, norb)
        return GivensAnsatzOp(norb, pairs, np.array(thetas), np.array(phis), np.angle(phases))

    def to_orbital_rotation(self) -> np.ndarray:
        """diag(exp(i phase_angles)) times the rotations, last pair first, each
        on columns (j, i): col_j <- c col_j + s col_i, col_i <- c col_i - conj(s) col_j
        with c = cos(theta), s = sin(theta) exp(-i phi) (givens.py:180-198)."""
        phis = np.zeros(len(self.interaction_pairs)) if self.phis is None else self.phis
        angles = np.zeros(self.norb) if self.phase_angles is None else self.phase_angles
        mat = np.diag(np.exp(1j * np.asarray(angles, dtype=float)))
        for (i, j), theta, phi in zip(self.interaction_pairs[::-1], self.thetas[::-1], phis[::-1]):
            c, s = np.cos(theta), np.sin(theta) * np.exp(-1j * phi)
            cj, ci = mat[:, j].copy(), mat[:, i].copy()
            mat[:, j] = c * cj + s * ci
            mat[:, i] = c * ci - np.conj(s) * cj
        return mat

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        from ffsim_gb300.gates import apply_orbital_rotation

        return apply_orbital_rotation(vec, self.to_orbital_rotation(), norb, nelec, copy=copy)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, GivensAnsatzOp):
            return NotImplemented
        if self.norb != other.norb or list(self.interaction_pairs) != list(other.interaction_pairs):
            return False
        return (bool(np.allclose(self.thetas, other.thetas, rtol=rtol, atol=atol))
                and _allclose_or_none(self.phis, other.phis, rtol, atol)
                and _allclose_or_none(self.phase_angles, other.phase_angles, rtol, atol))


@dataclass(frozen=True)
class NumNumAnsatzOpSpinBalanced:
    """Number-number interactions exp(i theta n_p n_q) on given same-spin and
    opposite-spin orbital pairs (python/ffsim/variational/num_num.py:42-193).
    Applying it is one diagonal Coulomb evolution with the matrices
    (J_aa, J_ab, J_aa) of the angles and time -1."""

    norb: int
    interaction_pairs: tuple
    thetas: tuple

    def __post_init__(self):
        for pairs, angles in zip(self.interaction_pairs, self.thetas):
            validate_interaction_pairs(pairs, ordered=False)
            if len(pairs) != len(angles):
                raise ValueError("The number of interaction pairs must be equal to the number of rotation angles."
                                 f"Got {len(pairs)}, and {len(angles)}.")

    @staticmethod
    def n_params(interaction_pairs) -> int:
        return sum(len(pairs) for pairs in interaction_pairs)

    def to_parameters(self) -> np.ndarray:
        return np.concatenate(self.thetas)

    @staticmethod
    def from_parameters(params: np.ndarray, norb: int, interaction_pairs) -> "NumNumAnsatzOpSpinBalanced":
        pairs_aa, pairs_ab = interaction_pairs
        params = _check_params(params, len(pairs_aa) + len(pairs_ab))
        return NumNumAnsatzOpSpinBalanced(norb, (pairs_aa, pairs_ab),
                                          (params[: len(pairs_aa)], params[len(pairs_aa):]))

    @staticmethod
    def from_diag_coulomb_mats(diag_coulomb_mats) -> "NumNumAnsatzOpSpinBalanced":
        """The pairs with a nonzero upper-triangle entry, in row-major order."""
        mat_aa, mat_ab = diag_coulomb_mats
        norb = mat_aa.shape[0]
        pairs, thetas = ([], []), ([], [])
        for t, mat in enumerate((mat_aa, mat_ab)):
            for i, j in itertools.combinations_with_replacement(range(norb), 2):
                if mat[i, j]:
                    pairs[t].append((i, j))
                    thetas[t].append(mat[i, j])
        return NumNumAnsatzOpSpinBalanced(norb, pairs, (np.array(thetas[0]), np.array(thetas[1])))

    def to_diag_coulomb_mats(self) -> np.ndarray:
        mats = np.zeros((2, self.norb, self.norb))
        for mat, pairs, thetas in zip(mats, self.interaction_pairs, self.thetas):
            for (i, j), theta in zip(pairs, thetas):
                mat[i, j] = mat[j, i] = theta
        return mats

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        from ffsim_gb300 import gates

        if isinstance(nelec, (int, np.integer)):
            return NotImplemented
        _check_norb(self.norb, norb)
        aa, ab = self.to_diag_coulomb_mats()
        return gates.apply_diag_coulomb_evolution(vec, (aa, ab, aa), -1.0, norb, nelec, copy=copy)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, NumNumAnsatzOpSpinBalanced):
            return NotImplemented
        return (self.norb == other.norb and list(map(list, self.interaction_pairs)) == list(
                    map(list, other.interaction_pairs))
                and all(bool(np.allclose(a, b, rtol=rtol, atol=atol)) for a, b in zip(self.thetas, other.thetas)))


@dataclass(frozen=True)
class HopGateAnsatzOperator:
    """Hop gates on a cycle of orbital pairs, one angle each, then an optional
    final orbital rotation (python/ffsim/variational/hopgate.py:27-137)."""

    norb: int
    interaction_pairs: list
    thetas: np.ndarray
    final_orbital_rotation: np.ndarray | None = None

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        from ffsim_gb300 import basic_gates, gates

        _check_norb(self.norb, norb)
        first = True
        for target_orbs, theta in zip(itertools.cycle(self.interaction_pairs), self.thetas):
            vec = basic_gates.apply_hop_gate(vec, theta, target_orbs, norb, nelec, copy=copy and first)
            first = False
        if self.final_orbital_rotation is not None:
            vec = gates.apply_orbital_rotation(vec, self.final_orbital_rotation, norb, nelec, copy=copy and first)
            first = False
        if first and copy:
            vec = vec.clone() if hasattr(vec, "clone") else np.array(vec, copy=True)
        return vec

    def to_parameters(self) -> np.ndarray:
        parts = [np.asarray(self.thetas, dtype=float)]
        if self.final_orbital_rotation is not None:
            parts.append(linalg.unitary_to_parameters(self.final_orbital_rotation))
        return np.concatenate(parts)

    @staticmethod
    def from_parameters(params: np.ndarray, norb: int, interaction_pairs,
                        with_final_orbital_rotation: bool = False) -> "HopGateAnsatzOperator":
        params = np.asarray(params, dtype=float)
        final = None
        if with_final_orbital_rotation:
            final = linalg.unitary_from_parameters(params[-(norb**2):], norb)
            params = params[: -(norb**2)]
        return HopGateAnsatzOperator(norb, interaction_pairs, params, final)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        if not isinstance(other, HopGateAnsatzOperator):
            return NotImplemented
        return (self.norb == other.norb and list(self.interaction_pairs) == list(other.interaction_pairs)
                and bool(np.allclose(self.thetas, other.thetas, rtol=rtol, atol=atol))
                and _allclose_or_none(self.final_orbital_rotation, other.final_orbital_rotation, rtol, atol))


def brickwork(norb: int, n_layers: int):
    """Adjacent pairs layer by layer, (0,1),(2,3),... then (1,2),(3,4),...
    (python/ffsim/variational/ucj_angles_spin_balanced.py:247-250)."""
    for i in range(n_layers):
        for j in range(i % 2, norb - 1, 2):
            yield (j, j + 1)


@dataclass(frozen=True)
class UCJAnglesOpSpinBalanced:
    """Spin-balanced UCJ operator parameterized by gate angles
    (python/ffsim/variational/ucj_angles_spin_balanced.py:26-244): per
    repetition a Givens-ansatz orbital rotation and a number-number ansatz,
    then an optional final Givens-ansatz rotation.  Applied like the matrix
    form: consecutive rotations merged into one orbital rotation on the GPU."""

    norb: int
    num_num_ansatz_ops: list
    givens_ansatz_ops: list
    final_givens_ansatz_op: "GivensAnsatzOp | None" = None

    def __post_init__(self):
        if len(self.num_num_ansatz_ops) != len(self.givens_ansatz_ops):
            raise ValueError("The number of number-number ansatz operations must equal the number of Givens ansatz "
                             f"operations. Got {len(self.num_num_ansatz_ops)} and {len(self.givens_ansatz_ops)}.")

    @property
    def n_reps(self) -> int:
        return len(self.num_num_ansatz_ops)

    @staticmethod
    def n_params(norb: int, n_reps: int, num_num_interaction_pairs, givens_interaction_pairs,
                 with_final_givens_ansatz_op: bool = False) -> int:
        per_rep = sum(len(p) for p in num_num_interaction_pairs) + 2 * len(givens_interaction_pairs) + norb
        return n_reps * per_rep + with_final_givens_ansatz_op * norb**2

    @staticmethod
    def from_parameters(params: np.ndarray, *, norb: int, n_reps: int, num_num_interaction_pairs,
                        givens_interaction_pairs, with_final_givens_ansatz_op: bool = False
                        ) -> "UCJAnglesOpSpinBalanced":
        """Per repetition the Givens ansatz's 2 len(pairs) + norb parameters,
        then the number-number angles; then the final brickwork Givens ansatz."""
        params = _check_params(params, UCJAnglesOpSpinBalanced.n_params(
            norb, n_reps, num_num_interaction_pairs, givens_interaction_pairs, with_final_givens_ansatz_op))
        n_nn = sum(len(p) for p in num_num_interaction_pairs)
        n_giv = 2 * len(givens_interaction_pairs) + norb
        nn_ops, giv_ops, index = [], [], 0
        for _ in range(n_reps):
            giv_ops.append(GivensAnsatzOp.from_parameters(params[index: index + n_giv], norb,
                                                          givens_interaction_pairs))
            index += n_giv
            nn_ops.append(NumNumAnsatzOpSpinBalanced.from_parameters(params[index: index + n_nn], norb,
                                                                     num_num_interaction_pairs))
            index += n_nn
        final = None
        if with_final_givens_ansatz_op:
            final = GivensAnsatzOp.from_parameters(params[index:], norb, list(brickwork(norb, norb)))
        return UCJAnglesOpSpinBalanced(norb, nn_ops, giv_ops, final)

    def to_parameters(self) -> np.ndarray:
        parts = []
        for giv, nn in zip(self.givens_ansatz_ops, self.num_num_ansatz_ops):
            parts += [giv.to_parameters(), nn.to_parameters()]
        if self.final_givens_ansatz_op is not None:
            parts.append(self.final_givens_ansatz_op.to_parameters())
        return np.concatenate(parts)

    @staticmethod
    def from_ucj_op(ucj_op: UCJOpSpinBalanced) -> "UCJAnglesOpSpinBalanced":
        """Angles of a matrix-form UCJ operator: its Coulomb matrices as
        number-number ansätze, its rotations as Givens ansätze."""
        nn_ops = [NumNumAnsatzOpSpinBalanced.from_diag_coulomb_mats(m) for m in ucj_op.diag_coulomb_mats]
        giv_ops = [GivensAnsatzOp.from_orbital_rotation(u) for u in ucj_op.orbital_rotations]
        final = None
        if ucj_op.final_orbital_rotation is not None:
            final = GivensAnsatzOp.from_orbital_rotation(ucj_op.final_orbital_rotation)
        return UCJAnglesOpSpinBalanced(ucj_op.norb, nn_ops, giv_ops, final)

    @staticmethod
    def from_t_amplitudes(t2: np.ndarray, *, t1: np.ndarray | None = None, n_reps: int | None = None,
                          interaction_pairs=None, tol: float = 1e-8) -> "UCJAnglesOpSpinBalanced":
        return UCJAnglesOpSpinBalanced.from_ucj_op(UCJOpSpinBalanced.from_t_amplitudes(
            t2, t1=t1, n_reps=n_reps, interaction_pairs=interaction_pairs, tol=tol))

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool):
        from ffsim_gb300 import gates

        if isinstance(nelec, (int, np.integer)):
            return NotImplemented
        _check_norb(self.norb, norb)
        basis = np.eye(norb)
        first = copy
        for nn, giv in zip(self.num_num_ansatz_ops, self.givens_ansatz_ops):
            u = giv.to_orbital_rotation()
            vec = gates.apply_orbital_rotation(vec, u.conj().T @ basis, norb, nelec, copy=first)
            vec = nn._apply_unitary_(vec, norb, nelec, copy=False)
            basis, first = u, False
        if self.final_givens_ansatz_op is not None:
            basis = self.final_givens_ansatz_op.to_orbital_rotation() @ basis
        return gates.apply_orbital_rotation(vec, basis, norb, nelec, copy=first)

    def _approx_eq_(self, other, rtol: float, atol: float) -> bool:
        from ffsim_gb300.protocols import approx_eq

        if not isinstance(other, UCJAnglesOpSpinBalanced):
            return NotImplemented
        if self.norb != other.norb or self.n_reps != other.n_reps:
            return False
        if not approx_eq(self.final_givens_ansatz_op, other.final_givens_ansatz_op):
            return False
        return all(approx_eq(a, b, rtol=rtol, atol=atol) for a, b in
                   zip(self.num_num_ansatz_ops + self.givens_ansatz_ops, other.num_num_ansatz_ops + other.givens_ansatz_ops))
