"""Gates on fermionic state vectors: the GPU counterparts of
python/ffsim/gates/{orbital_rotation,diag_coulomb,num_op_sum}.py.

Signatures, argument meaning, ``copy`` semantics and errors follow the
reference.  Vectors may be torch CUDA complex tensors (complex64 or
complex128, shape ``[dim]`` or ``[dim_a, dim_b]``) or numpy arrays (moved to
the GPU and back).  The result keeps the input's shape and dtype.
"""

from __future__ import annotations

import numpy as np

from ffsim_gb300 import _lib
from ffsim_gb300._state import prepare, scratch, split_nelec, stream_ptr


def _split_pair(mat):
    """(mat_a, mat_b) from a single matrix, a pair, or a stacked (2, n, n) array
    (python/ffsim/gates/orbital_rotation.py:157-174)."""
    if isinstance(mat, np.ndarray) and mat.ndim == 2:
        return mat, mat
    if hasattr(mat, "ndim") and not isinstance(mat, np.ndarray) and mat.ndim == 2:
        m = np.asarray(mat.cpu() if hasattr(mat, "cpu") else mat)
        return m, m
    mat_a, mat_b = mat
    return mat_a, mat_b


def _dagger(m):
    return None if m is None else np.asarray(m).conj().T


def apply_orbital_rotation(vec, mat, norb: int, nelec, *, copy: bool = True):
    r"""Apply the orbital rotation :math:`a^\dagger_{i\sigma} \mapsto \sum_j U^{(\sigma)}_{ji} a^\dagger_{j\sigma}`.

    Mirrors ``ffsim.apply_orbital_rotation`` (python/ffsim/gates/orbital_rotation.py:44-99).
    ``mat`` is one unitary for both spins, a pair ``(mat_a, mat_b)`` (entries
    may be ``None``) or a stacked ``(2, norb, norb)`` array.
    """
    p = prepare(vec, norb, nelec, copy=copy)
    n_alpha, n_beta = split_nelec(nelec)
    if n_beta < 0:
        ma, mb = np.asarray(mat), None
    else:
        ma, mb = _split_pair(mat)
    ma = _lib.cmat(ma, (norb, norb), "orbital rotation")
    mb = _lib.cmat(mb, (norb, norb), "orbital rotation")
    buf, nbytes = scratch(p.tensor, 0, norb, n_alpha, n_beta)
    _lib.call(
        "ffgb_apply_orbital_rotation", p.ptr(), p.dtype_code, norb, n_alpha, n_beta,
        _lib.dptr(ma), _lib.dptr(mb), buf.data_ptr(), nbytes, stream_ptr(p.tensor),
    )
    return p.finish()


def _split_three(mat):
    """(aa, ab, bb) as in python/ffsim/gates/diag_coulomb.py:223-275."""
    if isinstance(mat, np.ndarray) and mat.ndim == 2:
        return mat, mat, mat
    aa, ab, bb = mat
    return aa, ab, bb


def apply_diag_coulomb_evolution(vec, mat, time: float, norb: int, nelec, *, orbital_rotation=None,
                                 z_representation: bool = False, copy: bool = True):
    r"""Apply :math:`\mathcal{U} \exp(-i t \sum J^{(\sigma\tau)}_{ij} n_{i\sigma} n_{j\tau}/2) \mathcal{U}^\dagger`.

    Mirrors ``ffsim.apply_diag_coulomb_evolution`` (python/ffsim/gates/diag_coulomb.py:68-153).
    """
    n_alpha, n_beta = split_nelec(nelec)
    if n_beta < 0 and z_representation:
        raise NotImplementedError
    p = prepare(vec, norb, nelec, copy=copy)
    aa, ab, bb = _split_three(mat)
    aa, ab, bb = (_lib.rmat(m, (norb, norb), "diagonal Coulomb matrix") for m in (aa, ab, bb))
    ra = rb = None
    if orbital_rotation is not None:
        if n_beta < 0:
            ra = np.asarray(orbital_rotation)
        else:
            ra, rb = _split_pair(orbital_rotation)
    ra, rb = (_lib.cmat(r, (norb, norb), "orbital rotation") for r in (ra, rb))
    buf, nbytes = scratch(p.tensor, 0, norb, n_alpha, n_beta)
    _lib.call(
        "ffgb_apply_diag_coulomb_evolution", p.ptr(), p.dtype_code, norb, n_alpha, n_beta,
        _lib.dptr(aa), _lib.dptr(ab), _lib.dptr(bb), float(time), int(bool(z_representation)),
        _lib.dptr(ra), _lib.dptr(rb), buf.data_ptr(), nbytes, stream_ptr(p.tensor),
    )
    return p.finish()


def apply_num_op_sum_evolution(vec, coeffs, time: float, norb: int, nelec, *, orbital_rotation=None,
                               copy: bool = True):
    r"""Apply :math:`\mathcal{U} \exp(-i t \sum \lambda^{(\sigma)}_i n_{i\sigma}) \mathcal{U}^\dagger`.

    Mirrors ``ffsim.apply_num_op_sum_evolution`` (python/ffsim/gates/num_op_sum.py:62-140).
    """
    n_alpha, n_beta = split_nelec(nelec)
    p = prepare(vec, norb, nelec, copy=copy)
    if isinstance(coeffs, np.ndarray) or n_beta < 0:
        ca = cb = np.asarray(coeffs)
    else:
        ca, cb = coeffs
    ca, cb = (_lib.rmat(c, (norb,), "coefficients") for c in (ca, cb))
    ra = rb = None
    if orbital_rotation is not None:
        if n_beta < 0:
            ra = np.asarray(orbital_rotation)
        else:
            ra, rb = _split_pair(orbital_rotation)
    ra, rb = (_lib.cmat(r, (norb, norb), "orbital rotation") for r in (ra, rb))
    buf, nbytes = scratch(p.tensor, 0, norb, n_alpha, n_beta)
    _lib.call(
        "ffgb_apply_num_op_sum_evolution", p.ptr(), p.dtype_code, norb, n_alpha, n_beta,
        _lib.dptr(ca), _lib.dptr(cb), float(time), _lib.dptr(ra), _lib.dptr(rb),
        buf.data_ptr(), nbytes, stream_ptr(p.tensor),
    )
    return p.finish()


def apply_givens_rotation_in_place(vec, c: float, s: complex, target_orbs: tuple[int, int], norb: int,
                                   nelec, spin: int = 0) -> None:
    """One adjacent Givens rotation on one spin sector, in place (the kernel behind
    ``_apply_orbital_rotation_adjacent_spin_in_place``,
    python/ffsim/gates/orbital_rotation.py:177-199 and src/gates/orbital_rotation.rs:18-104).

    Strings with ``i`` occupied and ``j`` empty become ``c x + s y`` and their
    partners ``c y - conj(s) x``.  ``vec`` must be a contiguous CUDA tensor."""
    i, j = target_orbs
    if abs(i - j) != 1:
        raise AssertionError("Target orbitals must be adjacent.")
    n_alpha, n_beta = split_nelec(nelec)
    p = prepare(vec, norb, nelec, copy=False)
    s = complex(s)
    _lib.call("ffgb_apply_givens_rotation", p.ptr(), p.dtype_code, norb, n_alpha, n_beta, int(spin),
              float(c), s.real, s.imag, int(i), int(j), stream_ptr(p.tensor))


def apply_phase_shift_in_place(vec, phase: complex, orb: int, norb: int, nelec, spin: int = 0) -> None:
    """Multiply strings with ``orb`` occupied in one sector by ``phase``
    (src/gates/phase_shift.rs:17-30)."""
    n_alpha, n_beta = split_nelec(nelec)
    p = prepare(vec, norb, nelec, copy=False)
    phase = complex(phase)
    _lib.call("ffgb_apply_phase_shift", p.ptr(), p.dtype_code, norb, n_alpha, n_beta, int(spin),
              phase.real, phase.imag, int(orb), stream_ptr(p.tensor))
