"""Trotter-Suzuki time evolution of a double-factorized Hamiltonian, the GPU
counterpart of python/ffsim/trotter/double_factorized.py:25-127.

A step runs the Hamiltonian's terms in the order of the step sequence: the
one-body term multiplies the running orbital basis by exp(-i t h) on the host;
a two-body term t rotates the state from the running basis into U_t's basis
(one orbital rotation, ``ffgb_apply_orbital_rotation``) and applies
exp(-i t J_t n n) (``ffgb_apply_diag_coulomb_evolution``).  The last basis and
the global phase exp(-i T constant) close the evolution, so a step costs one
orbital rotation and one diagonal evolution per two-body term.

``simulate_trotter_diag_coulomb_split_op`` is the split-operator counterpart
for a diagonal Coulomb Hamiltonian
(python/ffsim/trotter/diagonal_coulomb_split_op.py:25-122): two terms, the
Coulomb one applied in the occupation basis.
"""

from __future__ import annotations

import cmath
from collections.abc import Iterator

import numpy as np

from ffsim_gb300._state import prepare
from ffsim_gb300.gates import apply_diag_coulomb_evolution, apply_orbital_rotation
from ffsim_gb300.linalg import eigh


def simulate_trotter_step_iterator(n_terms: int, time: float, order: int = 0) -> Iterator[tuple[int, float]]:
    """(term index, time) pairs of one Trotter step (python/ffsim/trotter/_util.py:18-60).

    Order 0 is the plain product of the terms.  Order 1 is the symmetric
    product: every term but the last at half time, the last at full time, then
    the first ones again in reverse.  Order k > 1 is Suzuki's fractal
    construction (J. Math. Phys. 32, 400 (1991)): five order-(k-1) steps with
    times p, p, 1 - 4p, p, p where p = 1 / (4 - 4^(1 / (2k - 1))).
    """
    if order == 0:
        for i in range(n_terms):
            yield i, time
        return
    if order == 1:
        for i in range(n_terms - 1):
            yield i, time / 2
        yield n_terms - 1, time
        for i in reversed(range(n_terms - 1)):
            yield i, time / 2
        return
    p = time / (4 - 4 ** (1 / (2 * order - 1)))
    for _ in range(2):
        yield from simulate_trotter_step_iterator(n_terms, p, order - 1)
    yield from simulate_trotter_step_iterator(n_terms, time - 4 * p, order - 1)
    for _ in range(2):
        yield from simulate_trotter_step_iterator(n_terms, p, order - 1)


def _expm_hermitian(h: np.ndarray, t: float) -> np.ndarray:
    """exp(-i t h) for Hermitian h, from its eigendecomposition (FP64)."""
    w, v = eigh(h)
    return (v * np.exp(-1j * t * w)) @ v.conj().T


def simulate_trotter_double_factorized(vec, hamiltonian, time: float, *, norb: int, nelec: tuple[int, int],
                                       n_steps: int = 1, order: int = 0, copy: bool = True):
    """Evolve ``vec`` by exp(-i time H) with ``n_steps`` Trotter steps of the
    given order (``ffsim.simulate_trotter_double_factorized``).

    ``hamiltonian`` is a ``DoubleFactorizedHamiltonian``; ``vec`` a torch CUDA
    complex tensor (or a numpy array, moved to the GPU and back).  ``copy``
    follows the reference: with ``copy=False`` the input may be overwritten.
    """
    if order < 0:
        raise ValueError(f"order must be non-negative, got {order}.")
    if n_steps < 0:
        raise ValueError(f"n_steps must be non-negative, got {n_steps}.")
    p = prepare(vec, norb, nelec, copy=copy)
    if n_steps == 0:
        return p.finish()
    state = p.tensor.reshape(-1)
    one_body = np.asarray(hamiltonian.one_body_tensor, dtype=complex)
    dcm = np.asarray(hamiltonian.diag_coulomb_mats, dtype=float)
    rots = np.asarray(hamiltonian.orbital_rotations, dtype=complex)
    z_rep = bool(hamiltonian.z_representation)
    step = time / n_steps
    basis = np.eye(norb, dtype=complex)
    for _ in range(n_steps):
        for k, t in simulate_trotter_step_iterator(1 + len(dcm), step, order):
            if k == 0:
                basis = _expm_hermitian(one_body, t) @ basis
            else:
                u = rots[k - 1]
                state = apply_orbital_rotation(state, u.T.conj() @ basis, norb, nelec, copy=False)
                state = apply_diag_coulomb_evolution(state, dcm[k - 1], t, norb, nelec,
                                                     z_representation=z_rep, copy=False)
                basis = u
    state = apply_orbital_rotation(state, basis, norb, nelec, copy=False)
    if hamiltonian.constant:
        state.mul_(cmath.exp(-1j * time * hamiltonian.constant))
    if state.data_ptr() != p.tensor.data_ptr():
        p.tensor.reshape(-1).copy_(state)
    return p.finish()


def simulate_trotter_diag_coulomb_split_op(vec, hamiltonian, time: float, *, norb: int, nelec: tuple[int, int],
                                           n_steps: int = 1, order: int = 0, copy: bool = True):
    """Evolve ``vec`` by exp(-i time H) for a ``DiagonalCoulombHamiltonian`` with
    the split-operator method (``ffsim.simulate_trotter_diag_coulomb_split_op``,
    python/ffsim/trotter/diagonal_coulomb_split_op.py:25-122).

    The step sequence has two terms.  The one-body term multiplies the running
    orbital basis by exp(-i t h) on the host; the Coulomb term rotates the
    state by that basis (``ffgb_apply_orbital_rotation``), applies
    exp(-i t J n n) with (J_aa, J_ab, J_aa) in the occupation basis
    (``ffgb_apply_diag_coulomb_evolution``) and resets the basis to the identity.
    """
    if order < 0:
        raise ValueError(f"order must be non-negative, got {order}.")
    if n_steps < 0:
        raise ValueError(f"n_steps must be non-negative, got {n_steps}.")
    p = prepare(vec, norb, nelec, copy=copy)
    if n_steps == 0:
        return p.finish()
    state = p.tensor.reshape(-1)
    one_body = np.asarray(hamiltonian.one_body_tensor, dtype=complex)
    aa, ab = np.asarray(hamiltonian.diag_coulomb_mats, dtype=float)
    step = time / n_steps
    basis = None  # the identity: a rotation by it is skipped (it changes no amplitude)
    for _ in range(n_steps):
        for k, t in simulate_trotter_step_iterator(2, step, order):
            if k == 0:
                u = _expm_hermitian(one_body, t)
                basis = u if basis is None else u @ basis
            else:
                if basis is not None:
                    state = apply_orbital_rotation(state, basis, norb, nelec, copy=False)
                state = apply_diag_coulomb_evolution(state, (aa, ab, aa), t, norb, nelec, copy=False)
                basis = None
    if basis is not None:
        state = apply_orbital_rotation(state, basis, norb, nelec, copy=False)
    if hamiltonian.constant:
        state.mul_(cmath.exp(-1j * time * hamiltonian.constant))
    if state.data_ptr() != p.tensor.data_ptr():
        p.tensor.reshape(-1).copy_(state)
    return p.finish()
