"""Multireference states (python/ffsim/variational/multireference.py) against
the reference's own code (golden vectors)."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import ffsim_oracle as o

OCCS = [([0, 1], [0, 1]), ([0, 2], [0, 1]), ([0, 1], [1, 3])]


def _check(golden, root, energy, state):
    assert abs(energy - float(golden[f"mr{root}_energy"])) < 1e-10
    ref = golden[f"mr{root}_state"]
    overlap = np.vdot(ref, state)
    assert abs(abs(overlap) - np.vdot(ref, ref).real) < 1e-10
    np.testing.assert_allclose(state * np.conj(overlap) / abs(overlap), ref, atol=1e-10)


def test_host_sequence(golden, monkeypatch):
    """The composition on the CPU: determinants and the ansatz from the oracle,
    the Hamiltonian as a SciPy operator over the oracle's matvec."""
    import scipy.sparse.linalg as sla

    import ffsim_gb300 as f
    from ffsim_gb300 import multireference as mr

    ucj = f.UCJOpSpinBalanced.from_parameters(golden["mr_params"], norb=4, n_reps=2)
    monkeypatch.setattr(mr, "slater_determinant",
                        lambda norb, occ, dtype=None: f.slater_determinant(norb, occ, device="cpu").numpy())
    monkeypatch.setattr(mr, "apply_unitary", lambda vec, op, norb, nelec, copy=True: o.ucj_spin_balanced_apply(
        vec, op.diag_coulomb_mats, op.orbital_rotations, op.final_orbital_rotation, norb, nelec))
    mv = o.df_hamiltonian_matvec(golden["mr_h1"], golden["mr_dcm"], golden["mr_rots"], 0.7, 4, (2, 2))
    lin = sla.LinearOperator((36, 36), matvec=mv, dtype=complex)
    for root in (0, 1):
        energy, state = mr.multireference_state(lin, ucj, OCCS, 4, (2, 2), root=root)
        _check(golden, root, energy, state)


@pytest.mark.gpu
def test_gpu(cuda, golden):
    import ffsim_gb300 as f

    ucj = f.UCJOpSpinBalanced.from_parameters(golden["mr_params"], norb=4, n_reps=2)
    ham = f.DoubleFactorizedHamiltonian(golden["mr_h1"], golden["mr_dcm"], golden["mr_rots"], constant=0.7)
    for root in (0, 1):
        energy, state = f.multireference_state(ham, ucj, OCCS, 4, (2, 2), root=root)
        _check(golden, root, energy, state.cpu().numpy())
