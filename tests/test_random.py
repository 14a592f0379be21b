"""Seeded random constructors (python/ffsim/random/random.py): the same seed
gives the same matrices, Hamiltonians and operators as the reference's own
code (golden vectors made by it)."""

from __future__ import annotations

import numpy as np
import pytest


def _eq(a, b):
    np.testing.assert_allclose(np.asarray(a), b, rtol=0, atol=1e-14)


def test_matrices(golden):
    import ffsim_gb300 as f

    r = f.random
    _eq(r.random_density_matrix(4, seed=1), golden["rnd_density"])
    _eq(r.random_orthogonal(5, seed=2), golden["rnd_orth"])
    _eq(r.random_special_orthogonal(5, seed=3), golden["rnd_sorth"])
    assert np.linalg.det(r.random_special_orthogonal(5, seed=3)) > 0
    _eq(r.random_hermitian(4, seed=4), golden["rnd_herm"])
    _eq(r.random_antihermitian(4, seed=5), golden["rnd_antiherm"])
    _eq(r.random_two_body_tensor(3, seed=6), golden["rnd_tbt"])
    _eq(r.random_two_body_tensor(3, rank=2, seed=7, dtype=float), golden["rnd_tbt_real_r2"])
    with pytest.raises(ValueError):
        r.random_density_matrix(0)


def test_hamiltonians(golden):
    import ffsim_gb300 as f

    r = f.random
    for tag, dt in [("c", complex), ("r", float)]:
        m = r.random_molecular_hamiltonian(3, seed=8, dtype=dt)
        _eq(m.one_body_tensor, golden[f"rnd_mol{tag}_h1"])
        _eq(m.two_body_tensor, golden[f"rnd_mol{tag}_h2"])
        assert m.constant == float(golden[f"rnd_mol{tag}_const"])
    for tag, real in [("c", False), ("r", True)]:
        h = r.random_diagonal_coulomb_hamiltonian(4, real=real, seed=9)
        _eq(h.one_body_tensor, golden[f"rnd_dch{tag}_h1"])
        _eq(h.diag_coulomb_mats, golden[f"rnd_dch{tag}_dcm"])
        assert h.constant == float(golden[f"rnd_dch{tag}_const"])
        h = r.random_double_factorized_hamiltonian(3, rank=2, real=real, seed=10)
        _eq(h.one_body_tensor, golden[f"rnd_df{tag}_h1"])
        _eq(h.diag_coulomb_mats, golden[f"rnd_df{tag}_dcm"])
        _eq(h.orbital_rotations, golden[f"rnd_df{tag}_rots"])
        assert h.constant == float(golden[f"rnd_df{tag}_const"])
    h = r.random_double_factorized_hamiltonian(3, seed=11, z_representation=True)
    assert h.z_representation and h.diag_coulomb_mats.shape[0] == 6
    _eq(h.orbital_rotations, golden["rnd_dfz_rots"])


def test_ucj_operators(golden):
    import ffsim_gb300 as f

    r = f.random
    kws = [dict(n_reps=2, seed=12), dict(n_reps=1, with_final_orbital_rotation=True, diag_coulomb_normal=True,
                                         diag_coulomb_scale=0.3, seed=13)]
    for k, kw in enumerate(kws):
        for tag, fn in [("bal", r.random_ucj_op_spin_balanced), ("unb", r.random_ucj_op_spin_unbalanced),
                        ("sl", r.random_ucj_op_spinless)]:
            op = fn(4, **kw)
            _eq(op.diag_coulomb_mats, golden[f"rnd_{tag}{k}_dcm"])
            _eq(op.orbital_rotations, golden[f"rnd_{tag}{k}_rots"])
            if f"rnd_{tag}{k}_final" in golden:
                _eq(op.final_orbital_rotation, golden[f"rnd_{tag}{k}_final"])
            else:
                assert op.final_orbital_rotation is None
    op = r.random_ucj_op_spin_balanced(4, n_reps=2, interaction_pairs=([(0, 0), (1, 2)], [(0, 0), (3, 3)]), seed=14)
    _eq(op.diag_coulomb_mats, golden["rnd_balp_dcm"])
    op = r.random_ucj_op_spin_unbalanced(4, interaction_pairs=([(0, 1)], [(2, 0), (1, 1)], []), seed=15)
    _eq(op.diag_coulomb_mats, golden["rnd_unbp_dcm"])
    op = r.random_ucj_op_spinless(4, interaction_pairs=[(0, 3), (2, 2)], seed=16)
    _eq(op.diag_coulomb_mats, golden["rnd_slp_dcm"])
    with pytest.raises(ValueError):
        r.random_ucj_op_spin_balanced(4, interaction_pairs=([(1, 0)], None))
    with pytest.raises(ValueError):
        r.random_ucj_op_spinless(4, interaction_pairs=[(0, 1), (0, 1)])
