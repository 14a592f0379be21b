"""Two-orbital gates (python/ffsim/gates/basic_gates.py) and quadratic-Hamiltonian
evolution (python/ffsim/gates/quad_ham.py) against the reference's own code
(golden vectors).  The compositions run on the CPU here with the three gate
entry points and the occupied-orbital projector routed to the oracle; the GPU
entry points themselves are checked by the parity tests."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import ffsim_oracle as o

CASES = [("s", 5, (2, 2)), ("u", 4, (2, 1)), ("l", 5, 3)]


@pytest.fixture
def bg(monkeypatch):
    from ffsim_gb300 import _state
    from ffsim_gb300 import basic_gates as b

    monkeypatch.setattr(b, "apply_orbital_rotation",
                        lambda vec, mat, norb, nelec, copy=True: o.apply_orbital_rotation(vec, mat, norb, nelec))
    monkeypatch.setattr(b, "apply_num_op_sum_evolution",
                        lambda vec, c, t, norb, nelec, copy=True: o.apply_num_op_sum_evolution(vec, c, t, norb, nelec))
    monkeypatch.setattr(b, "apply_diag_coulomb_evolution",
                        lambda vec, m, t, norb, nelec, copy=True: o.apply_diag_coulomb_evolution(vec, m, t, norb, nelec))

    def prep(vec, norb, nelec, *, copy):
        arr = np.array(vec, dtype=complex)
        return _state.Prepared(torch.from_numpy(arr), arr.shape, True)

    def project(t, alpha, beta, norb, nelec):
        v2 = t.numpy().reshape(o.dim(norb, nelec[0]), o.dim(norb, nelec[1]))
        for spin, orbs in ((0, alpha), (1, beta)):
            for p in orbs:
                v2 = o._apply_excitation(v2, norb, nelec, p, p, spin)
        return torch.from_numpy(v2.reshape(-1).copy())

    monkeypatch.setattr(b, "prepare", prep)
    monkeypatch.setattr(b, "_project_occupied", project)
    return b


@pytest.mark.parametrize("tag, norb, nelec", CASES)
def test_gates_golden(bg, golden, tag, norb, nelec):
    g = lambda k: golden[f"bg{tag}_{k}"]  # noqa: E731
    vec = g("in")
    spins = [bg.Spin.ALPHA, bg.Spin.BETA, bg.Spin.ALPHA_AND_BETA] if isinstance(nelec, tuple) \
        else [bg.Spin.ALPHA_AND_BETA]
    for k, sp in enumerate(spins):
        checks = {
            "givens": bg.apply_givens_rotation(vec, 0.7, (0, 2), norb, nelec, sp, phi=0.3),
            "num": bg.apply_num_interaction(vec, 0.9, 1, norb, nelec, sp),
            "tunnel": bg.apply_tunneling_interaction(vec, 0.4, (3, 1), norb, nelec, sp),
            "numnum": bg.apply_num_num_interaction(vec, 1.1, (0, 3), norb, nelec, sp),
            "hop": bg.apply_hop_gate(vec, 0.5, (1, 2), norb, nelec, sp),
            "fsim": bg.apply_fsim_gate(vec, 0.6, 0.8, (2, 0), norb, nelec, sp),
            "fswap": bg.apply_fswap_gate(vec, (1, 3), norb, nelec, sp),
        }
        for name, got in checks.items():
            np.testing.assert_allclose(got, g(f"{name}{k}"), atol=1e-12, err_msg=f"{name} spin {sp}")
    np.testing.assert_allclose(bg.apply_quad_ham_evolution(vec, g("qmat"), 0.4, norb, nelec), g("quad"), atol=1e-12)
    if isinstance(nelec, tuple):
        np.testing.assert_allclose(bg.apply_quad_ham_evolution(vec, (g("qmat"), None), 0.4, norb, nelec),
                                   g("quadpair"), atol=1e-12)
        np.testing.assert_allclose(bg.apply_on_site_interaction(vec, 0.8, 2, norb, nelec), g("onsite"), atol=1e-12)
        for k, orbs in enumerate([((0, 2), (1,)), ((0, 1, 3), (2, 3)), ((), ()), ((1,), ()), ((0, 1), ()),
                                  ((), (2, 3)), ((0,), (1,)), ((0, 1, 2), ())]):
            np.testing.assert_allclose(bg.apply_num_op_prod_interaction(vec, 0.45, orbs, norb, nelec),
                                       g(f"prod{k}"), atol=1e-12, err_msg=str(orbs))


def test_argument_errors(bg):
    vec = o.random_state_vector(o.dim(4, (2, 1)), seed=1)
    with pytest.raises(ValueError):
        bg.apply_givens_rotation(vec, 0.1, (1, 1), 4, (2, 1))
    with pytest.raises(ValueError):
        bg.apply_num_num_interaction(vec, 0.1, (2, 2), 4, (2, 1))
    assert bg.pair_for_spin("x", bg.Spin.BETA) == (None, "x")


@pytest.fixture
def routed(bg, monkeypatch):
    """The gates module's entry points routed to the oracle too (the ansatz
    operators call them through the module)."""
    from ffsim_gb300 import gates

    monkeypatch.setattr(gates, "apply_orbital_rotation",
                        lambda vec, mat, norb, nelec, copy=True: o.apply_orbital_rotation(vec, mat, norb, nelec))
    monkeypatch.setattr(gates, "apply_diag_coulomb_evolution",
                        lambda vec, m, t, norb, nelec, copy=True: o.apply_diag_coulomb_evolution(vec, m, t, norb, nelec))
    return bg


def test_num_num_ansatz_golden(routed, golden):
    import ffsim_gb300 as f

    pairs = ([(0, 1), (1, 3), (2, 2)], [(0, 0), (1, 2)])
    op = f.NumNumAnsatzOpSpinBalanced.from_parameters(golden["nn_params"], norb=4, interaction_pairs=pairs)
    np.testing.assert_allclose(op.to_diag_coulomb_mats(), golden["nn_mats"], atol=1e-15)
    np.testing.assert_allclose(op._apply_unitary_(golden["nn_in"], 4, (2, 1), copy=True), golden["nn_out"], atol=1e-12)
    np.testing.assert_allclose(op.to_parameters(), golden["nn_params"])
    back = f.NumNumAnsatzOpSpinBalanced.from_diag_coulomb_mats(op.to_diag_coulomb_mats())
    assert f.approx_eq(back, op)
    assert f.NumNumAnsatzOpSpinBalanced.n_params(pairs) == 5
    with pytest.raises(ValueError):
        f.NumNumAnsatzOpSpinBalanced(4, ([(1, 0)], []), (np.ones(1), np.ones(0)))


def test_hop_gate_ansatz_golden(routed, golden):
    import ffsim_gb300 as f

    pairs = [(0, 1), (2, 3), (1, 2)]
    for k, final in enumerate((False, True)):
        op = f.HopGateAnsatzOperator.from_parameters(golden[f"hop{k}_params"], norb=4, interaction_pairs=pairs,
                                                     with_final_orbital_rotation=final)
        np.testing.assert_allclose(op._apply_unitary_(golden[f"hop{k}_in"], 4, (2, 2), copy=True),
                                   golden[f"hop{k}_out"], atol=1e-12)
        np.testing.assert_allclose(op.to_parameters(), golden[f"hop{k}_to"], atol=1e-10)
        assert f.approx_eq(op, op)


def test_ucj_angles_golden(routed, golden):
    """UCJ operator in gate angles: parameter layout, action and the conversion
    from the matrix form, against the reference's own code."""
    import ffsim_gb300 as f

    nn_pairs, giv_pairs = ([(0, 1), (2, 3)], [(0, 0), (1, 1), (0, 2)]), [(0, 1), (2, 3), (1, 2)]
    cls = f.variational.UCJAnglesOpSpinBalanced
    assert cls.n_params(4, 2, nn_pairs, giv_pairs, with_final_givens_ansatz_op=True) == len(golden["ang_params"])
    op = cls.from_parameters(golden["ang_params"], norb=4, n_reps=2, num_num_interaction_pairs=nn_pairs,
                             givens_interaction_pairs=giv_pairs, with_final_givens_ansatz_op=True)
    np.testing.assert_allclose(op._apply_unitary_(golden["ang_in"], 4, (2, 2), copy=True), golden["ang_out"],
                               atol=1e-12)
    np.testing.assert_allclose(op.to_parameters(), golden["ang_to"], atol=1e-12)
    assert f.approx_eq(op, op)
    ucj = f.UCJOpSpinBalanced.from_parameters(golden["ang_ucj_params"], norb=4, n_reps=2,
                                              with_final_orbital_rotation=True)
    conv = cls.from_ucj_op(ucj)
    np.testing.assert_allclose(conv.to_parameters(), golden["ang_from_ucj_to"], atol=1e-10)
    np.testing.assert_allclose(conv._apply_unitary_(golden["ang_in"], 4, (2, 2), copy=True),
                               golden["ang_from_ucj_out"], atol=1e-10)
