"""Spin-unbalanced and spinless UCJ operators (python/ffsim/variational/
ucj_spin_unbalanced.py, ucj_spinless.py) against golden vectors made by the
reference's own classes: parameter layout and the oracle on the CPU,
``apply_unitary`` on the GPU."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import ffsim_oracle as o


def _cases(golden):
    for idx, (kind, norb, na, nb, n_reps, final) in enumerate(golden["ucjx_cases"]):
        nelec = int(na) if nb < 0 else (int(na), int(nb))
        yield idx, int(kind), int(norb), nelec, int(n_reps), bool(final)


def _cls(kind):
    import ffsim_gb300 as f

    return f.UCJOpSpinUnbalanced if kind == 0 else f.UCJOpSpinless


def test_parameter_layout(golden):
    for idx, kind, norb, nelec, n_reps, final in _cases(golden):
        params = golden[f"ucjx{idx}_params"]
        op = _cls(kind).from_parameters(params, norb=norb, n_reps=n_reps, with_final_orbital_rotation=final)
        assert _cls(kind).n_params(norb, n_reps, with_final_orbital_rotation=final) == len(params)
        np.testing.assert_allclose(op.diag_coulomb_mats, golden[f"ucjx{idx}_dcm"], atol=1e-14)
        np.testing.assert_allclose(op.orbital_rotations, golden[f"ucjx{idx}_rots"], atol=1e-12)
        np.testing.assert_allclose(op.to_parameters(), params, atol=1e-10)
        with pytest.raises(ValueError):
            _cls(kind).from_parameters(params[:-1], norb=norb, n_reps=n_reps, with_final_orbital_rotation=final)


def test_oracle(golden):
    for idx, kind, norb, nelec, n_reps, final in _cases(golden):
        op = _cls(kind).from_parameters(golden[f"ucjx{idx}_params"], norb=norb, n_reps=n_reps,
                                        with_final_orbital_rotation=final)
        fn = o.ucj_spin_unbalanced_apply if kind == 0 else o.ucj_spinless_apply
        got = fn(golden[f"ucjx{idx}_in"], op.diag_coulomb_mats, op.orbital_rotations, op.final_orbital_rotation,
                 norb, nelec)
        np.testing.assert_allclose(got, golden[f"ucjx{idx}_out"], atol=1e-12)


def test_validation():
    import ffsim_gb300 as f

    with pytest.raises(ValueError):
        f.UCJOpSpinUnbalanced(np.zeros((1, 2, 3, 3)), np.stack([np.stack([np.eye(3)] * 2)]))
    with pytest.raises(ValueError):
        f.UCJOpSpinless(np.zeros((1, 3, 3)), np.zeros((1, 3, 3)))


@pytest.mark.gpu
def test_apply_unitary(cuda, golden):
    import torch

    import ffsim_gb300 as f

    for idx, kind, norb, nelec, n_reps, final in _cases(golden):
        op = _cls(kind).from_parameters(golden[f"ucjx{idx}_params"], norb=norb, n_reps=n_reps,
                                        with_final_orbital_rotation=final)
        for dtype, tol in [(torch.complex128, 1e-12), (torch.complex64, 2e-5)]:
            v = torch.from_numpy(golden[f"ucjx{idx}_in"]).to("cuda").to(dtype)
            out = f.apply_unitary(v, op, norb, nelec)
            np.testing.assert_allclose(out.cpu().numpy().astype(complex), golden[f"ucjx{idx}_out"], atol=tol)


def _giv(golden, idx):
    import ffsim_gb300 as f

    norb, na, nb, with_phis, with_angles = (int(x) for x in golden["giv_cases"][idx])
    pairs = [tuple(int(x) for x in p) for p in golden[f"giv{idx}_pairs"]]
    op = f.GivensAnsatzOp.from_parameters(golden[f"giv{idx}_params"], norb, pairs, with_phis=bool(with_phis),
                                          with_phase_angles=bool(with_angles))
    return op, norb, (na, nb)


def test_givens_ansatz(golden):
    """Parameters -> orbital rotation, and the brickwork from a rotation, against
    the reference's GivensAnsatzOp (variational/givens.py)."""
    import ffsim_gb300 as f

    for idx in range(len(golden["giv_cases"])):
        op, norb, _ = _giv(golden, idx)
        np.testing.assert_allclose(op.to_orbital_rotation(), golden[f"giv{idx}_rot"], atol=1e-13)
        np.testing.assert_allclose(op.to_parameters(), golden[f"giv{idx}_params"], atol=0)
    for norb in (4, 5):
        op = f.GivensAnsatzOp.from_orbital_rotation(golden[f"givu{norb}_u"])
        assert [list(p) for p in op.interaction_pairs] == golden[f"givu{norb}_pairs"].tolist()
        np.testing.assert_allclose(op.thetas, golden[f"givu{norb}_thetas"], atol=1e-12)
        np.testing.assert_allclose(op.phis, golden[f"givu{norb}_phis"], atol=1e-12)
        np.testing.assert_allclose(op.phase_angles, golden[f"givu{norb}_angles"], atol=1e-12)
        np.testing.assert_allclose(op.to_orbital_rotation(), golden[f"givu{norb}_u"], atol=1e-12)


@pytest.mark.gpu
def test_givens_ansatz_apply(cuda, golden):
    import torch

    import ffsim_gb300 as f

    for idx in range(len(golden["giv_cases"])):
        op, norb, nelec = _giv(golden, idx)
        for dtype, tol in [(torch.complex128, 1e-12), (torch.complex64, 2e-5)]:
            v = torch.from_numpy(golden[f"giv{idx}_in"]).to("cuda").to(dtype)
            out = f.apply_unitary(v, op, norb, nelec)
            np.testing.assert_allclose(out.cpu().numpy().astype(complex), golden[f"giv{idx}_out"], atol=tol)


def test_interaction_pairs(golden):
    """Local-UCJ parameter maps with restricted interaction pairs, against the
    reference's from_parameters / to_parameters of the three UCJ classes."""
    import ffsim_gb300 as f

    cases = [
        (f.UCJOpSpinBalanced, 4, 2, ([(0, 0), (1, 1), (0, 1), (2, 3)], [(0, 0), (1, 2), (3, 3)]), True),
        (f.UCJOpSpinBalanced, 5, 1, (None, [(p, p) for p in range(5)]), False),
        (f.UCJOpSpinUnbalanced, 4, 2, ([(0, 1), (2, 2)], [(1, 0), (0, 1), (3, 2)], None), True),
        (f.UCJOpSpinUnbalanced, 4, 1, ([], [(2, 2)], [(0, 3)]), False),
        (f.UCJOpSpinless, 4, 2, [(0, 0), (1, 3), (2, 3)], True),
    ]
    for idx, (cls, norb, n_reps, pairs, final) in enumerate(cases):
        params = golden[f"pairs{idx}_params"]
        assert cls.n_params(norb, n_reps, interaction_pairs=pairs, with_final_orbital_rotation=final) == len(params)
        op = cls.from_parameters(params, norb=norb, n_reps=n_reps, interaction_pairs=pairs,
                                 with_final_orbital_rotation=final)
        np.testing.assert_allclose(op.diag_coulomb_mats, golden[f"pairs{idx}_dcm"], atol=1e-15)
        np.testing.assert_allclose(op.orbital_rotations, golden[f"pairs{idx}_rots"], atol=1e-12)
        np.testing.assert_allclose(op.to_parameters(interaction_pairs=pairs), golden[f"pairs{idx}_to"], atol=1e-10)


def test_interaction_pair_validation():
    import ffsim_gb300 as f

    with pytest.raises(ValueError):  # lower triangular same-spin pair
        f.UCJOpSpinBalanced.n_params(4, 1, interaction_pairs=([(1, 0)], None))
    with pytest.raises(ValueError):  # duplicates
        f.UCJOpSpinUnbalanced.n_params(4, 1, interaction_pairs=(None, [(1, 0), (1, 0)], None))
    assert f.UCJOpSpinUnbalanced.n_params(4, 1, interaction_pairs=(None, [(1, 0)], None)) == 10 + 1 + 10 + 32
