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


def _t2_case(golden, idx):
    norb, nocc, _, _ = (int(x) for x in golden["t2_cases"][idx])
    return norb, nocc, golden[f"t2{idx}_t2"], golden[f"t2{idx}_t1"]


def test_double_factorized_t2_golden(golden):
    """Coulomb matrices entry by entry; rotations up to each eigenvector's phase,
    through the reconstructed amplitudes."""
    import ffsim_gb300 as f

    for idx in range(len(golden["t2_cases"])):
        norb, nocc, t2, _ = _t2_case(golden, idx)
        mats, rots = f.linalg.double_factorized_t2(t2)
        np.testing.assert_allclose(mats, golden[f"t2{idx}_mats"], atol=1e-10)
        gr = golden[f"t2{idx}_rots"]
        np.testing.assert_allclose(np.abs(rots), np.abs(gr), atol=1e-8)
        rec = lambda m, u: 1j * np.einsum("kpq,kap,kip,kbq,kjq->ijab", m, u, u.conj(), u, u.conj())[  # noqa: E731
            :nocc, :nocc, nocc:, nocc:]
        np.testing.assert_allclose(rec(mats, rots), rec(golden[f"t2{idx}_mats"], gr), atol=1e-10)
        np.testing.assert_allclose(f.linalg.double_factorized_t2(t2, max_terms=3)[0], golden[f"t2{idx}_mats3"],
                                   atol=1e-10)
    with pytest.raises(ValueError):
        f.linalg.double_factorized_t2(golden["t20_t2"], max_terms=0)
    with pytest.raises(NotImplementedError):
        f.linalg.double_factorized_t2(golden["t20_t2"], optimize=True)


def test_from_t_amplitudes_golden(golden):
    """The operators' matrices, and their action (through the oracle) against
    the reference's own apply_unitary on the same vectors."""
    import ffsim_gb300 as f

    for idx in range(len(golden["t2_cases"])):
        norb, nocc, t2, t1 = _t2_case(golden, idx)
        np.testing.assert_allclose(f.variational.orbital_rotation_from_t1_amplitudes(t1), golden[f"t2{idx}_t1rot"],
                                   atol=1e-12)
        for tag, kw in [("a", {}), ("b", {"n_reps": 2, "t1": t1}), ("c", {"n_reps": 40}),
                        ("d", {"interaction_pairs": ([(0, 1), (1, 2)], [(0, 0)]), "n_reps": 3})]:
            op = f.UCJOpSpinBalanced.from_t_amplitudes(t2, **kw)
            np.testing.assert_allclose(op.diag_coulomb_mats, golden[f"t2{idx}_op{tag}_dcm"], atol=1e-10)
            assert op.orbital_rotations.shape == golden[f"t2{idx}_op{tag}_rots"].shape
            got = o.ucj_spin_balanced_apply(golden[f"t2{idx}_op{tag}_in"], op.diag_coulomb_mats, op.orbital_rotations,
                                            op.final_orbital_rotation, norb, (nocc, nocc))
            np.testing.assert_allclose(got, golden[f"t2{idx}_op{tag}_out"], atol=1e-10)
    with pytest.raises(ValueError):
        f.UCJOpSpinBalanced.from_t_amplitudes(golden["t20_t2"], n_reps=0)


def test_random_t2_amplitudes_symmetry():
    import ffsim_gb300 as f

    t2 = f.random.random_t2_amplitudes(6, 2, seed=3)
    np.testing.assert_allclose(t2, t2.transpose(1, 0, 3, 2), atol=1e-12)


def test_interaction_pair_layouts():
    import ffsim_gb300 as f

    ip = f.variational.interaction_pairs_spin_balanced
    assert ip("all-to-all", 4) == (None, None)
    assert ip("square", 3) == ([(0, 1), (1, 2)], [(0, 0), (1, 1), (2, 2)])
    assert ip("heavy-hex", 6)[1] == [(0, 0), (4, 4)]
    with pytest.raises(ValueError):
        ip("ring", 4)


@pytest.mark.gpu
def test_gpu_from_t_amplitudes_golden(cuda, golden):
    import torch

    import ffsim_gb300 as f

    for idx in range(len(golden["t2_cases"])):
        norb, nocc, t2, t1 = _t2_case(golden, idx)
        for tag, kw in [("a", {}), ("b", {"n_reps": 2, "t1": t1}), ("c", {"n_reps": 40})]:
            op = f.UCJOpSpinBalanced.from_t_amplitudes(t2, **kw)
            vin = golden[f"t2{idx}_op{tag}_in"]
            for dtype, tol in [(torch.complex128, 1e-10), (torch.complex64, 1e-4)]:
                v = torch.from_numpy(vin).to("cuda").to(dtype)
                out = f.apply_unitary(v, op, norb, (nocc, nocc))
                np.testing.assert_allclose(out.cpu().numpy().astype(complex), golden[f"t2{idx}_op{tag}_out"],
                                           atol=tol)
