"""Diagonal Coulomb Hamiltonian (python/ffsim/hamiltonians/diagonal_coulomb_hamiltonian.py)
and its split-operator Trotter evolution (python/ffsim/trotter/diagonal_coulomb_split_op.py):
the oracle against the reference's golden vectors on the CPU, the GPU path
against both."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import ffsim_oracle as o


def _dch(g, key, idx):
    return g[f"{key}{idx}_h1"], g[f"{key}{idx}_dcm"], float(g[f"{key}{idx}_const"])


def test_oracle_matvec_and_diag_golden(golden):
    for idx, (n, a, b) in enumerate(golden["dch_cases"]):
        n, ne = int(n), (int(a), int(b))
        h1, dcm, c = _dch(golden, "dch", idx)
        v = golden[f"dch{idx}_in"]
        np.testing.assert_allclose(o.diag_coulomb_hamiltonian_action(v, h1, dcm, c, n, ne),
                                   golden[f"dch{idx}_matvec"], atol=1e-12)
        np.testing.assert_allclose(o.diag_coulomb_hamiltonian_diag(h1, dcm, c, n, ne),
                                   golden[f"dch{idx}_diag"], atol=1e-12)


def test_oracle_diag_is_operator_diagonal():
    """The diagonal equals <e_i|H|e_i> of the operator itself (n=4, (2,1))."""
    rng = np.random.default_rng(3)
    n, ne = 4, (2, 1)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    h1 = (g + g.conj().T) / 2
    dcm = np.stack([o.random_symmetric_normal(n, seed=rng), o.random_symmetric_normal(n, seed=rng)])
    d = o.dim(n, ne)
    cols = np.stack([o.diag_coulomb_hamiltonian_action(np.eye(d)[i], h1, dcm, 0.25, n, ne) for i in range(d)], 1)
    np.testing.assert_allclose(np.diag(cols).real, o.diag_coulomb_hamiltonian_diag(h1, dcm, 0.25, n, ne),
                               atol=1e-12)
    np.testing.assert_allclose(cols, cols.conj().T, atol=1e-12)


def test_oracle_split_op_golden(golden):
    for idx, (n, a, b, t, steps, order) in enumerate(golden["split_cases"]):
        n, ne = int(n), (int(a), int(b))
        h1, dcm, c = _dch(golden, "split", idx)
        got = o.simulate_trotter_diag_coulomb_split_op(golden[f"split{idx}_in"], h1, dcm, c, float(t), n, ne,
                                                        n_steps=int(steps), order=int(order))
        np.testing.assert_allclose(got, golden[f"split{idx}_out"], atol=1e-12)


def test_oracle_split_op_converges():
    """With many steps the split-operator evolution approaches exp(-iTH)
    (the reference's trotter/diag_coulomb_split_op_test.py:32-84 checks the same)."""
    import scipy.linalg

    rng = np.random.default_rng(11)
    n, ne = 4, (2, 1)
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    h1 = (g + g.conj().T) / 2
    dcm = np.stack([o.random_symmetric_normal(n, seed=rng), o.random_symmetric_normal(n, seed=rng)])
    d = o.dim(n, ne)
    hmat = np.stack([o.diag_coulomb_hamiltonian_action(np.eye(d)[i], h1, dcm, 0.3, n, ne) for i in range(d)], 1)
    v = o.random_state_vector(d, seed=rng)
    exact = scipy.linalg.expm(-1j * 0.5 * hmat) @ v
    got = o.simulate_trotter_diag_coulomb_split_op(v, h1, dcm, 0.3, 0.5, n, ne, n_steps=40, order=1)
    assert abs(np.vdot(exact, got)) > 1 - 1e-4


def test_argument_errors():
    import ffsim_gb300 as f

    ham = f.DiagonalCoulombHamiltonian(np.eye(4), np.zeros((2, 4, 4)))
    with pytest.raises(ValueError):
        f.simulate_trotter_diag_coulomb_split_op(np.zeros(36, dtype=complex), ham, 0.1, norb=4, nelec=(2, 2),
                                                 order=-1)
    with pytest.raises(ValueError):
        f.simulate_trotter_diag_coulomb_split_op(np.zeros(36, dtype=complex), ham, 0.1, norb=4, nelec=(2, 2),
                                                 n_steps=-1)


def test_approx_eq():
    import ffsim_gb300 as f

    a = f.DiagonalCoulombHamiltonian(np.eye(3), np.ones((2, 3, 3)), constant=1.0)
    b = f.DiagonalCoulombHamiltonian(np.eye(3) + 1e-12, np.ones((2, 3, 3)), constant=1.0)
    c = f.DiagonalCoulombHamiltonian(np.eye(3), np.ones((2, 3, 3)), constant=1.5)
    assert a._approx_eq_(b, rtol=1e-9, atol=1e-9)
    assert not a._approx_eq_(c, rtol=1e-9, atol=1e-9)
    assert a._approx_eq_(object(), rtol=1e-9, atol=1e-9) is NotImplemented


@pytest.mark.gpu
def test_gpu_linear_operator_and_diag_golden(cuda, golden):
    import torch

    import ffsim_gb300 as f

    for idx, (n, a, b) in enumerate(golden["dch_cases"]):
        n, ne = int(n), (int(a), int(b))
        h1, dcm, c = _dch(golden, "dch", idx)
        ham = f.DiagonalCoulombHamiltonian(h1, dcm, constant=c)
        lin = f.linear_operator(ham, n, ne)
        v = golden[f"dch{idx}_in"]
        np.testing.assert_allclose(lin @ v, golden[f"dch{idx}_matvec"], atol=1e-11)
        got64 = (lin @ torch.from_numpy(v).to("cuda").to(torch.complex64)).cpu().numpy()
        np.testing.assert_allclose(got64, golden[f"dch{idx}_matvec"], atol=1e-4)
        np.testing.assert_allclose(f.diag(ham, n, ne), golden[f"dch{idx}_diag"], atol=1e-11)
        assert abs(f.trace(ham, n, ne) - golden[f"dch{idx}_diag"].sum()) < 1e-9
        e = lin.expectation(v)
        assert abs(e - float(np.vdot(v, golden[f"dch{idx}_matvec"]).real)) < 1e-10


@pytest.mark.gpu
def test_gpu_split_op_golden(cuda, golden):
    import torch

    import ffsim_gb300 as f

    for idx, (n, a, b, t, steps, order) in enumerate(golden["split_cases"]):
        n, ne = int(n), (int(a), int(b))
        h1, dcm, c = _dch(golden, "split", idx)
        ham = f.DiagonalCoulombHamiltonian(h1, dcm, constant=c)
        vin = golden[f"split{idx}_in"]
        for dtype, tol in [(torch.complex128, 1e-11), (torch.complex64, 1e-4)]:
            v = torch.from_numpy(vin).to("cuda").to(dtype)
            keep = v.clone()
            out = f.simulate_trotter_diag_coulomb_split_op(v, ham, float(t), norb=n, nelec=ne,
                                                           n_steps=int(steps), order=int(order))
            assert torch.equal(v, keep)
            np.testing.assert_allclose(out.cpu().numpy().astype(complex), golden[f"split{idx}_out"], atol=tol)


@pytest.mark.gpu
def test_gpu_split_op_stage_path(cuda):
    """norb=12 (6,6), a Hubbard chain, on the complex64 stage kernels and the
    complex128 sector kernel, against the oracle (about 6 s on one core)."""
    import torch

    import ffsim_gb300 as f

    norb, nelec = 12, (6, 6)
    h1 = np.zeros((norb, norb))
    for p in range(norb - 1):
        h1[p, p + 1] = h1[p + 1, p] = -1.0
    dcm = np.stack([np.zeros((norb, norb)), 4.0 * np.eye(norb)])
    ham = f.DiagonalCoulombHamiltonian(h1, dcm, constant=0.5)
    rng = np.random.default_rng(21)
    d = f.dim(norb, nelec)
    v = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    v /= np.linalg.norm(v)
    outs = {}
    for dtype in (torch.complex64, torch.complex128):
        t = torch.from_numpy(v).to("cuda").to(dtype)
        r = f.simulate_trotter_diag_coulomb_split_op(t, ham, 0.3, norb=norb, nelec=nelec, n_steps=3, order=1)
        outs[dtype] = r.cpu().numpy().astype(complex)
    exp = o.simulate_trotter_diag_coulomb_split_op(v, h1, dcm, 0.5, 0.3, norb, nelec, n_steps=3, order=1)
    assert np.linalg.norm(outs[torch.complex128] - exp) < 1e-10
    assert np.linalg.norm(outs[torch.complex64] - exp) < 1e-4
    # the evolution nearly conserves the energy (the oracle's drift is 6.7e-5)
    lin = f.linear_operator(ham, norb, nelec)
    assert abs(lin.expectation(outs[torch.complex128]) - lin.expectation(v)) < 1e-3


def test_split_op_host_sequence(golden, monkeypatch):
    """The host-side step logic of the GPU evolution (basis products, skipped
    identity rotations, the closing phase) with the two gate entry points
    replaced by the oracle's, against the reference's golden vectors."""
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _state
    from ffsim_gb300 import trotter as tr

    def rot(state, mat, norb, nelec, copy=False):
        return torch.from_numpy(o.apply_orbital_rotation(state.numpy(), mat, norb, nelec))

    def evo(state, mat, t, norb, nelec, copy=False):
        return torch.from_numpy(o.apply_diag_coulomb_evolution(state.numpy(), mat, t, norb, nelec))

    def prep(vec, norb, nelec, *, copy):
        arr = np.array(vec, dtype=complex)
        return _state.Prepared(torch.from_numpy(arr), arr.shape, True)

    calls = []
    monkeypatch.setattr(tr, "apply_orbital_rotation", lambda *a, **k: calls.append("rot") or rot(*a, **k))
    monkeypatch.setattr(tr, "apply_diag_coulomb_evolution", evo)
    monkeypatch.setattr(tr, "prepare", prep)
    for idx, (n, a, b, t, steps, order) in enumerate(golden["split_cases"]):
        n, ne = int(n), (int(a), int(b))
        h1, dcm, c = _dch(golden, "split", idx)
        ham = f.DiagonalCoulombHamiltonian(h1, dcm, constant=c)
        calls.clear()
        out = tr.simulate_trotter_diag_coulomb_split_op(golden[f"split{idx}_in"], ham, float(t), norb=n, nelec=ne,
                                                        n_steps=int(steps), order=int(order))
        np.testing.assert_allclose(np.asarray(out).reshape(-1), golden[f"split{idx}_out"], atol=1e-12)
        if int(order) == 0:  # one rotation per step; the closing identity is skipped
            assert len(calls) == int(steps)
