"""Molecular Hamiltonian (python/ffsim/hamiltonians/molecular_hamiltonian.py)
through its exact double-factorized form: the conversion on the CPU against the
oracle's definition, the GPU linear operator and energy against the same."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import ffsim_oracle as o

CASES = [(3, (1, 2), True), (4, (2, 2), True), (4, (2, 1), False), (5, (2, 2), True)]


def _ham(norb, complex_tensors, seed):
    import ffsim_gb300 as f

    rng = np.random.default_rng(seed)
    g = rng.standard_normal((norb, norb)) + (1j * rng.standard_normal((norb, norb)) if complex_tensors else 0)
    h1 = (g + g.conj().T) / 2
    h2 = o.random_two_body_tensor(norb, seed=rng)
    if not complex_tensors:  # real integrals with the eightfold symmetry
        h2 = h2.real
        h2 = (h2 + h2.transpose(1, 0, 2, 3)) / 2
        h2 = (h2 + h2.transpose(0, 1, 3, 2)) / 2
    return f.MolecularHamiltonian(h1, h2, constant=float(rng.standard_normal()))


@pytest.mark.parametrize("norb, nelec, cplx", CASES)
def test_exact_double_factorization(norb, nelec, cplx):
    ham = _ham(norb, cplx, norb * 10 + nelec[1])
    df = ham.to_double_factorized()
    assert df.diag_coulomb_mats.shape[0] <= 2 * norb**2
    vec = o.random_state_vector(o.dim(norb, nelec), seed=1)
    exp = o.molecular_hamiltonian_action(vec, ham.one_body_tensor, ham.two_body_tensor, ham.constant, norb, nelec)
    got = o.df_hamiltonian_matvec(df.one_body_tensor, df.diag_coulomb_mats, df.orbital_rotations, df.constant,
                                  norb, nelec)(vec)
    np.testing.assert_allclose(got, exp, atol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("norb, nelec, cplx", CASES)
def test_linear_operator(cuda, norb, nelec, cplx):
    import ffsim_gb300 as f

    ham = _ham(norb, cplx, norb * 10 + nelec[1])
    vec = o.random_state_vector(o.dim(norb, nelec), seed=2)
    exp = o.molecular_hamiltonian_action(vec, ham.one_body_tensor, ham.two_body_tensor, ham.constant, norb, nelec)
    lin = f.linear_operator(ham, norb, nelec)
    for dtype, tol in [(torch.complex128, 1e-9), (torch.complex64, 2e-4)]:
        t = torch.from_numpy(vec).to("cuda").to(dtype)
        np.testing.assert_allclose((lin @ t).cpu().numpy(), exp, atol=tol * max(1.0, np.abs(exp).max()))
        e = lin.expectation(t)
        assert abs(e - np.vdot(vec, exp).real) < tol * max(1.0, abs(e))


def _mol(g, idx):
    import ffsim_gb300 as f

    return f.MolecularHamiltonian(g[f"mol{idx}_h1"], g[f"mol{idx}_h2"], constant=float(g[f"mol{idx}_const"]))


def _df_tensor(mats, rots):
    return np.einsum("kij,kpi,kqi,krj,ksj->pqrs", mats, rots, rots.conj(), rots, rots.conj())


def test_modified_cholesky_golden(golden):
    import ffsim_gb300 as f

    for idx, norb in enumerate(golden["mol_cases"]):
        flat = golden[f"mol{idx}_h2"].reshape(norb**2, norb**2)
        np.testing.assert_allclose(f.linalg.modified_cholesky(flat, tol=1e-8), golden[f"mol{idx}_chol"], atol=1e-12)
        np.testing.assert_allclose(f.linalg.modified_cholesky(flat, tol=1e-8, max_vecs=2),
                                   golden[f"mol{idx}_chol_max2"], atol=1e-12)
    assert f.linalg.modified_cholesky(np.zeros((0, 0))).shape == (0, 0)


def test_double_factorized_golden(golden):
    """Coulomb matrices element by element; rotations up to the phase of each
    eigenvector (the operator does not depend on it), through the tensor."""
    import ffsim_gb300 as f

    for idx, norb in enumerate(golden["mol_cases"]):
        h2 = golden[f"mol{idx}_h2"]
        for tag, kw in [("c", {}), ("c3", {"max_vecs": 3}), ("e", {"cholesky": False}),
                        ("e3", {"cholesky": False, "max_vecs": 3})]:
            mats, rots = f.linalg.double_factorized(h2, tol=1e-8, **kw)
            gm, gr = golden[f"mol{idx}_df{tag}_mats"], golden[f"mol{idx}_df{tag}_rots"]
            np.testing.assert_allclose(mats, gm, atol=1e-10)
            np.testing.assert_allclose(np.abs(rots), np.abs(gr), atol=1e-8)
            np.testing.assert_allclose(_df_tensor(mats, rots), _df_tensor(gm, gr), atol=1e-10)
            if tag in ("c", "e"):  # untruncated: the factorization is exact
                np.testing.assert_allclose(_df_tensor(mats, rots), h2, atol=1e-7)


def test_double_factorized_errors():
    import ffsim_gb300 as f

    with pytest.raises(ValueError):
        f.linalg.double_factorized(np.zeros((2, 2, 2, 2), dtype=complex))
    with pytest.raises(NotImplementedError):
        f.linalg.double_factorized(np.zeros((2, 2, 2, 2)), optimize=True)
    mats, rots = f.linalg.double_factorized(np.zeros((0, 0, 0, 0)))
    assert mats.shape == rots.shape == (0, 0, 0)


def test_from_and_to_molecular_hamiltonian_golden(golden):
    import ffsim_gb300 as f

    for idx, norb in enumerate(golden["mol_cases"]):
        mol = _mol(golden, idx)
        for z in (0, 1):
            df = f.DoubleFactorizedHamiltonian.from_molecular_hamiltonian(mol, z_representation=bool(z))
            assert df.z_representation == bool(z)
            np.testing.assert_allclose(df.one_body_tensor, golden[f"mol{idx}_from{z}_h1"], atol=1e-10)
            assert abs(df.constant - float(golden[f"mol{idx}_from{z}_const"])) < 1e-10
            np.testing.assert_allclose(df.diag_coulomb_mats, golden[f"mol{idx}_from{z}_mats"], atol=1e-10)
            back = df.to_molecular_hamiltonian()
            np.testing.assert_allclose(back.one_body_tensor, golden[f"mol{idx}_back{z}_h1"], atol=1e-10)
            np.testing.assert_allclose(back.two_body_tensor, golden[f"mol{idx}_back{z}_h2"], atol=1e-10)
            # the round trip returns the molecular Hamiltonian (the factorization is exact)
            assert back._approx_eq_(mol, rtol=0, atol=1e-7)
            assert df._approx_eq_(df, rtol=0, atol=0) and df._approx_eq_(mol, rtol=0, atol=0) is NotImplemented


def test_rotated_golden(golden):
    for idx, norb in enumerate(golden["mol_cases"]):
        rot = _mol(golden, idx).rotated(golden[f"mol{idx}_u"])
        np.testing.assert_allclose(rot.one_body_tensor, golden[f"mol{idx}_rot_h1"], atol=1e-12)
        np.testing.assert_allclose(rot.two_body_tensor, golden[f"mol{idx}_rot_h2"], atol=1e-12)


@pytest.mark.parametrize("idx, nelec", [(0, (1, 2)), (1, (2, 2)), (2, (3, 1))])
def test_diagonal_mapping(golden, idx, nelec):
    """The diagonal of a real molecular Hamiltonian equals that of the diagonal
    Coulomb Hamiltonian with J^aa = J - K and J^ab = J (J_pr = h_pprr,
    K_pr = h_prrp), checked against the operator's own diagonal."""
    norb = int(golden["mol_cases"][idx])
    h1, h2, c = golden[f"mol{idx}_h1"], golden[f"mol{idx}_h2"], float(golden[f"mol{idx}_const"])
    d = o.dim(norb, nelec)
    exp = np.array([o.molecular_hamiltonian_action(np.eye(d)[i], h1, h2, c, norb, nelec)[i] for i in range(d)])
    jm, km = np.einsum("pprr->pr", h2), np.einsum("prrp->pr", h2)
    got = o.diag_coulomb_hamiltonian_diag(h1, np.stack([jm - km, jm]), c, norb, nelec)
    np.testing.assert_allclose(got, exp.real, atol=1e-12)


def test_diagonal_complex_raises():
    import ffsim_gb300 as f

    ham = f.MolecularHamiltonian(np.eye(2, dtype=complex), np.zeros((2, 2, 2, 2)))
    with pytest.raises(NotImplementedError):
        ham._diag_(2, (1, 1))


@pytest.mark.gpu
@pytest.mark.parametrize("idx, nelec", [(0, (1, 2)), (1, (2, 2)), (2, (3, 1))])
def test_gpu_diagonals(cuda, golden, idx, nelec):
    """Molecular and double-factorized diagonals on the GPU (diagonal
    contractions of the all-ones vector) against the operator's diagonal."""
    import ffsim_gb300 as f

    norb = int(golden["mol_cases"][idx])
    mol = _mol(golden, idx)
    d = o.dim(norb, nelec)
    exp = np.array([o.molecular_hamiltonian_action(np.eye(d)[i], mol.one_body_tensor, mol.two_body_tensor,
                                                   mol.constant, norb, nelec)[i] for i in range(d)]).real
    np.testing.assert_allclose(f.diag(mol, norb, nelec), exp, atol=1e-10)
    df = f.DoubleFactorizedHamiltonian.from_molecular_hamiltonian(mol)
    np.testing.assert_allclose(f.diag(df, norb, nelec), exp, atol=1e-7)
    assert abs(f.trace(mol, norb, nelec) - exp.sum()) < 1e-8
