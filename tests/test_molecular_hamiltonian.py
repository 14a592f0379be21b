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
