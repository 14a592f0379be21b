"""One-body operators (python/ffsim/contract/one_body.py) and 1-RDMs
(python/ffsim/states/rdm.py) on the GPU against the oracle's definitions
(<a+_p a_q> evaluated string by string) and the Slater-determinant known answer."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import ffsim_oracle as o

CASES = [(4, (2, 2)), (5, (3, 2)), (3, (1, 2)), (2, (0, 1)), (6, (3, 3))]


def test_rdm_rank_errors():
    import ffsim_gb300 as f

    with pytest.raises(NotImplementedError):
        f.rdms(np.zeros(36, dtype=complex), 4, (2, 2), rank=3)


def test_oracle_rdm2_slater():
    """For a Slater determinant the same-spin 2-RDM is the antisymmetrised
    product of 1-RDMs and the opposite-spin one the plain product (Wick)."""
    norb, nelec = 4, (2, 1)
    u = o.random_unitary(norb, seed=9)
    psi = o.apply_orbital_rotation(o.hartree_fock_state(norb, nelec), u, norb, nelec)
    g = o.rdm1s(psi, norb, nelec)
    r2 = o.rdm2s(psi, norb, nelec, reorder=True)
    # <p+ r+ s q> = g[p,q] g[r,s] - g[p,s] g[r,q] (same spin), g_a[p,q] g_b[r,s] (ab)
    np.testing.assert_allclose(r2[0], np.einsum("pq,rs->pqrs", g[0], g[0]) - np.einsum("ps,rq->pqrs", g[0], g[0]),
                               atol=1e-12)
    np.testing.assert_allclose(r2[1], np.einsum("pq,rs->pqrs", g[0], g[1]), atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("norb, nelec", CASES)
def test_rdm1(cuda, norb, nelec):
    import ffsim_gb300 as f

    vec = o.random_state_vector(o.dim(norb, nelec), seed=norb * 7 + nelec[0])
    exp = o.rdm1s(vec, norb, nelec)
    for dtype, tol in [(torch.complex128, 1e-12), (torch.complex64, 1e-5)]:
        t = torch.from_numpy(vec).to("cuda").to(dtype)
        np.testing.assert_allclose(f.rdms(t, norb, nelec), exp, atol=tol)
        np.testing.assert_allclose(f.rdms(t, norb, nelec, spin_summed=True), exp.sum(0), atol=2 * tol)


@pytest.mark.gpu
def test_rdm1_slater_and_large(cuda):
    """Slater determinant W(U)|HF>: rdm1_sigma = conj(U_occ) U_occ^T, at norb=12 on the stage path."""
    import ffsim_gb300 as f

    norb, nelec = 12, (6, 5)
    u = o.random_unitary(norb, seed=5)
    for dtype, tol in [(torch.complex128, 1e-10), (torch.complex64, 1e-5)]:
        psi = f.hartree_fock_state(norb, nelec, dtype=dtype)
        psi = f.apply_orbital_rotation(psi, u, norb, nelec)
        rdm = f.rdms(psi, norb, nelec)
        for s, n in enumerate(nelec):
            np.testing.assert_allclose(rdm[s], np.conj(u[:, :n]) @ u[:, :n].T, atol=tol)


@pytest.mark.gpu
@pytest.mark.parametrize("norb, nelec", CASES)
def test_one_body_linop(cuda, norb, nelec):
    import ffsim_gb300 as f

    rng = np.random.default_rng(norb + 3 * nelec[1])
    m = rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))
    vec = o.random_state_vector(o.dim(norb, nelec), seed=rng)
    lin = f.contract.one_body_linop(m, norb, nelec)
    for dtype, tol in [(torch.complex128, 1e-11), (torch.complex64, 5e-5)]:
        t = torch.from_numpy(vec).to("cuda").to(dtype)
        np.testing.assert_allclose((lin @ t).cpu().numpy(), o.one_body_action(vec, m, norb, nelec), atol=tol)
        np.testing.assert_allclose(lin.rmatvec(t).cpu().numpy(), o.one_body_action(vec, m.conj().T, norb, nelec),
                                   atol=tol)
    np.testing.assert_allclose(f.contract.contract_one_body(vec, m, norb, nelec),
                               o.one_body_action(vec, m, norb, nelec), atol=1e-11)


@pytest.mark.gpu
@pytest.mark.parametrize("norb, nelec", [(4, (2, 2)), (3, (1, 2)), (2, (0, 1)), (1, (0, 0)), (5, (2, 2))])
def test_rdm2(cuda, norb, nelec):
    import ffsim_gb300 as f

    vec = o.random_state_vector(o.dim(norb, nelec), seed=norb * 3 + nelec[0])
    for reorder in (True, False):
        exp = o.rdm2s(vec, norb, nelec, reorder=reorder)
        exp1 = o.rdm1s(vec, norb, nelec)
        for dtype, tol in [(torch.complex128, 1e-12), (torch.complex64, 1e-5)]:
            t = torch.from_numpy(vec).to("cuda").to(dtype)
            r1, r2 = f.rdms(t, norb, nelec, rank=2, reorder=reorder)
            np.testing.assert_allclose(r1, exp1, atol=tol)
            np.testing.assert_allclose(r2, exp, atol=tol)
            s1, s2 = f.rdms(t, norb, nelec, rank=2, reorder=reorder, spin_summed=True)
            np.testing.assert_allclose(s1, exp1.sum(0), atol=2 * tol)
            np.testing.assert_allclose(s2, exp[0] + exp[1] + exp[1].transpose(2, 3, 0, 1) + exp[2], atol=4 * tol)
