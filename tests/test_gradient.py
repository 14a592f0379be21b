"""Adjoint gradient of the LUCJ energy against central finite differences of
the complex128 energy (h = 1e-5, FP64)."""

from __future__ import annotations

import numpy as np
import pytest


def test_dexp_matches_finite_differences():
    scipy_linalg = pytest.importorskip("scipy.linalg")
    from ffsim_gb300.gradient import _antihermitian_basis, _dexp
    from ffsim_gb300.linalg import antihermitians_from_parameters

    rng = np.random.default_rng(3)
    norb = 5
    K = antihermitians_from_parameters(rng.normal(scale=0.7, size=norb * norb), norb, 1)[0]
    basis = _antihermitian_basis(norb)
    got = _dexp(K, basis)
    h = 1e-6
    for n in range(0, norb * norb, 3):
        fd = (scipy_linalg.expm(K + h * basis[n]) - scipy_linalg.expm(K - h * basis[n])) / (2 * h)
        np.testing.assert_allclose(got[n], fd, atol=1e-8)


def _setup(norb, n_reps, rank, seed, with_final):
    import ffsim_gb300 as f

    rng = np.random.default_rng(seed)
    n = f.UCJOpSpinBalanced.n_params(norb, n_reps, with_final_orbital_rotation=with_final)
    params = rng.normal(scale=0.4, size=n)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=rank, seed=seed + 1)
    return params, ham


def _energy(params, norb, nelec, n_reps, ham, with_final, dtype):
    import ffsim_gb300 as f

    op = f.UCJOpSpinBalanced.from_parameters(params, norb=norb, n_reps=n_reps,
                                             with_final_orbital_rotation=with_final)
    return f.lucj_energy(op, ham, norb, nelec, dtype=dtype)


@pytest.mark.gpu
@pytest.mark.parametrize("with_final", [False, True])
def test_gradient_small_full(cuda, with_final):
    import torch

    from ffsim_gb300.gradient import LUCJGradient

    norb, nelec, n_reps = 6, (3, 3), 2
    params, ham = _setup(norb, n_reps, 4, 11, with_final)
    h = 1e-5
    fd = np.array([
        (_energy(params + h * e, norb, nelec, n_reps, ham, with_final, torch.complex128)
         - _energy(params - h * e, norb, nelec, n_reps, ham, with_final, torch.complex128)) / (2 * h)
        for e in np.eye(len(params))])
    e128 = _energy(params, norb, nelec, n_reps, ham, with_final, torch.complex128)
    for dtype, tol in [(torch.complex128, 1e-6), (torch.complex64, 1e-4)]:
        ev = LUCJGradient(norb, nelec, dtype=dtype)
        e, g = ev.value_and_grad(params, n_reps, ham, with_final_orbital_rotation=with_final)
        assert abs(e - e128) < (1e-10 if dtype == torch.complex128 else 1e-5)
        rel = np.linalg.norm(g - fd) / np.linalg.norm(fd)
        assert rel < tol, (dtype, rel)


@pytest.mark.gpu
def test_gradient_norb12_directional(cuda):
    """norb=12, (6,6), three repetitions, rank 24: directional derivatives of
    two parameter vectors along random directions."""
    import torch

    from ffsim_gb300.gradient import LUCJGradient

    norb, nelec, n_reps = 12, (6, 6), 3
    params0, ham = _setup(norb, n_reps, 24, 21, False)
    rng = np.random.default_rng(5)
    ev = LUCJGradient(norb, nelec, dtype=torch.complex64)
    h = 1e-5
    for b in range(2):
        params = params0 + 0.1 * b * rng.normal(size=len(params0))
        _, g = ev.value_and_grad(params, n_reps, ham)
        for _ in range(2):
            d = rng.normal(size=len(params))
            d /= np.linalg.norm(d)
            fd = (_energy(params + h * d, norb, nelec, n_reps, ham, False, torch.complex128)
                  - _energy(params - h * d, norb, nelec, n_reps, ham, False, torch.complex128)) / (2 * h)
            assert abs(g @ d - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.linalg.norm(g)), (g @ d, fd)


@pytest.mark.gpu
def test_a_failing_lane_raises_and_the_evaluator_stays_usable(cuda):
    """A state whose backward pass raises on one worker lane: the batch call
    raises that error once every lane has finished, and the next batch on the
    same evaluator gives the same results as before."""
    import torch

    from ffsim_gb300.gradient import LUCJGradient

    norb, nelec, n_reps = 6, (3, 3), 2
    p0, ham = _setup(norb, n_reps, 3, 41, False)
    params = np.stack([p0, 0.5 * p0, -0.3 * p0, 0.8 * p0, 0.1 * p0])
    ev = LUCJGradient(norb, nelec, dtype=torch.complex64, workers=3)
    e_ref, g_ref = ev.value_and_grad_batch(params, n_reps, ham)
    orig = ev._backward

    def failing(cur, lam, V, jaa, jab, L):
        if cur.data_ptr() == ev._bcur[1].data_ptr():
            raise RuntimeError("lane failure")
        return orig(cur, lam, V, jaa, jab, L)

    ev._backward = failing
    with pytest.raises(RuntimeError, match="lane failure"):
        ev.value_and_grad_batch(params, n_reps, ham)
    ev._backward = orig
    e2, g2 = ev.value_and_grad_batch(params, n_reps, ham)
    assert np.array_equal(e2, e_ref) and np.array_equal(g2, g_ref)


@pytest.mark.gpu
def test_autograd_function_batch(cuda):
    import torch

    from ffsim_gb300.gradient import LUCJGradient, lucj_energy_autograd

    norb, nelec, n_reps = 6, (3, 3), 1
    params, ham = _setup(norb, n_reps, 3, 31, False)
    batch = torch.tensor(np.stack([params, params * 0.5, params * -0.3]), dtype=torch.float64,
                         requires_grad=True)
    ev = LUCJGradient(norb, nelec, dtype=torch.complex128)
    energies = lucj_energy_autograd(batch, ev, n_reps, ham)
    assert energies.shape == (3,)
    energies.sum().backward()
    energies = energies.detach()
    for row in range(3):
        e, g = ev.value_and_grad(batch[row].detach().numpy(), n_reps, ham)
        assert abs(energies[row].item() - e) < 1e-12
        np.testing.assert_allclose(batch.grad[row].numpy(), g, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("norb,nelec", [(6, (3, 2)), (8, (4, 4)), (12, (6, 6)), (14, (7, 7))])
def test_gate_densities_match_the_single_density_calls(cuda, norb, nelec):
    """ffgb_gate_densities (both densities of a gate into device memory, one
    pair of transposes, no synchronization) equals ffgb_transition_rdm1 and
    ffgb_pair_density, in both precisions and on the small-sector and
    large-sector transition-density kernels (norb 14 is a large sector)."""
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib
    from ffsim_gb300._state import scratch

    rng = np.random.default_rng(norb)
    d = f.dim(norb, nelec)
    n2 = norb * norb
    for dtype, code in ((torch.complex64, _lib.FFGB_C64), (torch.complex128, _lib.FFGB_C128)):
        if norb == 14 and dtype == torch.complex128:
            continue
        x = torch.from_numpy(rng.standard_normal(d) + 1j * rng.standard_normal(d)).to("cuda").to(dtype)
        y = torch.from_numpy(rng.standard_normal(d) + 1j * rng.standard_normal(d)).to("cuda").to(dtype)
        buf, nbytes = scratch(x, 3, norb, *nelec)
        st = torch.cuda.current_stream().cuda_stream
        g = np.zeros(4 * n2)
        p = np.zeros(6 * n2)
        _lib.call("ffgb_transition_rdm1", x.data_ptr(), y.data_ptr(), code, norb, *nelec, _lib.dptr(g),
                  buf.data_ptr(), nbytes, st)
        _lib.call("ffgb_pair_density", x.data_ptr(), y.data_ptr(), code, norb, *nelec, _lib.dptr(p),
                  buf.data_ptr(), nbytes, st)
        for pair in (0, 1):
            out = torch.full((10 * n2,), np.nan, dtype=torch.float64, device="cuda")
            _lib.call("ffgb_gate_densities", x.data_ptr(), y.data_ptr(), code, norb, *nelec, pair,
                      out.data_ptr(), buf.data_ptr(), nbytes, st)
            h = out.cpu().numpy()
            np.testing.assert_array_equal(h[: 4 * n2], g)
            if pair:
                np.testing.assert_array_equal(h[4 * n2:], p)
            else:
                assert np.isnan(h[4 * n2:]).all()


def test_batched_circuits_and_chain_rule_on_the_host():
    """The gradient's host side: the circuit's rotations equal expm of the
    parameters' antihermitian matrices; the chain rule's dexp adjoint is the
    adjoint of dexp; and a state's circuit and chain rule are bit-identical
    alone and inside a batch."""
    scipy_linalg = pytest.importorskip("scipy.linalg")

    import ffsim_gb300 as f
    from ffsim_gb300.gradient import GradientHost, _dexp, _dexp_adjoint
    from ffsim_gb300.linalg import antihermitians_from_parameters

    norb, L = 5, 2
    g = GradientHost(norb)
    rng = np.random.default_rng(9)
    n = f.UCJOpSpinBalanced.n_params(norb, L, with_final_orbital_rotation=True)
    P = rng.normal(scale=0.5, size=(4, n))
    batch = g._circuits(P, L, True)
    op = f.UCJOpSpinBalanced.from_parameters(P[2], norb=norb, n_reps=L, with_final_orbital_rotation=True)
    U, Uf = batch[2][0], batch[2][1]
    for k in range(L):
        np.testing.assert_allclose(U[k + 1], op.orbital_rotations[k], atol=1e-13)
        np.testing.assert_allclose(batch[2][3][k + 1], op.diag_coulomb_mats[k, 0], atol=0)
        np.testing.assert_allclose(batch[2][4][k + 1], op.diag_coulomb_mats[k, 1], atol=0)
    np.testing.assert_allclose(Uf, op.final_orbital_rotation, atol=1e-13)
    # adjoint of dexp
    K = antihermitians_from_parameters(P[0, : norb * norb], norb, 1)[0]
    w, W = np.linalg.eigh(-1j * K)
    gam = rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb))
    G = _dexp_adjoint(w[None], W[None], gam[None])[0]
    for dK in g.basis[::3]:
        lhs = np.sum(_dexp(K, dK[None])[0] * gam).real
        assert abs(lhs - np.sum(dK * G).real) < 1e-12
    np.testing.assert_allclose(scipy_linalg.expm(K), W @ np.diag(np.exp(1j * w)) @ W.conj().T, atol=1e-13)
    # alone and in a batch
    dens = [([None] + [rng.normal(size=(norb, norb)) + 1j * rng.normal(size=(norb, norb)) for _ in range(L + 1)],
             [None] + [rng.normal(size=(3, norb, norb)) + 1j * rng.normal(size=(3, norb, norb)) for _ in range(L)])
            for _ in range(4)]
    grads = g._chains(n, batch, dens, L, True)
    for b in range(4):
        alone = g._circuits(P[b:b + 1], L, True)
        for a, c in zip(alone[0][:2], batch[b][:2]):
            assert np.array_equal(np.asarray(a), np.asarray(c))
        assert np.array_equal(g._chains(n, alone, [dens[b]], L, True)[0], grads[b])
