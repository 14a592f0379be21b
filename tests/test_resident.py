"""Resident evaluator (persistent kernel, host-mapped work queue): energies
against the complex128 path and the FP64 oracle, gradients against the batch
path and finite differences, results independent of the mix, the bounded
wait for work, cancellation and a full queue."""

from __future__ import annotations

import time
from concurrent.futures import CancelledError

import numpy as np
import pytest
import torch

import ffsim_gb300 as f
from ffsim_gb300 import resident
from oracle import ffsim_oracle as o

pytestmark = pytest.mark.gpu

SHAPES = [(8, (4, 4), 1), (8, (4, 4), 2), (8, (4, 4), 3), (8, (5, 3), 2), (7, (3, 4), 2), (6, (3, 3), 4),
          (4, (2, 1), 1), (2, (1, 1), 2), (1, (1, 0), 1)]


def _case(norb, n_reps, seed, final=False):
    ucj = f.random.random_ucj_op_spin_balanced(norb, n_reps=n_reps, diag_coulomb_normal=True,
                                               diag_coulomb_scale=0.1, with_final_orbital_rotation=final,
                                               seed=seed)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=2 * norb, seed=seed + 1000)
    return ucj, ham


@pytest.fixture(scope="module")
def ev():
    r = resident.ResidentEvaluator(n_slots=512, n_ctas=8, idle_seconds=2.0)
    yield r
    r.close()


@pytest.mark.parametrize("norb,nelec,n_reps", SHAPES)
def test_matches_complex128_path(ev, norb, nelec, n_reps):
    ucj, ham = _case(norb, n_reps, seed=10 * norb + n_reps, final=(norb % 2 == 0))
    e_res = ev.wait(ev.submit(ucj, ham, nelec))
    e128 = f.lucj_energy(ucj, ham, norb, nelec, dtype=torch.complex128)
    assert abs(e_res - e128) <= 1e-6, (e_res, e128)


def test_matches_oracle():
    norb, nelec = 4, (2, 2)
    ucj, ham = _case(norb, 2, seed=77, final=True)
    psi = o.ucj_spin_balanced_apply(o.hartree_fock_state(norb, nelec), ucj.diag_coulomb_mats,
                                    ucj.orbital_rotations, ucj.final_orbital_rotation, norb, nelec)
    e_ref = o.df_energy(psi, ham.one_body_tensor, ham.diag_coulomb_mats, ham.orbital_rotations, ham.constant,
                        norb, nelec)
    r = resident.ResidentEvaluator(n_slots=4, n_ctas=1, idle_seconds=1.0)
    try:
        e = r.wait(r.submit(ucj, ham, nelec))
    finally:
        r.close()
    assert abs(e - e_ref) <= 1e-6


def test_same_result_alone_and_in_a_mixed_queue(ev):
    """Requests of several shapes and two Hamiltonians per shape, interleaved:
    each energy equals that of the same request alone, bit for bit."""
    cases = []
    for i in range(24):
        norb, nelec, n_reps = SHAPES[i % 4]
        ucj, ham = _case(norb, n_reps, seed=500 + i)
        cases.append((ucj, ham, nelec))
    alone = [ev.wait(ev.submit(u, h, ne)) for u, h, ne in cases]
    tickets = [ev.submit(u, h, ne) for u, h, ne in cases]
    mixed = [ev.wait(t) for t in tickets]
    assert mixed == alone


def test_wait_for_work_is_bounded_and_the_kernel_restarts():
    """No request within the idle limit: every CTA's wait runs out, the kernel
    exits with FFGB_ERR_TIMEOUT, and the next request launches it again."""
    r = resident.ResidentEvaluator(n_slots=8, n_ctas=4, idle_seconds=0.05)
    try:
        r.start()
        deadline = time.perf_counter() + 10.0
        while r.status()[0] and time.perf_counter() < deadline:
            time.sleep(0.01)
        running, status = r.status()
        assert not running
        assert status == 5  # FFGB_ERR_TIMEOUT
        ucj, ham = _case(6, 2, seed=3)
        e = r.wait(r.submit(ucj, ham, (3, 3)))
        assert abs(e - f.lucj_energy(ucj, ham, 6, (3, 3), dtype=torch.complex128)) <= 1e-6
    finally:
        r.close()


def test_cancel_a_queued_request():
    """One CTA serves the queue in order, so the last of many requests is still
    queued when it is cancelled: it ends cancelled, the others finish."""
    r = resident.ResidentEvaluator(n_slots=64, n_ctas=1, idle_seconds=2.0)
    try:
        ucj, ham = _case(8, 3, seed=11)
        tickets = [r.submit(ucj, ham, (4, 4)) for _ in range(40)]
        r.cancel(tickets[-1])
        energies = [r.wait(t) for t in tickets[:-1]]
        assert len(set(energies)) == 1
        with pytest.raises(CancelledError):
            r.wait(tickets[-1])
    finally:
        r.close()


def test_full_queue_and_invalid_requests():
    r = resident.ResidentEvaluator(n_slots=3, n_ctas=2, idle_seconds=1.0)
    try:
        ucj, ham = _case(6, 1, seed=5)
        tickets = [r.submit(ucj, ham, (3, 3)) for _ in range(3)]
        with pytest.raises(MemoryError):
            r.submit(ucj, ham, (3, 3))
        r.wait(tickets[0])  # collecting frees a slot
        tickets.append(r.submit(ucj, ham, (3, 3)))
        vals = [r.wait(t) for t in tickets[1:]]
        assert len(set(vals)) == 1
        with pytest.raises(ValueError):
            r.poll(tickets[0])  # already collected
        big, hbig = _case(9, 1, seed=6)
        with pytest.raises(NotImplementedError):
            r.submit(big, hbig, (4, 5))
        deep, hdeep = _case(6, 5, seed=7)
        with pytest.raises(NotImplementedError):
            r.submit(deep, hdeep, (3, 3))
        with pytest.raises(ValueError):
            r.submit(ucj, ham, (7, 3))
    finally:
        r.close()


@pytest.mark.parametrize("norb,nelec,n_reps,final", [(6, (3, 3), 2, False), (8, (4, 4), 1, True), (5, (3, 2), 3, False)])
def test_gradient_matches_the_batch_path(ev, norb, nelec, n_reps, final):
    """The resident kernel's energy and adjoint gradient (the circuit, the
    Hamiltonian matvec and the backward pass on the device, the chain rule on
    the host) against LUCJGradient's."""
    from ffsim_gb300.gradient import LUCJGradient

    rng = np.random.default_rng(40 + norb)
    n = f.UCJOpSpinBalanced.n_params(norb, n_reps, with_final_orbital_rotation=final)
    params = rng.normal(scale=0.4, size=n)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=norb, seed=norb + 50)
    e, g = ev.wait_grad(ev.submit_grad(params, n_reps, ham, nelec, with_final_orbital_rotation=final))
    e_ref, g_ref = LUCJGradient(norb, nelec, dtype=torch.complex64).value_and_grad(
        params, n_reps, ham, with_final_orbital_rotation=final)
    assert abs(e - e_ref) <= 1e-6
    assert np.linalg.norm(g - g_ref) <= 1e-4 * np.linalg.norm(g_ref)


def test_gradient_against_finite_differences(ev):
    """Every coordinate of the resident gradient against central differences
    of the complex128 energy (h = 1e-5)."""
    norb, nelec, n_reps = 4, (2, 2), 2
    rng = np.random.default_rng(3)
    n = f.UCJOpSpinBalanced.n_params(norb, n_reps)
    params = rng.normal(scale=0.5, size=n)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=4, seed=8)
    _, g = ev.wait_grad(ev.submit_grad(params, n_reps, ham, nelec))

    def energy(p):
        op = f.UCJOpSpinBalanced.from_parameters(p, norb=norb, n_reps=n_reps)
        return f.lucj_energy(op, ham, norb, nelec, dtype=torch.complex128)

    h = 1e-5
    fd = np.array([(energy(params + h * np.eye(n)[i]) - energy(params - h * np.eye(n)[i])) / (2 * h)
                   for i in range(n)])
    assert np.linalg.norm(g - fd) <= 1e-4 * np.linalg.norm(fd)


def test_gradient_requests_mix_with_energies(ev):
    """Energies and gradients of several shapes in one queue: each equals the
    same request alone, bit for bit."""
    reqs = []
    for i in range(12):
        norb, nelec, n_reps = SHAPES[i % 4]
        ucj, ham = _case(norb, n_reps, seed=900 + i)
        if i % 3 == 0:
            reqs.append(("grad", ucj.to_parameters(), n_reps, ham, nelec))
        else:
            reqs.append(("energy", ucj, n_reps, ham, nelec))

    def submit(r):
        if r[0] == "grad":
            return ev.submit_grad(r[1], r[2], r[3], r[4])
        return ev.submit(r[1], r[3], r[4])

    def wait(r, t):
        if r[0] == "grad":
            e, g = ev.wait_grad(t)
            return (e, tuple(g))
        return ev.wait(t)

    alone = [wait(r, submit(r)) for r in reqs]
    tickets = [submit(r) for r in reqs]
    assert [wait(r, t) for r, t in zip(reqs, tickets)] == alone
