"""Batches of states under one Hamiltonian (ffgb_batch_df_matvec,
ffgb_batch_lucj_energy, the batched gradient): against the per-state entry
points, and a state's result alone against the same state inside a batch.

complex64 with 9 <= norb <= 16 runs every Hamiltonian term once over all the
states side by side (each padded to whole 128-column tiles); other shapes run
state by state.  The shapes below include sectors of 126, 252, 330 and 462
strings, so the padding varies.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STACKED = [(9, (4, 5)), (10, (5, 5)), (11, (5, 4))]


def _states(n, d, dtype, seed, cuda):
    import torch

    gen = torch.Generator(device="cpu").manual_seed(seed)
    v = torch.randn((n, d), dtype=torch.complex128, generator=gen)
    v /= torch.linalg.vector_norm(v, dim=1, keepdim=True)
    return v.to(dtype).to(cuda)


@pytest.mark.parametrize("norb, nelec", STACKED + [(6, (3, 3))])
@pytest.mark.parametrize("dtype_name", ["complex64", "complex128"])
def test_batch_matvec_matches_per_state(cuda, norb, nelec, dtype_name):
    import torch

    import ffsim_gb300 as f

    dtype = getattr(torch, dtype_name)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=3, seed=norb)
    lin = f.linear_operator(ham, norb, nelec)
    x = _states(5, f.dim(norb, nelec), dtype, norb, cuda)
    got = lin @ x.T  # (dim, 5): one batched call
    tol = 2e-5 if dtype == torch.complex64 else 1e-11
    for b in range(5):
        want = lin @ x[b]
        err = float((got[:, b] - want).abs().max()) / float(want.abs().max())
        assert err <= tol, (b, err)


@pytest.mark.parametrize("norb, nelec", [(10, (5, 5)), (12, (6, 6)), (14, (7, 6))])
def test_stage_path_matvec_matches_complex128(cuda, norb, nelec):
    """complex64 matvecs on the stage path, one state and three side by side,
    against complex128: each term's W(U) Z W(U^dag) runs with the phases of
    the U^dag plan carried by the plan of U diag(d) and the last row phases
    fused into the accumulation."""
    import torch

    import ffsim_gb300 as f

    ham = f.random.random_df_hamiltonian_normal(norb, rank=3, seed=40 + norb)
    lin = f.linear_operator(ham, norb, nelec)
    x = _states(3, f.dim(norb, nelec), torch.complex128, norb, cuda)
    want = torch.stack([lin @ x[b] for b in range(3)])
    one = lin @ x[0].to(torch.complex64)
    many = (lin @ x.to(torch.complex64).T).T
    scale = float(torch.linalg.vector_norm(want[0]))
    assert float(torch.linalg.vector_norm(one.to(torch.complex128) - want[0])) <= 1e-5 * scale
    for b in range(3):
        err = float(torch.linalg.vector_norm(many[b].to(torch.complex128) - want[b]))
        assert err <= 1e-5 * float(torch.linalg.vector_norm(want[b])), (b, err)


@pytest.mark.parametrize("norb, nelec", STACKED + [(8, (4, 4))])
@pytest.mark.parametrize("dtype_name", ["complex64", "complex128"])
def test_batch_energy_matches_per_state(cuda, norb, nelec, dtype_name):
    import torch

    import ffsim_gb300 as f

    dtype = getattr(torch, dtype_name)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=4, seed=norb + 1)
    ops = [f.random.random_ucj_op_spin_balanced(norb, n_reps=2, diag_coulomb_normal=True, diag_coulomb_scale=0.1,
                                                seed=100 + k, with_final_orbital_rotation=(k == 1))
           for k in range(3)]
    got = f.lucj_energies(ops, ham, norb, nelec, dtype=dtype)
    tol = 1e-6 if dtype == torch.complex64 else 1e-10
    for k, op in enumerate(ops):
        want = f.lucj_energy(op, ham, norb, nelec, dtype=dtype)
        assert abs(got[k] - want) <= tol, (k, got[k], want)


@pytest.mark.parametrize("norb, nelec", [(13, (6, 7)), (14, (7, 7)), (16, (8, 7))])
def test_stage_path_energies_match_complex128(cuda, norb, nelec):
    """For 13-16 orbitals (five-stage plans, windows of 6-8 orbitals) the
    complex64 energies of the stage path, alone and in a batch, against the
    complex128 path (sector kernel, no stage kernels)."""
    import torch

    import ffsim_gb300 as f

    ham = f.random.random_df_hamiltonian_normal(norb, rank=3, seed=norb + 7)
    ops = [f.random.random_ucj_op_spin_balanced(norb, n_reps=1, diag_coulomb_normal=True, diag_coulomb_scale=0.1,
                                                seed=300 + k) for k in range(2)]
    want = [f.lucj_energy(op, ham, norb, nelec, dtype=torch.complex128) for op in ops]
    single = [f.lucj_energy(op, ham, norb, nelec, dtype=torch.complex64) for op in ops]
    batch = f.lucj_energies(ops, ham, norb, nelec, dtype=torch.complex64)
    for k in range(2):
        assert abs(single[k] - want[k]) <= 1e-6, (k, single[k], want[k])
        assert abs(batch[k] - want[k]) <= 1e-6, (k, batch[k], want[k])


def test_batch_energy_alone_equals_in_batch(cuda):
    """A state's energy does not depend on the other states of its batch."""
    import torch

    import ffsim_gb300 as f

    norb, nelec = 12, (6, 6)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=6, seed=5)
    ops = [f.random.random_ucj_op_spin_balanced(norb, n_reps=2, diag_coulomb_normal=True, diag_coulomb_scale=0.1,
                                                seed=200 + k) for k in range(4)]
    ev = f.BatchLUCJEnergy(norb, nelec, 4, dtype=torch.complex64)
    together = ev(ops, ham)
    for k, op in enumerate(ops):
        alone = ev([op], ham)[0]
        assert abs(alone - together[k]) <= 1e-12, (k, alone, together[k])


def test_batched_gradient_matches_per_vector(cuda):
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300.gradient import LUCJGradient

    norb, nelec, n_reps = 10, (5, 5), 2
    ham = f.random.random_df_hamiltonian_normal(norb, rank=5, seed=9)
    rng = np.random.default_rng(9)
    params = rng.normal(scale=0.3, size=(3, f.UCJOpSpinBalanced.n_params(norb, n_reps)))
    ev = LUCJGradient(norb, nelec, dtype=torch.complex64)
    energies, grads = ev.value_and_grad_batch(params, n_reps, ham)
    for b in range(3):
        e, g = ev.value_and_grad(params[b], n_reps, ham)
        assert abs(energies[b] - e) <= 1e-6
        assert np.linalg.norm(grads[b] - g) <= 1e-5 * np.linalg.norm(g)


def _batch_inputs(norb, n, seed):
    import ffsim_gb300 as f

    ham = f.random.random_df_hamiltonian_normal(norb, rank=norb, seed=seed)
    ops = [f.random.random_ucj_op_spin_balanced(norb, n_reps=1, diag_coulomb_normal=True, diag_coulomb_scale=0.1,
                                                seed=seed + k) for k in range(n)]
    return ham, ops


def test_batch_deadline_and_cancel(cuda):
    """A deadline that has passed and a cancellation set beforehand both stop
    the batch with their own error; the stream and the evaluator stay usable
    and the next call gives the right energies."""
    import concurrent.futures

    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib

    norb, nelec = 10, (5, 5)
    ham, ops = _batch_inputs(norb, 3, 31)
    ev = f.BatchLUCJEnergy(norb, nelec, 3, dtype=torch.complex64)
    want = ev(ops, ham)
    with pytest.raises(TimeoutError):
        ev(ops, ham, control=_lib.Control(timeout_s=1e-9))
    ctl = _lib.Control()
    ctl.request_cancel()
    with pytest.raises(concurrent.futures.CancelledError):
        ev(ops, ham, control=ctl)
    np.testing.assert_allclose(ev(ops, ham), want, rtol=0, atol=1e-12)
    # an unset control changes nothing
    np.testing.assert_allclose(ev(ops, ham, control=_lib.Control(timeout_s=600)), want, rtol=0, atol=1e-12)


def test_batch_cancel_from_another_thread(cuda):
    """A running batch is cancelled by another thread: the call returns
    CancelledError within about two Hamiltonian terms of the request."""
    import concurrent.futures
    import threading
    import time

    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib

    norb, nelec = 14, (7, 7)
    ham, ops = _batch_inputs(norb, 6, 41)
    ev = f.BatchLUCJEnergy(norb, nelec, 6, dtype=torch.complex64)
    ev(ops[:1], ham)  # tables and buffers
    torch.cuda.synchronize()
    ctl = _lib.Control()
    timer = threading.Timer(0.05, ctl.request_cancel)
    t0 = time.perf_counter()
    timer.start()
    try:
        ev(ops, ham, control=ctl)
        finished = True
    except concurrent.futures.CancelledError:
        finished = False
    elapsed = time.perf_counter() - t0
    timer.join()
    if not finished:  # cancelled: well before the batch would have ended
        assert elapsed < 5.0
    torch.cuda.synchronize()
    assert np.all(np.isfinite(ev(ops[:2], ham)))
