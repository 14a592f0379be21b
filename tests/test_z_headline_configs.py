"""Parity at the sizes the throughput figures are quoted on.

* LUCJ energy, norb 16, (8, 8), n_reps 2, double-factorized rank 32 (the
  benchmark's seeds): complex64 against the FP64 (complex128) GPU path,
  |dE| <= 1e-6 Ha.  The complex128 path is pinned to the FP64 oracle at
  smaller sizes to 1e-12.
* Adjoint gradient, norb 12, (6, 6), n_reps 3, rank 24: the complex64
  gradient against FP64 central finite differences (h = 1e-5) of the
  complex128 energy, relative error <= 1e-4 over a fixed sample of 160 of the
  900 coordinates (every parameter block is sampled).
* norb 18, (9, 9): a random normalised state, one Haar orbital rotation, one
  diagonal Coulomb evolution (J entries N(0, 0.1), t = 1), then the energy of
  a rank-18 double-factorized Hamiltonian, complex64 against complex128,
  |dE| <= 1e-6 Ha.  About 57 GB of device memory at the peak.

The energy pattern is the reference's
tests/python/variational/ucj_spin_balanced_test.py:152-158 (vdot of psi with
H psi); the finite-difference gradient is python/ffsim/optimize/_util.py:60-110.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_lucj_energy_norb16_complex64_vs_fp64(cuda):
    import torch

    import ffsim_gb300 as f

    norb, nelec = 16, (8, 8)
    ucj = f.random.random_ucj_op_spin_balanced(norb, n_reps=2, diag_coulomb_normal=True,
                                               diag_coulomb_scale=0.1, seed=2026)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=32, seed=2027)
    ev64 = f.LUCJEnergy(norb, nelec, dtype=torch.complex64)
    e64 = ev64(ucj, ham)
    e64_again = ev64(ucj, ham)
    del ev64
    torch.cuda.empty_cache()
    e128 = f.lucj_energy(ucj, ham, norb, nelec, dtype=torch.complex128)
    torch.cuda.empty_cache()
    assert e64 == e64_again  # fixed reduction order: bit-reproducible
    assert abs(e64 - e128) <= 1e-6, (e64, e128)


def test_gradient_norb12_against_central_differences(cuda):
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300.gradient import LUCJGradient

    norb, nelec, n_reps, rank = 12, (6, 6), 3, 24
    params = f.random.random_ucj_op_spin_balanced(norb, n_reps=n_reps, diag_coulomb_normal=True,
                                                  diag_coulomb_scale=0.1, seed=2026).to_parameters()
    ham = f.random.random_df_hamiltonian_normal(norb, rank=rank, seed=2027)
    n = len(params)
    assert n == 900
    _, grad = LUCJGradient(norb, nelec, dtype=torch.complex64).value_and_grad(params, n_reps, ham)
    # per layer: 144 rotation parameters, then 78 + 78 diagonal Coulomb parameters
    rng = np.random.default_rng(12)
    per_layer = n // n_reps
    picks = []
    for k in range(n_reps):
        base = k * per_layer
        picks += list(base + rng.choice(144, 24, replace=False))
        picks += list(base + 144 + rng.choice(156, 29, replace=False))
    picks = sorted(set(int(p) for p in picks))[:160]
    assert len(picks) >= 150
    ev128 = f.LUCJEnergy(norb, nelec, dtype=torch.complex128)
    h = 1e-5

    def energy(p):
        return ev128(f.UCJOpSpinBalanced.from_parameters(p, norb=norb, n_reps=n_reps), ham)

    fd = np.empty(len(picks))
    for t, i in enumerate(picks):
        e = np.zeros(n)
        e[i] = h
        fd[t] = (energy(params + e) - energy(params - e)) / (2 * h)
    got = grad[picks]
    rel = np.linalg.norm(got - fd) / np.linalg.norm(fd)
    assert rel <= 1e-4, rel


def test_norb18_energy_complex64_vs_complex128(cuda):
    import torch

    import ffsim_gb300 as f

    norb, nelec = 18, (9, 9)
    rng = np.random.default_rng(18_18)
    u = f.random.random_unitary(norb, seed=rng)
    j = f.random.random_symmetric_matrix_normal(norb, scale=0.1, seed=rng)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=18, seed=1818)
    lin = f.linear_operator(ham, norb, nelec)
    d = f.dim(norb, nelec)
    gen = torch.Generator(device=cuda).manual_seed(18)
    energies = {}
    for dtype in (torch.complex128, torch.complex64):
        # the same amplitudes in both precisions: drawn in FP64, then rounded
        v = torch.randn(d, dtype=torch.complex128, device=cuda, generator=gen.manual_seed(18))
        v /= torch.linalg.vector_norm(v)
        v = v.to(dtype)
        v = f.apply_orbital_rotation(v, u, norb, nelec, copy=False)
        v = f.apply_diag_coulomb_evolution(v, j, 1.0, norb, nelec, copy=False)
        energies[dtype] = lin.expectation(v)
        del v
        torch.cuda.empty_cache()
    e64, e128 = energies[torch.complex64], energies[torch.complex128]
    assert abs(e64 - e128) <= 1e-6, (e64, e128)
