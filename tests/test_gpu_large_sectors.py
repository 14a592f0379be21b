"""Sectors too large for the shared-memory sector kernel (norb 17, 24,310
strings at half filling), against the FP64 oracle.  complex128: one adjacent
Givens rotation per pass and row-streamed diagonals.  complex64: the stage
kernels, also for one spin sector alone and for spinless vectors.  The other
sector holds one electron so the oracle stays fast."""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from oracle import ffsim_oracle as o

pytestmark = pytest.mark.gpu

TOL = 1e-10
NORB = 17
CASES = [(8, 1), (1, 8)]


def _t(x):
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda").to(torch.complex128)


def _n(t):
    return t.cpu().numpy().astype(np.complex128)


def _inputs(nelec, seed):
    rng = np.random.default_rng(seed)
    d = math.comb(NORB, nelec[0]) * math.comb(NORB, nelec[1])
    vec = o.random_state_vector(d, seed=rng)
    u = o.random_unitary(NORB, seed=rng)
    j = o.random_symmetric_normal(NORB, scale=0.3, seed=rng)
    return vec, u, j


@pytest.mark.parametrize("nelec", CASES)
def test_rotation_and_evolutions(cuda, nelec):
    import ffsim_gb300 as f

    vec, u, j = _inputs(nelec, 17 + nelec[0])
    got = _n(f.apply_orbital_rotation(_t(vec), u, NORB, nelec))
    np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, u, NORB, nelec), atol=TOL)
    # one sector only
    got = _n(f.apply_orbital_rotation(_t(vec), (None, u), NORB, nelec))
    np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, (None, u), NORB, nelec), atol=TOL)
    got = _n(f.apply_diag_coulomb_evolution(_t(vec), j, 0.7, NORB, nelec, orbital_rotation=u))
    exp = o.apply_diag_coulomb_evolution(vec, j, 0.7, NORB, nelec, orbital_rotation=u)
    np.testing.assert_allclose(got, exp, atol=TOL)
    coeffs = np.random.default_rng(3).standard_normal(NORB)
    got = _n(f.apply_num_op_sum_evolution(_t(vec), coeffs, 0.4, NORB, nelec, orbital_rotation=u))
    exp = o.apply_num_op_sum_evolution(vec, coeffs, 0.4, NORB, nelec, orbital_rotation=u)
    np.testing.assert_allclose(got, exp, atol=TOL)


@pytest.mark.parametrize("nelec", CASES)
def test_contractions_and_linops(cuda, nelec):
    import ffsim_gb300 as f

    vec, u, j = _inputs(nelec, 29 + nelec[0])
    got = _n(f.contract.contract_diag_coulomb(_t(vec), j, NORB, nelec))
    np.testing.assert_allclose(got, o.contract_diag_coulomb(vec, j, NORB, nelec), atol=TOL)
    lin = f.contract.diag_coulomb_linop(j, NORB, nelec, orbital_rotation=u)
    exp = o.diag_coulomb_linop_matvec(j, NORB, nelec, orbital_rotation=u)(vec)
    np.testing.assert_allclose(_n(lin @ _t(vec)), exp, atol=TOL)


def test_lucj_energy(cuda):
    import ffsim_gb300 as f

    nelec = CASES[0]
    ucj = f.random.random_ucj_op_spin_balanced(NORB, n_reps=1, seed=7)
    ham = f.random.random_df_hamiltonian_normal(NORB, rank=2, seed=8)
    psi = o.ucj_spin_balanced_apply(o.hartree_fock_state(NORB, nelec), ucj.diag_coulomb_mats,
                                    ucj.orbital_rotations, None, NORB, nelec)
    e_ref = o.df_energy(psi, ham.one_body_tensor, ham.diag_coulomb_mats, ham.orbital_rotations,
                        ham.constant, NORB, nelec)
    e = f.lucj_energy(ucj, ham, NORB, nelec, dtype=torch.complex128)
    assert abs(e - e_ref) < 1e-9


def test_spinless_rotation(cuda):
    import ffsim_gb300 as f

    rng = np.random.default_rng(41)
    vec = o.random_state_vector(math.comb(NORB, 8), seed=rng)
    u = o.random_unitary(NORB, seed=rng)
    got = _n(f.apply_orbital_rotation(_t(vec), u, NORB, 8))
    np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, u, NORB, 8), atol=TOL)


TOL64 = 2e-5


@pytest.mark.parametrize("nelec", CASES)
def test_complex64_one_sector_and_spinless(cuda, nelec):
    import ffsim_gb300 as f

    vec, u, j = _inputs(nelec, 53 + nelec[0])

    def c64(x):
        return torch.from_numpy(np.ascontiguousarray(x)).to("cuda").to(torch.complex64)

    for mat in (u, (None, u), (u, None)):
        got = _n(f.apply_orbital_rotation(c64(vec), mat, NORB, nelec))
        np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, mat, NORB, nelec), atol=TOL64)
    got = _n(f.apply_diag_coulomb_evolution(c64(vec), j, 0.7, NORB, nelec, orbital_rotation=u))
    exp = o.apply_diag_coulomb_evolution(vec, j, 0.7, NORB, nelec, orbital_rotation=u)
    np.testing.assert_allclose(got, exp, atol=TOL64)


def test_complex64_spinless(cuda):
    import ffsim_gb300 as f

    rng = np.random.default_rng(61)
    vec = o.random_state_vector(math.comb(NORB, 8), seed=rng)
    u = o.random_unitary(NORB, seed=rng)
    t = torch.from_numpy(vec).to("cuda").to(torch.complex64)
    got = _n(f.apply_orbital_rotation(t, u, NORB, 8))
    np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, u, NORB, 8), atol=TOL64)
    coeffs = rng.standard_normal(NORB)
    got = _n(f.apply_num_op_sum_evolution(t, coeffs, 0.4, NORB, 8, orbital_rotation=u))
    exp = o.apply_num_op_sum_evolution(vec, coeffs, 0.4, NORB, 8, orbital_rotation=u)
    np.testing.assert_allclose(got, exp, atol=TOL64)
