"""The FP64 oracle against the reference's golden vectors and known answers (CPU)."""

from __future__ import annotations

import itertools
import math

import numpy as np
import pytest

from conftest import NORB_NELEC_CASES
from oracle import ffsim_oracle as o

TOL = 1e-12


def test_layout_kat():
    # tests/python/states/bitstring_test.py: norb=3, nocc=2 -> [0b011, 0b101, 0b110]
    assert list(o.make_strings(3, 2)) == [0b011, 0b101, 0b110]
    assert list(o.make_strings(4, 1)) == [1, 2, 4, 8]
    occ = o.gen_occslst(4, 2)
    assert occ.tolist() == [[0, 1], [0, 2], [1, 2], [0, 3], [1, 3], [2, 3]]


def test_index_subsets(golden):
    for k in golden.files:
        if k.startswith("zero_one_"):
            _, _, n, c, ij = k.split("_")
            got = o.zero_one_subspace_indices(int(n), int(c), (int(ij[0]), int(ij[1])))
            np.testing.assert_array_equal(got, golden[k])
        elif k.startswith("one_"):
            _, n, c, i = k.split("_")
            np.testing.assert_array_equal(o.one_subspace_indices(int(n), int(c), (int(i),)), golden[k])


def test_orbital_rotation(golden):
    for idx, (n, a, b) in enumerate(golden["rot_cases"]):
        n, ne = int(n), (int(a), int(b))
        v, ua, ub = golden[f"rot{idx}_in"], golden[f"rot{idx}_ua"], golden[f"rot{idx}_ub"]
        np.testing.assert_allclose(o.apply_orbital_rotation(v, ua, n, ne), golden[f"rot{idx}_same"], atol=TOL)
        np.testing.assert_allclose(o.apply_orbital_rotation(v, (ua, ub), n, ne), golden[f"rot{idx}_pair"], atol=TOL)
        np.testing.assert_allclose(o.apply_orbital_rotation(v, (ua, None), n, ne), golden[f"rot{idx}_aonly"], atol=TOL)
        np.testing.assert_allclose(o.apply_orbital_rotation(v, (None, ub), n, ne), golden[f"rot{idx}_bonly"], atol=TOL)
    np.testing.assert_allclose(o.apply_orbital_rotation(golden["rotsl_in"], golden["rotsl_u"], 6, 2),
                               golden["rotsl_out"], atol=TOL)


def test_orbital_rotation_fixture_det_minor(golden):
    # reference fixture tests/python/test_data/orbital_rotation-0.npy on HF (8, (5, 5))
    mat = golden["fix_mat"]
    out = o.apply_orbital_rotation(o.hartree_fock_state(8, (5, 5)), mat, 8, (5, 5))
    np.testing.assert_allclose(out, golden["fix_out"], atol=TOL)
    va = o.slater_rotation_amplitudes(mat, 8, 5, range(5))
    np.testing.assert_allclose(out.reshape(56, 56), np.outer(va, va), atol=TOL)
    assert abs(np.linalg.norm(out) - 1) < TOL


def test_diag_coulomb_and_contractions(golden):
    for idx, (n, a, b) in enumerate(golden["dc_cases"]):
        n, ne = int(n), (int(a), int(b))
        g = lambda s: golden[f"dc{idx}_{s}"]  # noqa: E731
        v, t = g("in"), float(g("t"))
        mats = (g("jaa"), g("jab"), g("jbb"))
        np.testing.assert_allclose(o.apply_diag_coulomb_evolution(v, mats, t, n, ne), g("num"), atol=TOL)
        np.testing.assert_allclose(o.apply_diag_coulomb_evolution(v, mats, t, n, ne, z_representation=True), g("z"), atol=TOL)
        np.testing.assert_allclose(o.apply_diag_coulomb_evolution(v, g("jaa"), t, n, ne), g("single"), atol=TOL)
        np.testing.assert_allclose(o.apply_diag_coulomb_evolution(v, (None, g("jab"), None), t, n, ne), g("none"), atol=TOL)
        np.testing.assert_allclose(o.apply_diag_coulomb_evolution(v, mats, t, n, ne, orbital_rotation=g("u")), g("rot"), atol=TOL)
        np.testing.assert_allclose(o.apply_diag_coulomb_evolution(v, g("jaa"), t, n, ne, orbital_rotation=g("u"), z_representation=True), g("zrot"), atol=TOL)
        np.testing.assert_allclose(o.contract_diag_coulomb(v, mats, n, ne), g("cnum"), atol=TOL)
        np.testing.assert_allclose(o.contract_diag_coulomb(v, mats, n, ne, z_representation=True), g("cz"), atol=TOL)
        np.testing.assert_allclose(o.contract_diag_coulomb(v, g("jaa"), n, ne), g("csingle"), atol=TOL)
        np.testing.assert_allclose(o.diag_coulomb_linop_matvec(g("jaa"), n, ne, orbital_rotation=g("u"))(v), g("linop"), atol=TOL)
    np.testing.assert_allclose(o.apply_diag_coulomb_evolution(golden["dcsl_in"], golden["dcsl_j"], 0.3, 5, 2),
                               golden["dcsl_out"], atol=TOL)


def test_num_op_sum(golden):
    for idx, (n, ne) in enumerate([(5, (3, 2)), (4, (1, 3))]):
        g = lambda s: golden[f"nos{idx}_{s}"]  # noqa: E731
        v, t = g("in"), float(g("t"))
        np.testing.assert_allclose(o.apply_num_op_sum_evolution(v, (g("ca"), g("cb")), t, n, ne), g("pair"), atol=TOL)
        np.testing.assert_allclose(o.apply_num_op_sum_evolution(v, g("ca"), t, n, ne, orbital_rotation=g("u")), g("rot"), atol=TOL)
        np.testing.assert_allclose(o.apply_num_op_sum_evolution(v, (None, g("cb")), t, n, ne), g("bonly"), atol=TOL)
        np.testing.assert_allclose(o.contract_num_op_sum(v, g("ca"), n, ne), g("contract"), atol=TOL)
        np.testing.assert_allclose(o.num_op_sum_linop_matvec(g("ca"), n, ne, orbital_rotation=g("u"))(v), g("linop"), atol=TOL)


def test_df_hamiltonian(golden):
    for idx, (n, a, b, _r) in enumerate(golden["df_cases"]):
        g = lambda s: golden[f"df{idx}_{s}"]  # noqa: E731
        mv = o.df_hamiltonian_matvec(g("h1"), g("dcm"), g("rots"), float(g("const")), int(n),
                                     (int(a), int(b)), bool(g("z")))
        np.testing.assert_allclose(mv(g("in")), g("hv"), atol=TOL)
        assert abs(np.vdot(g("in"), mv(g("in"))).real - float(g("energy"))) < TOL


def test_ucj(golden):
    for idx, (n, a, b, reps, fin) in enumerate(golden["ucj_cases"]):
        g = lambda s: golden[f"ucj{idx}_{s}"]  # noqa: E731
        n, ne = int(n), (int(a), int(b))
        dcm, rots, final = o.ucj_from_parameters(g("params"), n, int(reps), bool(fin))
        np.testing.assert_allclose(dcm, g("dcm"), atol=TOL)
        np.testing.assert_allclose(rots, g("rots"), atol=TOL)
        np.testing.assert_allclose(o.ucj_spin_balanced_apply(g("in"), dcm, rots, final, n, ne), g("out"), atol=TOL)
        hf = o.hartree_fock_state(n, ne)
        np.testing.assert_allclose(o.ucj_spin_balanced_apply(hf, dcm, rots, final, n, ne), g("hf_out"), atol=TOL)


def test_config0(golden):
    mid = o.apply_orbital_rotation(golden["cfg0_in"], golden["cfg0_u"], 8, (4, 4))
    out = o.apply_diag_coulomb_evolution(mid, golden["cfg0_j"], 0.7, 8, (4, 4))
    assert np.linalg.norm(out - golden["cfg0_out"]) <= 1e-12


def test_givens_reconstruction():
    # tests/python/linalg/givens_test.py: U = D G_L^* ... G_1^*, n(n-1)/2 rotations
    rng = np.random.default_rng(5)
    for n in range(1, 9):
        u = o.random_unitary(n, seed=rng)
        rots, diag = o.givens_decomposition(u)
        assert len(rots) == n * (n - 1) // 2
        m = np.diag(diag)
        for c, s, i, j in reversed(rots):
            g = np.eye(n, dtype=complex)
            g[np.ix_([i, j], [i, j])] = [[c, s], [-np.conj(s), c]]
            m = m @ g.conj()
        np.testing.assert_allclose(m, u, atol=1e-12)


@pytest.mark.parametrize("norb, nelec", NORB_NELEC_CASES)
def test_diag_coulomb_eigenphase_kat(norb, nelec):
    # closed form on Slater determinants: tests/python/gates/diag_coulomb_test.py:149-243
    rng = np.random.default_rng(norb * 7 + sum(nelec))
    time = rng.uniform(-10, 10)
    mat_aa = o.random_symmetric_normal(norb, seed=rng) if norb else np.zeros((0, 0))
    mat_ab = rng.standard_normal((norb, norb))
    mat_bb = o.random_symmetric_normal(norb, seed=rng) if norb else np.zeros((0, 0))
    na, nb = nelec
    da, db = math.comb(norb, na), math.comb(norb, nb)
    for ia, occ_a in enumerate(itertools.combinations(range(norb), na)):
        for ib, occ_b in enumerate(itertools.combinations(range(norb), nb)):
            a_addr = list(o.make_strings(norb, na)).index(sum(1 << i for i in occ_a))
            b_addr = list(o.make_strings(norb, nb)).index(sum(1 << i for i in occ_b))
            state = np.zeros(da * db, dtype=complex)
            state[a_addr * db + b_addr] = 1
            eig = 0.0
            occ = (occ_a, occ_b)
            for i, j in itertools.product(range(norb), repeat=2):
                for s, t in itertools.product(range(2), repeat=2):
                    if i in occ[s] and j in occ[t]:
                        eig += 0.5 * {(0, 0): mat_aa[i, j], (1, 1): mat_bb[i, j],
                                      (0, 1): mat_ab[i, j], (1, 0): mat_ab[j, i]}[(s, t)]
            res = o.apply_diag_coulomb_evolution(state, (mat_aa, mat_ab, mat_bb), time, norb, nelec)
            np.testing.assert_allclose(res, np.exp(-1j * eig * time) * state, atol=1e-12)


@pytest.mark.parametrize("norb, nelec", NORB_NELEC_CASES)
def test_num_op_sum_eigenphase_kat(norb, nelec):
    """Closed form on Slater determinants (tests/python/gates/num_op_sum_test.py:27-72):
    each configuration picks up exp(-i t sum of its occupied coefficients) in
    the sectors the coefficients act on; spinless as the (n, 0) sector."""
    rng = np.random.default_rng(norb * 11 + sum(nelec))
    coeffs = rng.standard_normal(norb)
    time = rng.standard_normal()
    na, nb = nelec
    da, db = math.comb(norb, na), math.comb(norb, nb)
    for spin in (1, 2, 3):
        pair = (coeffs if spin & 1 else np.zeros(norb), coeffs if spin & 2 else np.zeros(norb))
        for occ_a in itertools.combinations(range(norb), na):
            for occ_b in itertools.combinations(range(norb), nb):
                a_addr = list(o.make_strings(norb, na)).index(sum(1 << i for i in occ_a))
                b_addr = list(o.make_strings(norb, nb)).index(sum(1 << i for i in occ_b))
                state = np.zeros(da * db, dtype=complex)
                state[a_addr * db + b_addr] = 1
                eig = pair[0][list(occ_a)].sum() + pair[1][list(occ_b)].sum()
                res = o.apply_num_op_sum_evolution(state, pair, time, norb, nelec)
                np.testing.assert_allclose(res, np.exp(-1j * eig * time) * state, atol=1e-12)


def _trotter_case(golden, idx, row):
    n, a, b, t, steps, order, z = row
    g = lambda s: golden[f"trot{idx}_{s}"]  # noqa: E731
    return (int(n), (int(a), int(b)), float(t), int(steps), int(order), bool(z), g)


def test_trotter_double_factorized(golden):
    """Trotter-Suzuki evolution (orders 0-2) against the reference's own
    trotter/double_factorized.py run over its kernels."""
    for idx, row in enumerate(golden["trot_cases"]):
        n, ne, t, steps, order, z, g = _trotter_case(golden, idx, row)
        got = o.simulate_trotter_double_factorized(g("in"), g("h1"), g("dcm"), g("rots"), float(g("const")), t,
                                                   n, ne, n_steps=steps, order=order, z_representation=z)
        np.testing.assert_allclose(got, g("out"), atol=TOL)


def test_trotter_converges_to_exact_evolution():
    """Higher order and more steps approach exp(-i t H) psi (the reference's own
    accuracy test, trotter/double_factorized_test.py:23-85, on the oracle)."""
    scipy_sparse_linalg = pytest.importorskip("scipy.sparse.linalg")
    rng = np.random.default_rng(11)
    norb, nelec, t = 4, (2, 2), 0.4
    d = o.dim(norb, nelec)
    g = rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))
    h1 = (g + g.conj().T) / 4
    dcm = np.stack([o.random_symmetric_normal(norb, scale=0.5, seed=rng) for _ in range(3)])
    rots = np.stack([o.random_unitary(norb, seed=rng) for _ in range(3)])
    vec = o.random_state_vector(d, seed=rng)
    mv = o.df_hamiltonian_matvec(h1, dcm, rots, 0.3, norb, nelec)
    op = scipy_sparse_linalg.LinearOperator((d, d), matvec=mv, rmatvec=mv, dtype=complex)
    exact = scipy_sparse_linalg.expm_multiply(-1j * t * op, vec, traceA=-1j * t)
    errs = [np.linalg.norm(o.simulate_trotter_double_factorized(vec, h1, dcm, rots, 0.3, t, norb, nelec,
                                                                 n_steps=s, order=k) - exact)
            for s, k in [(2, 0), (8, 0), (4, 1), (4, 2)]]
    assert errs[1] < errs[0] and errs[2] < errs[1] and errs[3] < errs[2] and errs[3] < 1e-4, errs
