"""Parity of the CUDA path (through the C ABI) with the oracle and the golden vectors.

Tolerances: complex128 results must match to 1e-12 (max abs; the synthetic
configuration ||dpsi||_2 <= 1e-12); complex64 results to 2e-5 max abs on
unit-norm vectors (FP32 arithmetic, FP64 angles and reductions); energies in
complex64 to 1e-6 Ha.
"""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from conftest import NORB_NELEC_CASES
from oracle import ffsim_oracle as o

pytestmark = pytest.mark.gpu

TOL128 = 1e-12
TOL64 = 2e-5
DTYPES = [(torch.complex128, TOL128), (torch.complex64, TOL64)]


def _t(x, dtype):
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda").to(dtype)


def _n(t):
    return t.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_orbital_rotation_golden(cuda, golden, dtype, tol):
    import ffsim_gb300 as f

    for idx, (n, a, b) in enumerate(golden["rot_cases"]):
        n, ne = int(n), (int(a), int(b))
        v = _t(golden[f"rot{idx}_in"], dtype)
        ua, ub = golden[f"rot{idx}_ua"], golden[f"rot{idx}_ub"]
        for mat, key in [(ua, "same"), ((ua, ub), "pair"), ((ua, None), "aonly"), ((None, ub), "bonly"),
                         (np.stack([ua, ub]), "pair")]:
            out = f.apply_orbital_rotation(v, mat, n, ne)
            np.testing.assert_allclose(_n(out), golden[f"rot{idx}_{key}"], atol=tol, err_msg=f"{idx} {key}")
        np.testing.assert_allclose(_n(v), golden[f"rot{idx}_in"], atol=tol)  # copy=True left input intact
    out = f.apply_orbital_rotation(_t(golden["rotsl_in"], dtype), golden["rotsl_u"], 6, 2)
    np.testing.assert_allclose(_n(out), golden["rotsl_out"], atol=tol)


def test_config0_complex128(cuda, golden):
    """norb=8, (4,4): rotation then diag-Coulomb t=0.7; ||dpsi||_2 <= 1e-12 and identical layout."""
    import ffsim_gb300 as f

    v = _t(golden["cfg0_in"], torch.complex128).reshape(70, 70)
    mid = f.apply_orbital_rotation(v, golden["cfg0_u"], 8, (4, 4))
    out = f.apply_diag_coulomb_evolution(mid, golden["cfg0_j"], 0.7, 8, (4, 4))
    assert tuple(out.shape) == (70, 70)
    assert np.linalg.norm(_n(out).reshape(-1) - golden["cfg0_out"]) <= 1e-12


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_fixture_rotation(cuda, golden, dtype, tol):
    import ffsim_gb300 as f

    hf = f.hartree_fock_state(8, (5, 5), dtype=dtype)
    out = f.apply_orbital_rotation(hf, golden["fix_mat"], 8, (5, 5))
    np.testing.assert_allclose(_n(out), golden["fix_out"], atol=tol)
    assert abs(torch.linalg.vector_norm(out).item() - 1) < 10 * tol


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_diag_coulomb_golden(cuda, golden, dtype, tol):
    import ffsim_gb300 as f

    for idx, (n, a, b) in enumerate(golden["dc_cases"]):
        n, ne = int(n), (int(a), int(b))
        g = lambda s: golden[f"dc{idx}_{s}"]  # noqa: E731
        v, t = _t(g("in"), dtype), float(g("t"))
        mats = (g("jaa"), g("jab"), g("jbb"))
        checks = [
            (f.apply_diag_coulomb_evolution(v, mats, t, n, ne), "num"),
            (f.apply_diag_coulomb_evolution(v, mats, t, n, ne, z_representation=True), "z"),
            (f.apply_diag_coulomb_evolution(v, g("jaa"), t, n, ne), "single"),
            (f.apply_diag_coulomb_evolution(v, (None, g("jab"), None), t, n, ne), "none"),
            (f.apply_diag_coulomb_evolution(v, mats, t, n, ne, orbital_rotation=g("u")), "rot"),
            (f.apply_diag_coulomb_evolution(v, g("jaa"), t, n, ne, orbital_rotation=g("u"), z_representation=True), "zrot"),
            (f.contract.contract_diag_coulomb(v, mats, n, ne), "cnum"),
            (f.contract.contract_diag_coulomb(v, mats, n, ne, z_representation=True), "cz"),
            (f.contract.contract_diag_coulomb(v, g("jaa"), n, ne), "csingle"),
            (f.contract.diag_coulomb_linop(g("jaa"), n, ne, orbital_rotation=g("u")) @ v, "linop"),
        ]
        for out, key in checks:
            scale = max(1.0, float(np.abs(g(key)).max()))
            np.testing.assert_allclose(_n(out), g(key), atol=tol * scale, err_msg=f"dc{idx} {key}")
    out = f.apply_diag_coulomb_evolution(_t(golden["dcsl_in"], dtype), golden["dcsl_j"], 0.3, 5, 2)
    np.testing.assert_allclose(_n(out), golden["dcsl_out"], atol=tol)


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_num_op_sum_golden(cuda, golden, dtype, tol):
    import ffsim_gb300 as f

    for idx, (n, ne) in enumerate([(5, (3, 2)), (4, (1, 3))]):
        g = lambda s: golden[f"nos{idx}_{s}"]  # noqa: E731
        v, t = _t(g("in"), dtype), float(g("t"))
        checks = [
            (f.apply_num_op_sum_evolution(v, (g("ca"), g("cb")), t, n, ne), "pair"),
            (f.apply_num_op_sum_evolution(v, g("ca"), t, n, ne, orbital_rotation=g("u")), "rot"),
            (f.apply_num_op_sum_evolution(v, (None, g("cb")), t, n, ne), "bonly"),
            (f.contract.contract_num_op_sum(v, g("ca"), n, ne), "contract"),
            (f.contract.num_op_sum_linop(g("ca"), n, ne, orbital_rotation=g("u")) @ v, "linop"),
        ]
        for out, key in checks:
            scale = max(1.0, float(np.abs(g(key)).max()))
            np.testing.assert_allclose(_n(out), g(key), atol=tol * scale, err_msg=f"nos{idx} {key}")


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_df_hamiltonian_golden(cuda, golden, dtype, tol):
    import ffsim_gb300 as f

    for idx, (n, a, b, _r) in enumerate(golden["df_cases"]):
        g = lambda s: golden[f"df{idx}_{s}"]  # noqa: E731
        ham = f.DoubleFactorizedHamiltonian(g("h1"), g("dcm"), g("rots"), float(g("const")), bool(g("z")))
        op = f.linear_operator(ham, int(n), (int(a), int(b)))
        v = _t(g("in"), dtype)
        hv = op @ v
        scale = max(1.0, float(np.abs(g("hv")).max()))
        np.testing.assert_allclose(_n(hv), g("hv"), atol=tol * scale)
        e_tol = 1e-10 if dtype == torch.complex128 else 1e-6
        assert abs(op.expectation(v) - float(g("energy"))) < e_tol
        assert abs(f.vdot(v, hv).real - float(g("energy"))) < e_tol * 10


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_ucj_golden(cuda, golden, dtype, tol):
    import ffsim_gb300 as f

    for idx, (n, a, b, reps, fin) in enumerate(golden["ucj_cases"]):
        g = lambda s: golden[f"ucj{idx}_{s}"]  # noqa: E731
        n, ne = int(n), (int(a), int(b))
        op = f.UCJOpSpinBalanced.from_parameters(g("params"), norb=n, n_reps=int(reps),
                                                 with_final_orbital_rotation=bool(fin))
        out = f.apply_unitary(_t(g("in"), dtype), op, n, ne)
        np.testing.assert_allclose(_n(out), g("out"), atol=tol)
        out = f.apply_unitary(f.hartree_fock_state(n, ne, dtype=dtype), op, n, ne)
        np.testing.assert_allclose(_n(out), g("hf_out"), atol=tol)


@pytest.mark.parametrize("norb, nelec", NORB_NELEC_CASES)
@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_edge_cases(cuda, norb, nelec, dtype, tol):
    import ffsim_gb300 as f

    rng = np.random.default_rng(norb * 13 + nelec[0] * 3 + nelec[1])
    d = math.comb(norb, nelec[0]) * math.comb(norb, nelec[1])
    vec = o.random_state_vector(d, seed=rng)
    u = o.random_unitary(norb, seed=rng) if norb else np.zeros((0, 0), dtype=complex)
    j = o.random_symmetric_normal(norb, seed=rng) if norb else np.zeros((0, 0))
    v = _t(vec, dtype)
    np.testing.assert_allclose(_n(f.apply_orbital_rotation(v, u, norb, nelec)),
                               o.apply_orbital_rotation(vec, u, norb, nelec), atol=tol)
    np.testing.assert_allclose(_n(f.apply_diag_coulomb_evolution(v, j, 0.4, norb, nelec, orbital_rotation=u)),
                               o.apply_diag_coulomb_evolution(vec, j, 0.4, norb, nelec, orbital_rotation=u),
                               atol=tol)
    coeffs = rng.standard_normal(norb)
    np.testing.assert_allclose(_n(f.apply_num_op_sum_evolution(v, coeffs, 0.9, norb, nelec)),
                               o.apply_num_op_sum_evolution(vec, coeffs, 0.9, norb, nelec), atol=tol)


@pytest.mark.parametrize("norb, nelec", [(9, (4, 5)), (10, (5, 5)), (11, (5, 4)), (12, (6, 6)), (13, (5, 6)),
                                         (14, (7, 7))])
def test_windows_complex64_vs_oracle(cuda, norb, nelec):
    """Register-window (cosine-sine) kernels at the sizes where they engage."""
    import ffsim_gb300 as f

    rng = np.random.default_rng(norb)
    d = math.comb(norb, nelec[0]) * math.comb(norb, nelec[1])
    vec = o.random_state_vector(d, seed=rng)
    ua, ub = o.random_unitary(norb, seed=rng), o.random_unitary(norb, seed=rng)
    ref = o.apply_orbital_rotation(vec, (ua, ub), norb, nelec)
    out = f.apply_orbital_rotation(_t(vec, torch.complex64), (ua, ub), norb, nelec)
    np.testing.assert_allclose(_n(out), ref, atol=TOL64)
    out = f.apply_orbital_rotation(_t(vec, torch.complex128), (ua, ub), norb, nelec)
    np.testing.assert_allclose(_n(out), ref, atol=TOL128)


@pytest.mark.parametrize("dtype, tol", DTYPES)
def test_low_level_kernels(cuda, dtype, tol):
    import ffsim_gb300 as f

    norb, nelec = 5, (3, 2)
    rng = np.random.default_rng(1)
    vec = o.random_state_vector(o.dim(norb, nelec), seed=rng)
    for spin in (0, 1):
        for (i, j) in [(1, 2), (3, 2)]:
            c, s = 0.6, 0.48 + 0.64j
            t = _t(vec, dtype)
            f.apply_givens_rotation_in_place(t, c, s, (i, j), norb, nelec, spin=spin)
            ref = vec.reshape(10, 10).copy()
            nocc = nelec[spin]
            idx = o.zero_one_subspace_indices(norb, nocc, (i, j))
            half = len(idx) // 2
            r = ref if spin == 0 else ref.T.copy()
            o.apply_givens_rotation_in_place(r, c, s, idx[:half], idx[half:])
            ref = r if spin == 0 else r.T
            np.testing.assert_allclose(_n(t), ref.reshape(-1), atol=tol)
        t = _t(vec, dtype)
        f.apply_phase_shift_in_place(t, np.exp(0.3j), 2, norb, nelec, spin=spin)
        ref = vec.reshape(10, 10).copy()
        rows = o.one_subspace_indices(norb, nelec[spin], (2,))
        if spin == 0:
            ref[rows] *= np.exp(0.3j)
        else:
            ref[:, rows] *= np.exp(0.3j)
        np.testing.assert_allclose(_n(t), ref.reshape(-1), atol=tol)


def test_copy_false_and_shapes(cuda):
    import ffsim_gb300 as f

    rng = np.random.default_rng(2)
    vec = o.random_state_vector(100, seed=rng)
    u = o.random_unitary(5, seed=rng)
    t = _t(vec, torch.complex128).reshape(10, 10)
    out = f.apply_orbital_rotation(t, u, 5, (3, 2), copy=False)
    assert tuple(out.shape) == (10, 10)
    np.testing.assert_allclose(_n(out).reshape(-1), o.apply_orbital_rotation(vec, u, 5, (3, 2)), atol=TOL128)
    arr = f.apply_orbital_rotation(vec, u, 5, (3, 2))  # numpy in, numpy out
    assert isinstance(arr, np.ndarray)
    np.testing.assert_allclose(arr, o.apply_orbital_rotation(vec, u, 5, (3, 2)), atol=TOL128)


def test_norb16_properties_complex64(cuda):
    """Full size of the metric workload: unitarity and U then U^dag round trip."""
    import ffsim_gb300 as f

    norb, nelec = 16, (8, 8)
    rng = np.random.default_rng(16)
    u = o.random_unitary(norb, seed=rng)
    d = f.dim(norb, nelec)
    g = torch.Generator(device="cuda").manual_seed(7)
    v = torch.randn(d, dtype=torch.complex64, device="cuda", generator=g)
    v /= torch.linalg.vector_norm(v)
    w = f.apply_orbital_rotation(v, u, norb, nelec)
    assert abs(torch.linalg.vector_norm(w.to(torch.complex128)).item() - 1) < 1e-5
    back = f.apply_orbital_rotation(w, u.conj().T, norb, nelec)
    err = torch.linalg.vector_norm((back - v).to(torch.complex128)).item()
    assert err < 5e-5, err
    # HF rotated is a product of two Slater determinants: check a few amplitudes
    hf = f.hartree_fock_state(norb, nelec, dtype=torch.complex64)
    r = f.apply_orbital_rotation(hf, u, norb, nelec).reshape(12870, 12870)
    strings = o.make_strings(norb, 8)
    for a in (0, 17, 5000, 12869):
        occ = [i for i in range(norb) if (int(strings[a]) >> i) & 1]
        va = np.linalg.det(u[np.ix_(occ, range(8))])
        for b in (3, 12000):
            occb = [i for i in range(norb) if (int(strings[b]) >> i) & 1]
            vb = np.linalg.det(u[np.ix_(occb, range(8))])
            assert abs(complex(r[a, b].item()) - va * vb) < 1e-5


def test_lucj_energy_matches_oracle(cuda):
    """Fused LUCJ energy (complex64 and complex128) vs the FP64 oracle at norb=8, (4,4)."""
    import ffsim_gb300 as f

    norb, nelec = 8, (4, 4)
    ucj = f.random.random_ucj_op_spin_balanced(norb, n_reps=2, diag_coulomb_normal=True,
                                               diag_coulomb_scale=0.1, seed=3)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=5, seed=4)
    psi = o.ucj_spin_balanced_apply(o.hartree_fock_state(norb, nelec), ucj.diag_coulomb_mats,
                                    ucj.orbital_rotations, None, norb, nelec)
    e_ref = o.df_energy(psi, ham.one_body_tensor, ham.diag_coulomb_mats, ham.orbital_rotations,
                        ham.constant, norb, nelec)
    e128 = f.lucj_energy(ucj, ham, norb, nelec, dtype=torch.complex128)
    e64 = f.lucj_energy(ucj, ham, norb, nelec, dtype=torch.complex64)
    assert abs(e128 - e_ref) < 1e-10
    assert abs(e64 - e_ref) < 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("norb, nelec", [(17, (3, 4)), (18, (3, 2)), (18, (4, 4))])
def test_nested_cosine_sine_plans(cuda, norb, nelec):
    """norb 17 and 18: 9-orbital halves split again (4 + 5) on the complex64
    stage path, against the complex128 path (shared-memory kernel with the
    adjacent-Givens network) on the same inputs."""
    import torch

    import ffsim_gb300 as f

    rng = np.random.default_rng(norb * 10 + nelec[0])
    d = f.dim(norb, nelec)
    v = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    v /= np.linalg.norm(v)
    u = f.random.random_unitary(norb, seed=rng)
    j = f.random.random_symmetric_matrix_normal(norb, scale=0.1, seed=rng)
    for op in ("rot", "dc"):
        outs = {}
        for dtype in (torch.complex64, torch.complex128):
            t = torch.tensor(v, dtype=dtype, device=cuda)
            if op == "rot":
                t = f.apply_orbital_rotation(t, u, norb, nelec)
            else:
                t = f.apply_diag_coulomb_evolution(t, j, 0.7, norb, nelec, orbital_rotation=u)
            outs[dtype] = t.cpu().numpy().astype(np.complex128)
        assert np.linalg.norm(outs[torch.complex64] - outs[torch.complex128]) < 2e-5, op
    ham = f.random.random_df_hamiltonian_normal(norb, rank=3, seed=5)
    ucj = f.random.random_ucj_op_spin_balanced(norb, n_reps=1, seed=6)
    e64 = f.lucj_energy(ucj, ham, norb, nelec, dtype=torch.complex64)
    e128 = f.lucj_energy(ucj, ham, norb, nelec, dtype=torch.complex128)
    assert abs(e64 - e128) < 1e-5


@pytest.mark.parametrize("norb, nelec", [(10, (3, 4)), (13, (3, 3)), (16, (3, 2)), (17, (2, 3)), (18, (2, 2))])
def test_banded_and_near_identity_rotations(cuda, norb, nelec):
    """Short-time hopping evolutions exp(-i t h) (banded, near the identity) and
    a permutation: the cosine-sine plans resolve their small sines, on the
    complex64 stage kernels and the complex128 path, against the oracle."""
    import scipy.linalg

    import ffsim_gb300 as f

    rng = np.random.default_rng(norb * 3 + 1)
    d = math.comb(norb, nelec[0]) * math.comb(norb, nelec[1])
    vec = o.random_state_vector(d, seed=rng)
    hop = np.diag(-np.ones(norb - 1), 1)
    mats = [scipy.linalg.expm(-1j * t * (hop + hop.T)) for t in (1e-3, 0.1, 1.0)]
    mats.append(np.roll(np.eye(norb), 5, axis=0).astype(complex))
    for u in mats:
        ref = o.apply_orbital_rotation(vec, (u, u.conj()), norb, nelec)
        out = f.apply_orbital_rotation(_t(vec, torch.complex64), (u, u.conj()), norb, nelec)
        np.testing.assert_allclose(_n(out), ref, atol=TOL64)
        out = f.apply_orbital_rotation(_t(vec, torch.complex128), (u, u.conj()), norb, nelec)
        np.testing.assert_allclose(_n(out), ref, atol=TOL128)


@pytest.mark.parametrize("norb, nelec", NORB_NELEC_CASES)
def test_num_op_sum_eigenphase_kat(cuda, norb, nelec):
    """Every configuration is an eigenvector: exp(-i t sum of its occupied
    coefficients), per spin selection (tests/python/gates/num_op_sum_test.py:27-72),
    in both precisions, one configuration per call."""
    import itertools

    import ffsim_gb300 as f

    rng = np.random.default_rng(norb * 13 + sum(nelec))
    coeffs = rng.standard_normal(norb)
    time = rng.standard_normal()
    na, nb = nelec
    for spin in (1, 2, 3):
        pair = (coeffs if spin & 1 else None, coeffs if spin & 2 else None)
        for occ_a in itertools.combinations(range(norb), na):
            for occ_b in itertools.combinations(range(norb), nb):
                eig = (coeffs[list(occ_a)].sum() if spin & 1 else 0.0) + (coeffs[list(occ_b)].sum() if spin & 2 else 0.0)
                for dtype, tol in DTYPES:
                    state = f.slater_determinant(norb, (list(occ_a), list(occ_b)), dtype=dtype)
                    exp = np.exp(-1j * eig * time) * _n(state)
                    out = f.apply_num_op_sum_evolution(state, pair, time, norb, nelec)
                    np.testing.assert_allclose(_n(out), exp, atol=tol)
