"""Slater determinants (python/ffsim/states/slater.py): state vectors, closed-form
RDMs and amplitudes against the reference's own code (golden vectors)."""

from __future__ import annotations

import numpy as np
import pytest

CASES = [("a", ([0, 2], [1, 3, 4]), "u"), ("b", ([1], [0, 3]), ("u", "v")), ("c", [0, 3, 1], "v"),
         ("d", ([0, 1], []), (None, "v"))]


def _rot(golden, spec):
    if spec is None:
        return None
    if isinstance(spec, tuple):
        return tuple(_rot(golden, x) for x in spec)
    return golden[f"sl_{spec}"]


def test_unrotated_vectors_on_host(golden):
    """Index and sign of the configuration (the parity of the listed order)."""
    import ffsim_gb300 as f

    got = f.slater_determinant(5, ([3, 0], [4, 1, 2]), device="cpu").numpy()
    np.testing.assert_array_equal(got, golden["sl_vec_plain"])
    got = f.slater_determinant(5, [2, 4, 0], device="cpu").numpy()
    np.testing.assert_array_equal(got, golden["sl_vec_plain_spinless"])
    assert f.slater_determinant(0, ([], []), device="cpu").numpy().tolist() == [1]


def test_rdms(golden):
    import ffsim_gb300 as f

    for tag, occ, spec in CASES:
        rot = _rot(golden, spec)
        np.testing.assert_allclose(f.slater_determinant_rdms(5, occ, rot), golden[f"sl_rdm_{tag}_1"], atol=1e-13)
        for reorder in (True, False):
            _, rdm2 = f.slater_determinant_rdms(5, occ, rot, rank=2, reorder=reorder)
            np.testing.assert_allclose(rdm2, golden[f"sl_rdm_{tag}_2_{int(reorder)}"], atol=1e-13)
    with pytest.raises(NotImplementedError):
        f.slater_determinant_rdms(5, [0], rank=3)


def test_amplitudes(golden):
    import ffsim_gb300 as f

    u, v = golden["sl_u"], golden["sl_v"]
    got = f.slater_determinant_amplitudes(([0b00011, 0b10100], [0b01010, 0b11000]), 5, ([0, 1], [2, 3]), (u, v))
    np.testing.assert_allclose(got, golden["sl_amp_spinful"], atol=1e-13)
    got = f.slater_determinant_amplitudes([0b00111, 0b11010], 5, [0, 2, 4], v)
    np.testing.assert_allclose(got, golden["sl_amp_spinless"], atol=1e-13)


@pytest.mark.gpu
def test_gpu_rotated_vectors(cuda, golden):
    import torch

    import ffsim_gb300 as f

    u, v = golden["sl_u"], golden["sl_v"]
    for dtype, tol in [(torch.complex128, 1e-12), (torch.complex64, 2e-6)]:
        for got, key in [(f.slater_determinant(5, ([1, 3], [0, 4, 2]), u, dtype=dtype), "sl_vec_rot"),
                         (f.slater_determinant(5, ([2, 0], [1]), (u, None), dtype=dtype), "sl_vec_pair"),
                         (f.slater_determinant(5, [4, 1], v, dtype=dtype), "sl_vec_spinless_rot")]:
            np.testing.assert_allclose(got.cpu().numpy().astype(complex), golden[key], atol=tol)


def test_spin_square_oracle_known_answers():
    """S^2 of high-spin and closed-shell configurations and of the two
    open-shell combinations (the oracle builds S_+ psi string by string)."""
    from oracle import ffsim_oracle as o

    assert abs(o.spin_square(o.hartree_fock_state(3, (2, 0)), 3, (2, 0)) - 2.0) < 1e-12
    assert abs(o.spin_square(o.hartree_fock_state(4, (2, 2)), 4, (2, 2))) < 1e-12
    vals = []
    for sgn in (1, -1):
        v = np.zeros(4, dtype=complex)
        v[1], v[2] = 1 / np.sqrt(2), sgn / np.sqrt(2)
        vals.append(o.spin_square(v, 2, (1, 1)))
    np.testing.assert_allclose(sorted(vals), [0.0, 2.0], atol=1e-12)


def test_spin_square_host_sequence(monkeypatch):
    """The commutator form the GPU composition evaluates, with the excitation
    and inner-product entry points replaced by the oracle's, equals the
    oracle's S_+ construction."""
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _state
    from ffsim_gb300 import states as st
    from oracle import ffsim_oracle as o

    tensors = {}

    def keep(t):
        tensors[t.data_ptr()] = t
        return t

    def fake_call(name, src, dst, _code, norb, na, nb, spin, p, q, _stream):
        assert name == "ffgb_apply_excitation"
        v2 = tensors[src].numpy().reshape(o.dim(norb, na), o.dim(norb, nb))
        tensors[dst].copy_(torch.from_numpy(o._apply_excitation(v2, norb, (na, nb), p, q, spin).reshape(-1)))

    def prep(vec, norb, nelec, *, copy):
        arr = np.array(vec, dtype=complex)
        return _state.Prepared(keep(torch.from_numpy(arr)), arr.shape, True)

    real_empty_like = torch.empty_like
    monkeypatch.setattr(st._lib, "call", fake_call)
    monkeypatch.setattr(st, "prepare", prep)
    monkeypatch.setattr(st, "stream_ptr", lambda t: 0)
    monkeypatch.setattr(st, "vdot", lambda x, y: complex(np.vdot(x.numpy(), y.numpy())))
    monkeypatch.setattr(st.torch, "empty_like", lambda t: keep(real_empty_like(t)))
    rng = np.random.default_rng(5)
    for norb, ne in [(4, (2, 2)), (5, (3, 2)), (4, (1, 3)), (3, (0, 2))]:
        d = o.dim(norb, ne)
        v = rng.standard_normal(d) + 1j * rng.standard_normal(d)
        assert abs(f.spin_square(v, norb, ne) - o.spin_square(v, norb, ne)) < 1e-10


@pytest.mark.gpu
def test_gpu_spin_square(cuda):
    import torch

    import ffsim_gb300 as f
    from oracle import ffsim_oracle as o

    rng = np.random.default_rng(6)
    for norb, ne in [(4, (2, 2)), (5, (3, 2)), (6, (1, 4))]:
        d = o.dim(norb, ne)
        v = rng.standard_normal(d) + 1j * rng.standard_normal(d)
        exp = o.spin_square(v, norb, ne)
        assert abs(f.spin_square(v, norb, ne) - exp) < 1e-10 * max(1.0, abs(exp))
        t = torch.from_numpy(v / np.linalg.norm(v)).to("cuda").to(torch.complex64)
        assert abs(f.spin_square(t, norb, ne) - exp / np.vdot(v, v).real) < 1e-4
    assert abs(f.spin_square(f.hartree_fock_state(6, (3, 3)), 6, (3, 3))) < 1e-12


@pytest.mark.parametrize("norb, nelec", [(3, (2, 1)), (4, (2, 2)), (3, (1, 2))])
def test_spinful_to_spinless(norb, nelec):
    """The spinless RDMs of the converted vector (a (n_a + n_b, 0) system on
    2 norb orbitals, from the oracle's definition) equal the converted spinful
    RDMs: this fixes the address map and every block's sign."""
    import torch

    import ffsim_gb300 as f
    from oracle import ffsim_oracle as o

    v = o.random_state_vector(o.dim(norb, nelec), seed=norb + nelec[0])
    w = f.spinful_to_spinless_vec(v, norb, nelec)
    assert np.isclose(np.linalg.norm(w), 1.0)
    n2, ne = 2 * norb, (sum(nelec), 0)
    rdm1 = o.rdm1s(v, norb, nelec)
    np.testing.assert_allclose(f.spinful_to_spinless_rdm1(rdm1[0], rdm1[1]), o.rdm1s(w, n2, ne)[0], atol=1e-12)
    aa, ab, bb = o.rdm2s(v, norb, nelec)
    np.testing.assert_allclose(f.spinful_to_spinless_rdm2(aa, ab, bb), o.rdm2s(w, n2, ne)[0], atol=1e-12)
    wt = f.spinful_to_spinless_vec(torch.from_numpy(v), norb, nelec)
    np.testing.assert_allclose(wt.numpy(), w)


def test_wick_golden(golden):
    """Products and powers of one-body operators on a Slater determinant
    against the reference's own Wick code."""
    import ffsim_gb300 as f

    rho, mats = golden["wick_rho"], list(golden["wick_mats"])
    for k in range(5):
        assert abs(f.expectation_one_body_product(rho, mats[:k]) - golden["wick_prod"][k]) < 1e-10
    for k in range(4):
        assert abs(f.expectation_one_body_power(rho, mats[0], k) - golden["wick_pow"][k]) < 1e-10


def test_wick_against_state_vectors():
    """The same expectations from the state vector itself (oracle), for a
    determinant of 2 electrons in 5 spin orbitals."""
    import ffsim_gb300 as f
    from oracle import ffsim_oracle as o

    norb, ne = 5, (2, 0)
    rng = np.random.default_rng(1)
    u = o.random_unitary(norb, seed=rng)
    vec = np.zeros(o.dim(norb, ne), dtype=complex)
    vec[0] = 1
    vec = o.apply_orbital_rotation(vec, (u, None), norb, ne)
    rho = o.rdm1s(vec, norb, ne)[0]
    mats = [rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb)) for _ in range(3)]
    for k in range(1, 4):
        v = vec
        for m in reversed(mats[:k]):
            v = o.one_body_action(v, m, norb, ne)
        assert abs(np.vdot(vec, v) - f.expectation_one_body_product(rho, mats[:k])) < 1e-12
