"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared symbol, and the host planning code (Givens decomposition,
eigendecomposition, cosine-sine plans with the kernel's addressing) matches
the oracle."""

from __future__ import annotations

import math
import re
from pathlib import Path

import numpy as np
import pytest

import plan_emulator as pe
from oracle import ffsim_oracle as o

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    text = (ROOT / "include" / "ffsim_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(ffgb_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    from ffsim_gb300 import _lib

    lib = _lib.load()
    names = _declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, name
    assert lib.ffgb_version() >= 100


def test_givens_decomposition_matches_oracle():
    import ffsim_gb300 as f

    rng = np.random.default_rng(11)
    for n in range(1, 13):
        u = o.random_unitary(n, seed=rng)
        got, gd = f.linalg.givens_decomposition(u)
        ref, rd = o.givens_decomposition(u)
        assert len(got) == len(ref)
        for (c1, s1, i1, j1), (c2, s2, i2, j2) in zip(got, ref):
            assert (i1, j1) == (i2, j2)
            assert abs(c1 - c2) < 1e-12 and abs(s1 - s2) < 1e-12
        np.testing.assert_allclose(gd, rd, atol=1e-12)
    with pytest.raises(ValueError):
        f.linalg.givens_decomposition(np.zeros((2, 3)))


def test_givens_tolerance_skips_identity():
    import ffsim_gb300 as f

    rots, diag = f.linalg.givens_decomposition(np.eye(5))
    assert rots == []
    np.testing.assert_allclose(diag, np.ones(5))


def test_eigh():
    import ffsim_gb300 as f

    rng = np.random.default_rng(3)
    for n in (1, 4, 9, 16):
        g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        h = (g + g.conj().T) / 2
        w, v = f.linalg.eigh(h)
        np.testing.assert_allclose(w, np.linalg.eigvalsh(h), atol=1e-12)
        np.testing.assert_allclose(v @ np.diag(w) @ v.conj().T, h, atol=1e-12)


def _plan(u, use_windows):
    from ffsim_gb300 import _lib

    m = _lib.cmat(u)
    out = np.zeros(20000)
    n = np.zeros(1, dtype=np.int32)
    _lib.call("ffgb_debug_plan", _lib.dptr(m), u.shape[0], int(use_windows), _lib.dptr(out), len(out),
              n.ctypes.data_as(_lib._ip))
    return pe.parse(out[: n[0]])


@pytest.mark.parametrize("norb, nocc", [(1, 1), (2, 1), (4, 2), (5, 3), (7, 3), (8, 4), (9, 4), (9, 5),
                                         (10, 5), (11, 4), (12, 6), (13, 6)])
@pytest.mark.parametrize("use_windows", [True, False])
def test_plan_addressing_matches_oracle(norb, nocc, use_windows):
    """The serialized plan applied with the kernel's addressing equals W(U)."""
    rng = np.random.default_rng(norb * 31 + nocc)
    u = o.random_unitary(norb, seed=rng)
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    plan = _plan(u, use_windows)
    expect_kind = (2 if norb <= 8 else 3) if use_windows else 1
    assert plan["kind"] == expect_kind
    assert plan["err"] < 1e-12
    got = pe.apply_plan(plan, vec, norb, nocc)
    np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, u, norb, nocc), atol=1e-12)


@pytest.mark.parametrize("norb, nocc, n_stages", [(9, 1, 3), (9, 4, 3), (10, 3, 3), (11, 5, 3), (12, 3, 3),
                                                   (13, 2, 5), (16, 2, 5), (17, 2, 9), (17, 3, 9), (18, 2, 9),
                                                   (18, 3, 9)])
def test_stage_sequence_matches_oracle(norb, nocc, n_stages):
    """The stage kernels' sequence (three overlapping windows up to 12
    orbitals, cosine-sine stages above) applied string by string equals W(U)."""
    rng = np.random.default_rng(norb * 7 + nocc)
    u = o.random_unitary(norb, seed=rng)
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    plan = _plan(u, True)
    assert plan["kind"] == 3 and plan["err"] < 1e-10
    assert len(plan["ops"]) == n_stages
    assert all(op["b"] <= 8 for op in plan["ops"] if op["type"] == 0)
    got = pe.apply_ops(plan, vec, norb, nocc)
    np.testing.assert_allclose(got, o.apply_orbital_rotation(vec, u, norb, nocc), atol=1e-11)


@pytest.mark.parametrize("norb, nocc", [(10, 4), (12, 6), (14, 5)])
def test_sandwich_plans_carry_the_phases(norb, nocc):
    """The stage-path matvec term W(U) Z W(U^dag): with the plan of U^dag =
    diag(d) N run without its final phases, the plan of U diag(d) gives the
    same vector (Z diagonal in the strings, so it commutes with W(diag(d)))."""
    rng = np.random.default_rng(norb * 13 + nocc)
    u = o.random_unitary(norb, seed=rng)
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    z = rng.normal(size=vec.size)
    pd = _plan(u.conj().T, True)
    d = pd["ops_diag"]
    assert np.abs(d - 1).max() > 1e-3  # the phases are not trivial
    pu = _plan(u * d[None, :], True)
    assert pu["kind"] == 3 and pu["err"] < 1e-10
    half = pe.apply_ops(dict(pd, ops_diag=np.ones(norb)), vec, norb, nocc)
    got = pe.apply_ops(pu, z * half, norb, nocc)
    want = o.apply_orbital_rotation(z * o.apply_orbital_rotation(vec, u.conj().T, norb, nocc), u, norb, nocc)
    np.testing.assert_allclose(got, want, atol=1e-11)


def test_stage_sequence_special_matrices():
    """Block-diagonal, permutation and identity unitaries take the three-window form."""
    for norb, nocc in [(9, 3), (10, 4), (12, 2)]:
        blk = np.zeros((norb, norb), dtype=complex)
        blk[:8, :8] = o.random_unitary(8, seed=4)
        blk[8:, 8:] = o.random_unitary(norb - 8, seed=5)
        for u in [np.eye(norb, dtype=complex), np.eye(norb)[::-1].astype(complex),
                  np.roll(np.eye(norb), 5, axis=0).astype(complex), blk]:
            plan = _plan(u, True)
            assert plan["err"] < 1e-10
            vec = o.random_state_vector(math.comb(norb, nocc), seed=6)
            assert plan["kind"] == 3 and len(plan["ops"]) == 3
            np.testing.assert_allclose(pe.apply_ops(plan, vec, norb, nocc),
                                       o.apply_orbital_rotation(vec, u, norb, nocc), atol=1e-11)


def test_plan_special_matrices():
    """Identity, permutations and block-diagonal unitaries (degenerate cosine-sine cases)."""
    for norb, nocc in [(10, 5), (12, 5), (16, 8)]:
        mats = [np.eye(norb), np.eye(norb)[::-1].copy(), np.roll(np.eye(norb), 3, axis=0)]
        blk = np.zeros((norb, norb), dtype=complex)
        h = norb // 2
        blk[:h, :h] = o.random_unitary(h, seed=1)
        blk[h:, h:] = o.random_unitary(norb - h, seed=2)
        mats.append(blk)
        for u in mats:
            plan = _plan(u.astype(complex), True)
            assert plan["err"] < 1e-12
            if norb <= 12:
                vec = o.random_state_vector(math.comb(norb, nocc), seed=3)
                np.testing.assert_allclose(pe.apply_plan(plan, vec, norb, nocc),
                                           o.apply_orbital_rotation(vec, u, norb, nocc), atol=1e-12)


def _hopping_evolution(norb, t, band, seed):
    """exp(-i t h) for a random Hermitian h with the given bandwidth: a banded,
    near-identity unitary for small t (short-time evolutions, lattice models)."""
    import scipy.linalg

    rng = np.random.default_rng(seed)
    g = rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))
    h = np.triu(np.tril(g + g.conj().T, band), -band)
    return scipy.linalg.expm(-1j * t * h)


@pytest.mark.parametrize("norb, nocc", [(9, 3), (12, 4), (13, 3), (16, 2), (17, 2), (18, 2)])
@pytest.mark.parametrize("t, band", [(1e-6, 1), (0.01, 1), (0.1, 1), (1.0, 1), (0.3, 2), (1e-3, 17)])
def test_stage_sequence_banded_and_near_identity(norb, nocc, t, band):
    """Banded and near-identity unitaries stay on the stage sequence: cosines
    within rounding of 1 hide their sines from the diagonal block, so the
    cosine-sine split resolves them from the off-diagonal block."""
    u = _hopping_evolution(norb, t, band, seed=norb * 100 + band)
    plan = _plan(u, True)
    assert plan["kind"] == 3 and plan["err"] < 1e-10
    vec = o.random_state_vector(math.comb(norb, nocc), seed=9)
    np.testing.assert_allclose(pe.apply_ops(plan, vec, norb, nocc),
                               o.apply_orbital_rotation(vec, u, norb, nocc), atol=1e-11)


def test_scratch_sizes():
    from ffsim_gb300 import _lib

    lib = _lib.load()
    s64 = lib.ffgb_scratch_bytes(0, 0, 16, 8, 8)
    s128 = lib.ffgb_scratch_bytes(0, 1, 16, 8, 8)
    assert s64 >= 12870**2 * 8 and s128 >= 12870**2 * 16
    assert lib.ffgb_scratch_bytes(1, 0, 16, 8, 8) >= 2 * 12870**2 * 8


def test_argument_errors_map_to_python_exceptions():
    import ffsim_gb300 as f
    from ffsim_gb300 import _lib

    with pytest.raises(TypeError):
        _lib.call("ffgb_apply_orbital_rotation", None, 7, 4, 2, 2, None, None, None, 0, None)
    with pytest.raises(ValueError):
        _lib.call("ffgb_apply_orbital_rotation", None, 0, 4, 5, 2, None, None, None, 0, None)
    with pytest.raises(NotImplementedError):
        _lib.call("ffgb_apply_orbital_rotation", None, 0, 40, 2, 2, None, None, None, 0, None)
    assert f.dim(16, (8, 8)) == 12870**2


def test_mis_sized_inputs_are_rejected_on_the_host():
    """The C ABI reads norb x norb (or norb) elements through each pointer; the
    Python layer rejects arrays of another size before any call or launch."""
    import ffsim_gb300 as f
    from ffsim_gb300 import _lib

    with pytest.raises(ValueError, match="orbital rotation"):
        _lib.cmat(np.eye(3), (4, 4), "orbital rotation")
    assert _lib.cmat(None, (4, 4)) is None
    assert _lib.rmat(np.zeros(4), (4,)).shape == (4,)
    ham = f.random.random_double_factorized_hamiltonian(4, rank=2, seed=1)
    with pytest.raises(ValueError):
        f.linear_operator(ham, 5, (2, 2))
    bad = f.DoubleFactorizedHamiltonian(np.eye(4), np.zeros((2, 4, 4)), np.zeros((3, 4, 4), dtype=complex))
    with pytest.raises(ValueError):
        bad._arrays()
    ucj = f.random.random_ucj_op_spin_balanced(4, n_reps=1, seed=2)
    with pytest.raises(ValueError):
        f.apply_unitary(np.zeros(100, dtype=complex), ucj, 5, (2, 2))


def test_null_buffers_are_refused_before_any_launch():
    """A NULL state, output or result pointer is an argument error on the host
    (this runs without a GPU: the check comes before any CUDA call)."""
    from ffsim_gb300 import _lib

    with pytest.raises(ValueError):
        _lib.call("ffgb_apply_orbital_rotation", None, 0, 4, 2, 2, None, None, None, 0, None)
    with pytest.raises(ValueError):
        _lib.call("ffgb_apply_diag_coulomb_evolution", None, 1, 4, 2, 2, None, None, None, 0.5, 0, None, None,
                  None, 0, None)
    with pytest.raises(ValueError):
        _lib.call("ffgb_vdot", None, None, 0, 10, None, None)
    with pytest.raises(ValueError):
        _lib.call("ffgb_hartree_fock", None, 0, 10, None)
    with pytest.raises(TypeError):
        _lib.call("ffgb_hartree_fock", None, 5, 10, None)


def test_linear_operator_inputs_and_scipy_interop():
    """Vector-length checks, column-by-column application, device and dtype
    round trips, and SciPy's aslinearoperator / eigsh / expm_multiply on the
    operator (a dense Hermitian matrix stands in for the kernels, and a
    subclass keeps the vectors on the CPU)."""
    import scipy.sparse.linalg as sla
    import torch

    from ffsim_gb300.protocols import LinearOperator as GpuOperator

    class LinearOperator(GpuOperator):
        def _on_device(self, t):
            return t.to(torch.complex128) if t.dtype not in (torch.complex64, torch.complex128) else t
    rng = np.random.default_rng(4)
    n = 12
    g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    h = (g + g.conj().T) / 2
    ht = torch.from_numpy(h)

    def mv(t):
        assert t.dim() == 1 and t.numel() == n
        return (ht.to(t.dtype) @ t)

    op = LinearOperator((n, n), mv, expectation=lambda v: float(torch.vdot(v, mv(v)).real))
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(op @ x, h @ x, atol=1e-12)
    np.testing.assert_allclose(op @ x[:, None], (h @ x)[:, None], atol=1e-12)
    xs = rng.standard_normal((n, 3)) + 0j
    np.testing.assert_allclose(op.matvec(xs), h @ xs, atol=1e-12)
    np.testing.assert_allclose(op @ x.real, h @ x.real, atol=1e-12)  # real input promoted
    got = op @ torch.from_numpy(x).to(torch.complex64)
    assert got.dtype == torch.complex64 and got.device.type == "cpu"
    assert abs(op.expectation(x) - np.vdot(x, h @ x).real) < 1e-10
    for bad in (np.zeros(n + 1, dtype=complex), np.zeros((n - 1, 2), dtype=complex)):
        with pytest.raises(ValueError, match="dimension mismatch"):
            op @ bad
    with pytest.raises(ValueError, match="dimension mismatch"):
        op.expectation(np.zeros(n - 1, dtype=complex))
    # SciPy routines take the object as it is
    lo = sla.aslinearoperator(op)
    w = sla.eigsh(lo, k=1, which="SA", return_eigenvectors=False)
    assert abs(w[0] - np.linalg.eigvalsh(h)[0]) < 1e-8
    import scipy.linalg

    np.testing.assert_allclose(sla.expm_multiply(-0.3j * lo, x, traceA=0.0),
                               scipy.linalg.expm(-0.3j * h) @ x, atol=1e-10)


@pytest.mark.parametrize("norb, nocc", [(13, 3), (16, 2), (17, 2), (18, 2)])
def test_stage_sequence_permutations_and_blocks(norb, nocc):
    """Permutations (cosines and sines exactly 0 or 1) and block-diagonal
    unitaries take the stage sequence above 12 orbitals too, and the emulated
    kernels reproduce W(U)."""
    rng = np.random.default_rng(norb * 5 + nocc)
    h = norb // 2
    blk = np.zeros((norb, norb), dtype=complex)
    blk[:h, :h] = o.random_unitary(h, seed=rng)
    blk[h:, h:] = o.random_unitary(norb - h, seed=rng)
    mats = [np.eye(norb)[rng.permutation(norb)].astype(complex), np.eye(norb)[::-1].astype(complex), blk,
            blk @ np.eye(norb)[rng.permutation(norb)]]
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    for u in mats:
        plan = _plan(u, True)
        assert plan["kind"] == 3 and plan["err"] < 1e-10
        np.testing.assert_allclose(pe.apply_ops(plan, vec, norb, nocc), o.apply_orbital_rotation(vec, u, norb, nocc),
                                   atol=1e-11)


@pytest.mark.parametrize("norb, nocc", [(14, 2), (16, 2), (15, 3)])
def test_sector_kernel_plan_structured_matrices(norb, nocc):
    """The five-stage form the shared-memory sector kernel runs (complex128 and
    single-sector calls up to 16 orbitals), for banded, near-identity and
    permutation unitaries, emulated with the kernel's addressing."""
    rng = np.random.default_rng(norb * 9 + nocc)
    mats = [_hopping_evolution(norb, 0.05, 1, seed=norb), _hopping_evolution(norb, 1.0, 2, seed=norb + 1),
            np.eye(norb)[rng.permutation(norb)].astype(complex), o.random_unitary(norb, seed=rng)]
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    for u in mats:
        plan = _plan(u, True)  # carries the five-stage fields beside the stage sequence
        assert plan["kind"] == 3 and plan["err"] < 1e-10
        np.testing.assert_allclose(pe.apply_plan(plan, vec, norb, nocc), o.apply_orbital_rotation(vec, u, norb, nocc),
                                   atol=1e-11)


def test_approx_eq_protocol():
    import ffsim_gb300 as f

    a = f.random.random_double_factorized_hamiltonian(3, rank=2, seed=1)
    b = f.DoubleFactorizedHamiltonian(a.one_body_tensor + 1e-10, a.diag_coulomb_mats, a.orbital_rotations,
                                      constant=a.constant)
    assert f.approx_eq(a, b) and not f.approx_eq(a, b, rtol=0, atol=1e-12)
    ucj = f.random.random_ucj_op_spin_balanced(3, seed=2)
    assert f.approx_eq(ucj, ucj) and not f.approx_eq(ucj, a)
    assert f.approx_eq(1, 1) and not f.approx_eq(1, 2)


@pytest.mark.parametrize("norb, nocc", [(13, 6), (14, 7), (15, 7), (16, 8), (17, 8), (17, 9), (18, 9)])
def test_stage_sequence_full_size_sectors(norb, nocc):
    """The stage sequence with the kernels' addressing on whole half-filled
    sectors (48,620 strings at norb 18): the group bases, member offsets and
    cross-half partner tables the full-size launches use, for a random and a
    banded unitary."""
    rng = np.random.default_rng(norb * 3 + nocc)
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    for u in (o.random_unitary(norb, seed=rng), _hopping_evolution(norb, 0.2, 1, seed=norb)):
        plan = _plan(u, True)
        assert plan["kind"] == 3 and plan["err"] < 1e-10
        np.testing.assert_allclose(pe.apply_ops(plan, vec, norb, nocc), o.apply_orbital_rotation(vec, u, norb, nocc),
                                   atol=1e-12)


@pytest.mark.parametrize("norb, nocc", [(13, 6), (14, 7), (15, 8), (16, 8)])
def test_sector_kernel_plan_full_size_sectors(norb, nocc):
    """The shared-memory sector kernel's five-stage form (complex128 and
    single-sector calls) on whole half-filled sectors, random and banded."""
    rng = np.random.default_rng(norb * 7 + nocc)
    vec = o.random_state_vector(math.comb(norb, nocc), seed=rng)
    for u in (o.random_unitary(norb, seed=rng), _hopping_evolution(norb, 0.2, 1, seed=norb)):
        plan = _plan(u, True)
        np.testing.assert_allclose(pe.apply_plan(plan, vec, norb, nocc), o.apply_orbital_rotation(vec, u, norb, nocc),
                                   atol=1e-12)
