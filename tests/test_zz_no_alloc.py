"""ffgb_contract_diag_coulomb_static: the contraction with its scratch in a
fixed device array, checked against ffgb_contract_diag_coulomb.

The file name sorts last so that the GPU tests run it after every other
test; it also passes on its own."""

from __future__ import annotations

import numpy as np
import pytest

CASES = [(2, (1, 1)), (3, (2, 1)), (8, (4, 4)), (12, (6, 5))]


def _mats(norb, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(3):
        m = rng.standard_normal((norb, norb))
        out.append(np.ascontiguousarray(m + m.T))
    return out


def _call(name, vec, out, code, norb, nelec, mats, zrep, accumulate):
    import torch
    from ffsim_gb300 import _lib

    aa, ab, bb = mats
    _lib.call(name, vec.data_ptr(), out.data_ptr(), code, norb, nelec[0], nelec[1], _lib.dptr(aa),
              _lib.dptr(ab), _lib.dptr(bb), zrep, accumulate, torch.cuda.current_stream().cuda_stream)


@pytest.mark.gpu
@pytest.mark.parametrize("norb, nelec", CASES)
@pytest.mark.parametrize("dtype_name, rtol", [("complex64", 1e-6), ("complex128", 1e-12)])
@pytest.mark.parametrize("zrep", [0, 1])
@pytest.mark.parametrize("accumulate", [0, 1])
def test_static_matches_allocating_entry_point(cuda, norb, nelec, dtype_name, rtol, zrep, accumulate):
    import torch
    import ffsim_gb300 as f

    dtype = getattr(torch, dtype_name)
    code = 0 if dtype == torch.complex64 else 1
    dim = f.dim(norb, nelec)
    gen = torch.Generator(device="cpu").manual_seed(7 * norb + zrep)
    vec = torch.randn(dim, dtype=dtype, generator=gen).to(cuda)
    start = torch.randn(dim, dtype=dtype, generator=gen).to(cuda)
    mats = _mats(norb, seed=norb + 100 * zrep)

    expected = start.clone()
    _call("ffgb_contract_diag_coulomb", vec, expected, code, norb, nelec, mats, zrep, accumulate)
    torch.cuda.synchronize()
    want = expected.cpu().numpy()
    scale = max(1.0, float(np.abs(want).max()))

    first, second = start.clone(), start.clone()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    # two calls in a row on the same stream reuse the same fixed scratch
    _call("ffgb_contract_diag_coulomb_static", vec, first, code, norb, nelec, mats, zrep, accumulate)
    _call("ffgb_contract_diag_coulomb_static", vec, second, code, norb, nelec, mats, zrep, accumulate)
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    for got in (first, second):
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=rtol, atol=rtol * scale)
    assert free_after >= free_before


@pytest.mark.gpu
def test_static_allocates_nothing_on_a_fresh_shape(cuda):
    """The first call for a shape no other test uses (norb 9, (2, 6)): the
    allocating entry point would build and cache string tables here, so a
    static call that allocated anything would show in the library's
    allocation count or in the device's free memory."""
    import torch
    import ffsim_gb300 as f
    from ffsim_gb300 import _lib

    lib = _lib.load()
    norb, nelec = 9, (2, 6)
    dim = f.dim(norb, nelec)
    gen = torch.Generator(device="cpu").manual_seed(11)
    vec = torch.randn(dim, dtype=torch.complex64, generator=gen).to(cuda)
    mats = _mats(norb, seed=11)
    first, second = torch.zeros_like(vec), torch.zeros_like(vec)
    torch.cuda.synchronize()
    allocs = lib.ffgb_device_alloc_count()
    free_before = torch.cuda.mem_get_info()[0]
    _call("ffgb_contract_diag_coulomb_static", vec, first, 0, norb, nelec, mats, 0, 0)
    _call("ffgb_contract_diag_coulomb_static", vec, second, 0, norb, nelec, mats, 0, 0)
    torch.cuda.synchronize()
    assert lib.ffgb_device_alloc_count() == allocs
    assert torch.cuda.mem_get_info()[0] >= free_before
    expected = torch.zeros_like(vec)
    _call("ffgb_contract_diag_coulomb", vec, expected, 0, norb, nelec, mats, 0, 0)
    torch.cuda.synchronize()
    want = expected.cpu().numpy()
    for got in (first, second):
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-6, atol=1e-6 * float(np.abs(want).max()))


@pytest.mark.gpu
def test_static_follows_other_shapes(cuda):
    """A call after one with a larger shape must not see stale scratch."""
    import torch
    import ffsim_gb300 as f

    for norb, nelec in [(12, (6, 6)), (4, (2, 1)), (12, (6, 6))]:
        dim = f.dim(norb, nelec)
        gen = torch.Generator(device="cpu").manual_seed(norb)
        vec = torch.randn(dim, dtype=torch.complex128, generator=gen).to(cuda)
        mats = _mats(norb, seed=3)
        want = torch.empty_like(vec)
        got = torch.empty_like(vec)
        _call("ffgb_contract_diag_coulomb", vec, want, 1, norb, nelec, mats, 0, 0)
        _call("ffgb_contract_diag_coulomb_static", vec, got, 1, norb, nelec, mats, 0, 0)
        torch.cuda.synchronize()
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-12, atol=1e-12)


def test_static_rejects_shapes_beyond_its_scratch():
    """norb 18 at half filling in complex128 with a nonzero beta-beta block
    needs about 1.1 MiB (strings plus the column table); the check runs before
    any device work, so this needs no GPU."""
    from ffsim_gb300 import _lib

    lib = _lib.load()
    null = _lib._dp()
    bb = np.ascontiguousarray(np.eye(18))
    status = lib.ffgb_contract_diag_coulomb_static(None, None, 1, 18, 9, 9, null, null, _lib.dptr(bb), 0, 0, None)
    assert status == 1  # FFGB_ERR_ARG -> ValueError
    msg = lib.ffgb_last_error().decode()
    assert "bytes of scratch" in msg and str(1 << 20) in msg


def test_static_limit_counts_the_column_table_only_when_used():
    """With mat_bb zero there is no column table, so norb 18 (9, 9) in
    complex128 fits (two string tables, 389 KB) and the call gets past the
    size check to the buffer check."""
    from ffsim_gb300 import _lib

    lib = _lib.load()
    null = _lib._dp()
    status = lib.ffgb_contract_diag_coulomb_static(None, None, 1, 18, 9, 9, null, null, null, 0, 0, None)
    assert status == 1
    assert "bytes of scratch" not in lib.ffgb_last_error().decode()
