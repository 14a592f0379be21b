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
