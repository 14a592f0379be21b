"""Full-size closed-form checks at norb 18, (9, 9): 2.36e9 amplitudes (18.9 GB
in complex64), more than 2^31 elements, so element addresses above 2^31 are
read and written.  The rotated Hartree-Fock state is a Slater determinant
whose amplitudes are products of 9 x 9 minors of the rotation; a diagonal
Coulomb evolution multiplies each amplitude by a phase known in closed form.
Amplitudes are checked at rows and columns near both ends of the state.
Peak device memory is about two states (the state and the rotation scratch)."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import ffsim_oracle as o

pytestmark = pytest.mark.gpu


def test_norb18_full_size_complex64(cuda):
    import torch

    import ffsim_gb300 as f

    norb, nelec = 18, (9, 9)
    rng = np.random.default_rng(18)
    u = o.random_unitary(norb, seed=rng)
    j = o.random_symmetric_normal(norb, scale=0.1, seed=rng)
    strings = o.make_strings(norb, 9)
    dim_a = len(strings)
    picks = [0, 1, dim_a // 2, dim_a - 2, dim_a - 1]
    occ = {a: np.array([(int(strings[a]) >> i) & 1 for i in range(norb)], dtype=float) for a in picks}
    det = {a: np.linalg.det(u[np.ix_(np.flatnonzero(occ[a]), range(9))]) for a in picks}
    # the RMS amplitude of a unit vector with dim_a**2 entries; FP32 rotations
    # leave errors near 1e-6 of it, the bound is 1e-2 of it
    tol = 1e-2 / dim_a

    psi = f.hartree_fock_state(norb, nelec, dtype=torch.complex64)
    psi = f.apply_orbital_rotation(psi, u, norb, nelec, copy=False)
    assert abs(f.vdot(psi, psi).real - 1.0) < 1e-5
    r = psi.view(dim_a, dim_a)
    for a in picks:
        for b in picks:
            assert abs(complex(r[a, b].item()) - det[a] * det[b]) < tol, (a, b)

    t = 0.7
    psi = f.apply_diag_coulomb_evolution(psi, j, t, norb, nelec, copy=False)
    r = psi.view(dim_a, dim_a)
    for a in picks:
        for b in picks:
            n = occ[a] + occ[b]
            phase = np.exp(-1j * t * 0.5 * (n @ j @ n))
            assert abs(complex(r[a, b].item()) - phase * det[a] * det[b]) < tol, (a, b)

    # undo both: back to the Hartree-Fock state, |psi - e_0|^2 from FP64 sums
    psi = f.apply_diag_coulomb_evolution(psi, j, -t, norb, nelec, copy=False)
    psi = f.apply_orbital_rotation(psi, u.conj().T, norb, nelec, copy=False)
    x0 = complex(psi[0].item())
    dist2 = f.vdot(psi, psi).real - 2.0 * x0.real + 1.0
    assert abs(x0 - 1.0) < 1e-4 and dist2 < (5e-5) ** 2, (x0, dist2)
    del psi, r
    torch.cuda.empty_cache()
