"""Double-factorized Trotter evolution (python/ffsim/trotter/double_factorized.py):
the step sequence on the CPU, the GPU evolution against the reference's golden
vectors and across precisions."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import ffsim_oracle as o


@pytest.mark.parametrize("order", [0, 1, 2, 3])
@pytest.mark.parametrize("n_terms", [1, 2, 5])
def test_step_sequence_matches_oracle(order, n_terms):
    from ffsim_gb300.trotter import simulate_trotter_step_iterator

    got = list(simulate_trotter_step_iterator(n_terms, 0.37, order))
    exp = o.trotter_step_terms(n_terms, 0.37, order)
    assert [k for k, _ in got] == [k for k, _ in exp]
    np.testing.assert_allclose([t for _, t in got], [t for _, t in exp], rtol=0, atol=1e-15)
    # every term runs for the whole step time in total
    tot = np.zeros(n_terms)
    for k, t in got:
        tot[k] += t
    np.testing.assert_allclose(tot, 0.37, atol=1e-14)


def test_argument_errors():
    import ffsim_gb300 as f

    ham = f.random.random_df_hamiltonian_normal(4, rank=2, seed=1)
    with pytest.raises(ValueError):
        f.simulate_trotter_double_factorized(np.zeros(36, dtype=complex), ham, 0.1, norb=4, nelec=(2, 2), order=-1)
    with pytest.raises(ValueError):
        f.simulate_trotter_double_factorized(np.zeros(36, dtype=complex), ham, 0.1, norb=4, nelec=(2, 2),
                                             n_steps=-1)


def _ham(g, idx):
    import ffsim_gb300 as f

    return f.DoubleFactorizedHamiltonian(g[f"trot{idx}_h1"], g[f"trot{idx}_dcm"], g[f"trot{idx}_rots"],
                                         constant=float(g[f"trot{idx}_const"]),
                                         z_representation=bool(g["trot_cases"][idx][6]))


@pytest.mark.gpu
def test_golden(cuda, golden):
    import torch

    import ffsim_gb300 as f

    for idx, (n, a, b, t, steps, order, _) in enumerate(golden["trot_cases"]):
        n, ne = int(n), (int(a), int(b))
        ham = _ham(golden, idx)
        vin = golden[f"trot{idx}_in"]
        for dtype, tol in [(torch.complex128, 1e-11), (torch.complex64, 1e-4)]:
            v = torch.from_numpy(vin).to("cuda").to(dtype)
            keep = v.clone()
            out = f.simulate_trotter_double_factorized(v, ham, float(t), norb=n, nelec=ne, n_steps=int(steps),
                                                       order=int(order))
            assert torch.equal(v, keep)  # copy=True leaves the input alone
            np.testing.assert_allclose(out.cpu().numpy().astype(complex), golden[f"trot{idx}_out"], atol=tol)


@pytest.mark.gpu
def test_stage_path_precisions(cuda):
    """norb=12 (6,6) on the complex64 stage kernels against complex128."""
    import torch

    import ffsim_gb300 as f

    norb, nelec = 12, (6, 6)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=3, seed=7)
    rng = np.random.default_rng(8)
    d = f.dim(norb, nelec)
    v = rng.standard_normal(d) + 1j * rng.standard_normal(d)
    v /= np.linalg.norm(v)
    outs = {}
    for dtype in (torch.complex64, torch.complex128):
        t = torch.from_numpy(v).to("cuda").to(dtype)
        r = f.simulate_trotter_double_factorized(t, ham, 0.2, norb=norb, nelec=nelec, n_steps=2, order=1)
        outs[dtype] = r.cpu().numpy().astype(complex)
    assert abs(np.linalg.norm(outs[torch.complex128]) - 1) < 1e-10
    assert np.linalg.norm(outs[torch.complex64] - outs[torch.complex128]) < 1e-4
