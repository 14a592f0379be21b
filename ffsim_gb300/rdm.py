"""Reduced density matrices of a state vector, the GPU counterpart of
python/ffsim/states/rdm.py:73-274 (ranks 1 and 2).

rdm1[p, q] = <psi| a+_p a_q |psi> per spin sector comes from the transition
one-body density kernel (``ffgb_transition_rdm1``) with both states psi: one
CTA per orbital pair and block of rows, FP64 partial sums reduced on the host
in a fixed order.  Rank 2 uses <E^t_pq E^s_rs> = the transition density
between psi and E^s_rs psi (``ffgb_apply_excitation``), one pair of calls per
(s, r, s) index, and the reference's index conventions:
reorder=False: rdm2[p, q, r, s] = <p+ q r+ s>; reorder=True (default):
rdm2[p, q, r, s] = <p+ r+ s q>, which for one spin subtracts delta_qr rdm1[p, s].
"""

from __future__ import annotations

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import prepare, scratch, split_nelec, stream_ptr


def _transition(x: torch.Tensor, y: torch.Tensor, norb: int, nelec, buf, nbytes) -> np.ndarray:
    code = _lib.FFGB_C64 if x.dtype == torch.complex64 else _lib.FFGB_C128
    out = np.zeros(4 * norb * norb)
    _lib.call("ffgb_transition_rdm1", x.data_ptr(), y.data_ptr(), code, norb, nelec[0], nelec[1], _lib.dptr(out),
              buf.data_ptr(), nbytes, stream_ptr(x))
    return out.view(np.complex128).reshape(2, norb, norb)


def rdms(vec, norb: int, nelec: tuple[int, int], *, rank: int = 1, spin_summed: bool = False,
         reorder: bool = True):
    """The RDMs of ``vec`` up to ``rank`` (``ffsim.rdms``).

    rank 1: ``[rdm1_alpha, rdm1_beta]`` (2, norb, norb), or their sum with
    ``spin_summed=True``.  rank 2: ``(rdm1, rdm2)`` with rdm2 the stack
    ``[aa, ab, bb]`` (3, norb, norb, norb, norb), or aa + ab + ba + bb with
    ``spin_summed=True``."""
    if rank not in (1, 2):
        raise NotImplementedError(
            f"Computing the rank {rank} reduced density matrix is currently not supported.")
    n_alpha, n_beta = split_nelec(nelec)
    if n_beta < 0:
        raise ValueError("rdms needs the electron numbers of both spin sectors")
    ne = (n_alpha, n_beta)
    p = prepare(vec, norb, ne, copy=False)
    t = p.tensor.reshape(-1)
    buf, nbytes = scratch(t, 3, norb, n_alpha, n_beta)
    rdm1 = _transition(t, t, norb, ne, buf, nbytes)
    if rank == 1:
        return rdm1.sum(axis=0) if spin_summed else rdm1
    code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
    y = torch.empty_like(t)
    # ee[t][s][p, q, r, s'] = <E^t_pq E^s_rs'>
    ee = np.zeros((2, 2, norb, norb, norb, norb), dtype=complex)
    for sig in range(2):
        for r in range(norb):
            for s_ in range(norb):
                _lib.call("ffgb_apply_excitation", t.data_ptr(), y.data_ptr(), code, norb, n_alpha, n_beta, sig, r,
                          s_, stream_ptr(t))
                ee[:, sig, :, :, r, s_] = _transition(t, y, norb, ne, buf, nbytes)
    aa, ab, bb = ee[0, 0], ee[0, 1], ee[1, 1]
    if reorder:
        eye = np.eye(norb)
        aa = aa - np.einsum("qr,ps->pqrs", eye, rdm1[0])
        bb = bb - np.einsum("qr,ps->pqrs", eye, rdm1[1])
    if spin_summed:
        return rdm1.sum(axis=0), aa + ab + ab.transpose(2, 3, 0, 1) + bb
    return rdm1, np.stack([aa, ab, bb])
