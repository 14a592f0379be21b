"""Reduced density matrices of a state vector, the GPU counterpart of
python/ffsim/states/rdm.py:73-170 (rank 1).

rdm1[p, q] = <psi| a+_p a_q |psi> per spin sector, from the transition
one-body density kernel (``ffgb_transition_rdm1``) with both states psi:
one CTA per orbital pair and block of rows, FP64 partial sums reduced on the
host in a fixed order.
"""

from __future__ import annotations

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import prepare, scratch, split_nelec, stream_ptr


def rdms(vec, norb: int, nelec: tuple[int, int], *, rank: int = 1, spin_summed: bool = False,
         reorder: bool = True) -> np.ndarray:
    """The 1-RDMs of ``vec`` (``ffsim.rdms``): ``[rdm1_alpha, rdm1_beta]`` of
    shape (2, norb, norb), or their sum with ``spin_summed=True``.  Only rank 1
    is available (``reorder`` only affects rank 2 and higher)."""
    if rank != 1:
        raise NotImplementedError(
            f"Computing the rank {rank} reduced density matrix is currently not supported.")
    n_alpha, n_beta = split_nelec(nelec)
    if n_beta < 0:
        raise ValueError("rdms needs the electron numbers of both spin sectors")
    p = prepare(vec, norb, (n_alpha, n_beta), copy=False)
    t = p.tensor
    code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
    buf, nbytes = scratch(t, 3, norb, n_alpha, n_beta)
    out = np.zeros(4 * norb * norb)
    _lib.call("ffgb_transition_rdm1", t.data_ptr(), t.data_ptr(), code, norb, n_alpha, n_beta, _lib.dptr(out),
              buf.data_ptr(), nbytes, stream_ptr(t))
    rdm = out.view(np.complex128).reshape(2, norb, norb)
    return rdm.sum(axis=0) if spin_summed else rdm
