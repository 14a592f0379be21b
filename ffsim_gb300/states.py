"""State helpers: dimensions, string tables (host), Hartree-Fock state, inner products."""

from __future__ import annotations

import itertools
import math
from functools import lru_cache

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import dim, dims, stream_ptr

__all__ = ["dim", "dims", "make_strings", "hartree_fock_state", "vdot", "addresses_to_strings"]


@lru_cache(maxsize=None)
def make_strings(norb: int, nocc: int) -> np.ndarray:
    """Occupation bitstrings in address order (ascending integers with ``nocc``
    set bits); the string order of python/ffsim/_cistring.py:21-24."""
    if nocc < 0 or nocc > norb:
        return np.zeros(0, dtype=np.int64)
    out = np.fromiter(
        (sum(1 << i for i in c) for c in itertools.combinations(range(norb), nocc)),
        dtype=np.int64, count=math.comb(norb, nocc))
    out.sort()
    return out


def addresses_to_strings(addresses, norb: int, nocc: int) -> np.ndarray:
    """Bitstrings of the given addresses within one spin sector."""
    return make_strings(norb, nocc)[np.asarray(addresses)]


def hartree_fock_state(norb: int, nelec, *, dtype=torch.complex128, device="cuda") -> torch.Tensor:
    """The Hartree-Fock state: one-hot at address 0 (python/ffsim/states/slater.py:122-138)."""
    n = dim(norb, nelec)
    t = torch.empty(n, dtype=dtype, device=device)
    code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
    _lib.call("ffgb_hartree_fock", t.data_ptr(), code, n, stream_ptr(t))
    return t


def vdot(x: torch.Tensor, y: torch.Tensor) -> complex:
    """sum conj(x) y accumulated in FP64 on the device."""
    if x.dtype != y.dtype or x.numel() != y.numel():
        raise ValueError("vdot needs two vectors of the same dtype and size")
    x = x.contiguous()
    y = y.contiguous()
    out = np.zeros(2)
    code = _lib.FFGB_C64 if x.dtype == torch.complex64 else _lib.FFGB_C128
    _lib.call("ffgb_vdot", x.data_ptr(), y.data_ptr(), code, x.numel(), _lib.dptr(out), stream_ptr(x))
    return complex(out[0], out[1])

