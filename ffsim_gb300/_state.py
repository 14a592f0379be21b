"""Conversions between user vectors and device buffers for the C ABI."""

from __future__ import annotations

import math

import numpy as np
import torch

from ffsim_gb300 import _lib


def dims(norb: int, nelec) -> tuple[int, int]:
    """(dim_a, dim_b) of the FCI space (python/ffsim/states/dimensions.py:18-33)."""
    n_alpha, n_beta = nelec
    return math.comb(norb, n_alpha), math.comb(norb, n_beta)


def dim(norb: int, nelec) -> int:
    """Dimension of the FCI space (python/ffsim/states/dimensions.py:36-50)."""
    if isinstance(nelec, (int, np.integer)):
        return math.comb(norb, int(nelec))
    n_alpha, n_beta = nelec
    return math.comb(norb, n_alpha) * math.comb(norb, n_beta)


def split_nelec(nelec) -> tuple[int, int]:
    """(n_alpha, n_beta) with n_beta = -1 for a spinless system."""
    if isinstance(nelec, (int, np.integer)):
        return int(nelec), -1
    n_alpha, n_beta = nelec
    return int(n_alpha), int(n_beta)


class Prepared:
    """A device tensor ready for the C ABI plus how to hand it back."""

    def __init__(self, tensor: torch.Tensor, shape, to_numpy: bool):
        self.tensor = tensor
        self.shape = shape
        self.to_numpy = to_numpy

    @property
    def dtype_code(self) -> int:
        return _lib.FFGB_C64 if self.tensor.dtype == torch.complex64 else _lib.FFGB_C128

    def ptr(self) -> int:
        return self.tensor.data_ptr()

    def finish(self, t: torch.Tensor | None = None):
        t = self.tensor if t is None else t
        t = t.reshape(self.shape)
        if self.to_numpy:
            return t.cpu().numpy()
        return t


def prepare(vec, norb: int, nelec, *, copy: bool) -> Prepared:
    """Move `vec` to a contiguous complex CUDA tensor of the right size."""
    expected = dim(norb, nelec)
    to_numpy = not isinstance(vec, torch.Tensor)
    if to_numpy:
        arr = np.asarray(vec)
        if not np.iscomplexobj(arr) or arr.dtype not in (np.complex64, np.complex128):
            arr = arr.astype(np.complex128)
        t = torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")
        copy = False
    else:
        t = vec
        if not t.is_cuda:
            raise ValueError("ffsim_gb300 operates on CUDA tensors (or numpy arrays)")
        if t.dtype not in (torch.complex64, torch.complex128):
            t = t.to(torch.complex128)
            copy = False
    shape = tuple(t.shape)
    if t.numel() != expected:
        raise ValueError(f"vector has {t.numel()} entries, expected {expected} for norb={norb}, nelec={nelec}")
    if copy:
        t = t.clone(memory_format=torch.contiguous_format)
    elif not t.is_contiguous():
        t = t.contiguous()
    return Prepared(t, shape, to_numpy)


def stream_ptr(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def scratch(t: torch.Tensor, op: int, norb: int, n_alpha: int, n_beta: int) -> tuple[torch.Tensor, int]:
    code = _lib.FFGB_C64 if t.dtype == torch.complex64 else _lib.FFGB_C128
    n = int(_lib.load().ffgb_scratch_bytes(op, code, norb, n_alpha, n_beta))
    buf = torch.empty(max(n, 256), dtype=torch.uint8, device=t.device)
    return buf, n
