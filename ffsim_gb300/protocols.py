"""Protocol dispatch and the GPU linear-operator type.

``apply_unitary`` and ``linear_operator`` dispatch on the duck-typed
``_apply_unitary_`` / ``_linear_operator_`` methods exactly like
python/ffsim/protocols/apply_unitary_protocol.py:48-88 and
python/ffsim/protocols/linear_operator_protocol.py:40-60.
"""

from __future__ import annotations

from typing import Any, Callable, Protocol, runtime_checkable

import numpy as np
import torch


@runtime_checkable
class SupportsApplyUnitary(Protocol):
    """An object with a unitary effect on state vectors (apply_unitary_protocol.py)."""

    def _apply_unitary_(self, vec, norb: int, nelec, copy: bool): ...


@runtime_checkable
class SupportsLinearOperator(Protocol):
    """An object with a linear operator on state vectors (linear_operator_protocol.py)."""

    def _linear_operator_(self, norb: int, nelec): ...


@runtime_checkable
class SupportsApproximateEquality(Protocol):
    """An object comparable to tolerances (approximate_equality_protocol.py)."""

    def _approx_eq_(self, other: Any, rtol: float, atol: float) -> bool: ...


@runtime_checkable
class SupportsDiagonal(Protocol):
    """An operator whose diagonal can be returned (diagonal_protocol.py)."""

    def _diag_(self, norb: int, nelec): ...


@runtime_checkable
class SupportsTrace(Protocol):
    """An operator whose trace can be returned (trace_protocol.py)."""

    def _trace_(self, norb: int, nelec) -> float: ...


def apply_unitary(vec, obj: Any, norb: int, nelec, copy: bool = True):
    """Apply the unitary effect of ``obj`` to ``vec``."""
    method = getattr(obj, "_apply_unitary_", None)
    if method is not None:
        result = method(vec, norb=norb, nelec=nelec, copy=copy)
        if result is not NotImplemented:
            return result
    raise TypeError(
        "ffsim_gb300.apply_unitary failed. Object doesn't have a unitary effect.\n"
        f"type: {type(obj)}\nobject: {obj!r}\n"
        "The object did not have an _apply_unitary_ method that returned a value besides "
        "NotImplemented."
    )


def linear_operator(obj: Any, norb: int, nelec):
    """Return the GPU linear operator of ``obj``."""
    method = getattr(obj, "_linear_operator_", None)
    if method is not None:
        result = method(norb=norb, nelec=nelec)
        if result is not NotImplemented:
            return result
    raise TypeError(f"Object of type {type(obj)} has no _linear_operator_ method.")


def approx_eq(obj: Any, other: Any, rtol: float = 1e-5, atol: float = 1e-8) -> bool:
    """Whether two objects are equal to the given tolerances (``np.isclose``
    semantics): ``obj``'s ``_approx_eq_``, else ``other``'s, else ``==``
    (python/ffsim/protocols/approximate_equality_protocol.py:39-68)."""
    for a, b in ((obj, other), (other, obj)):
        method = getattr(a, "_approx_eq_", None)
        if method is not None:
            result = method(b, rtol=rtol, atol=atol)
            if result is not NotImplemented:
                return result
    return obj == other


def diag(obj: Any, norb: int, nelec) -> np.ndarray:
    """Diagonal entries of ``obj``'s operator
    (python/ffsim/protocols/diagonal_protocol.py:42-50)."""
    method = getattr(obj, "_diag_", None)
    if method is not None:
        return method(norb=norb, nelec=nelec)
    raise TypeError(
        f"Could not compute diagonal entries of object of type {type(obj)}.\n"
        "The object did not have a _diag_ method that returned its diagonal entries."
    )


def trace(obj: Any, norb: int, nelec) -> float:
    """Trace of ``obj``'s operator: its own ``_trace_`` or the sum of its
    diagonal (python/ffsim/protocols/trace_protocol.py)."""
    method = getattr(obj, "_trace_", None)
    if method is not None:
        return method(norb=norb, nelec=nelec)
    if getattr(obj, "_diag_", None) is not None:
        return float(np.sum(diag(obj, norb, nelec)))
    raise TypeError(f"Could not compute trace of object of type {type(obj)}.")


class LinearOperator:
    """A (dim x dim) operator acting on CUDA state vectors.

    ``matvec`` / ``rmatvec`` / ``@`` accept torch complex tensors (the result
    has the same dtype and device) or numpy arrays (a numpy array is
    returned).  A vector has ``dim`` entries in any shape; a ``(dim, k)``
    array is applied to every column (in one batched call when the operator
    provides ``matmat``, else column by column).  Anything else raises ``ValueError``
    before the library sees a pointer.  Like the reference's SciPy operators,
    the shape is ``(dim, dim)`` and ``dtype`` is complex, and
    ``scipy.sparse.linalg`` routines accept the object through
    ``aslinearoperator``.
    """

    def __init__(self, shape: tuple[int, int], matvec: Callable, rmatvec: Callable | None = None,
                 expectation: Callable | None = None, dtype=complex, matmat: Callable | None = None):
        self.shape = shape
        self.dtype = np.dtype(dtype)
        self._matvec = matvec
        self._rmatvec = rmatvec or matvec
        self._expectation = expectation
        # matmat(rows): the operator on every row of a contiguous (k, dim)
        # tensor in one call; also the adjoint's when rmatvec is matvec
        self._matmat = matmat
        self._rmatmat = matmat if rmatvec is None else None

    def _on_device(self, t: torch.Tensor) -> torch.Tensor:
        """The library's kernels read CUDA memory: a complex CUDA tensor."""
        if t.dtype not in (torch.complex64, torch.complex128):
            t = t.to(torch.complex128)
        return t.to("cuda")

    def _apply(self, fn, t: torch.Tensor, block_fn=None) -> torch.Tensor:
        n = self.shape[1]
        if t.dim() == 2 and t.shape[0] == n and t.shape[1] != 1:
            if block_fn is not None:
                return block_fn(self._on_device(t).transpose(0, 1).contiguous()).transpose(0, 1)
            return torch.stack([fn(self._on_device(t[:, k]).contiguous()) for k in range(t.shape[1])], dim=1)
        if t.numel() != n:
            raise ValueError(f"dimension mismatch: the operator is {self.shape}, the input has shape {tuple(t.shape)}")
        return fn(self._on_device(t).reshape(-1)).reshape(t.shape)

    def _run(self, fn, vec, block_fn=None):
        if isinstance(vec, torch.Tensor):
            return self._apply(fn, vec, block_fn).to(vec.device)
        arr = np.asarray(vec)
        if not np.iscomplexobj(arr):
            arr = arr.astype(np.complex128)
        return self._apply(fn, torch.from_numpy(np.ascontiguousarray(arr)), block_fn).cpu().numpy()

    def matvec(self, vec):
        return self._run(self._matvec, vec, self._matmat)

    def rmatvec(self, vec):
        return self._run(self._rmatvec, vec, self._rmatmat)

    def __matmul__(self, vec):
        return self.matvec(vec)

    def expectation(self, vec) -> float:
        """Real part of <vec|A|vec> in FP64 (fused when the operator supports it)."""
        t = vec if isinstance(vec, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(np.asarray(vec, dtype=complex)))
        if t.numel() != self.shape[1]:
            raise ValueError(f"dimension mismatch: the operator is {self.shape}, the input has shape {tuple(t.shape)}")
        v = self._on_device(t).reshape(-1).contiguous()
        if self._expectation is not None:
            return float(self._expectation(v))
        from ffsim_gb300.states import vdot

        return float(vdot(v, self._matvec(v)).real)
