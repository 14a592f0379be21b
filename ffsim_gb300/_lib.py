"""ctypes binding of the C ABI in ``include/ffsim_gb300.h`` (``libffgb.so``).

The library is built in-tree by ``ffsim_gb300._build.build()``.  There is no
fallback: if the shared library is missing or cannot be loaded, every entry
point raises ``ImportError``.
"""

from __future__ import annotations

import ctypes
import threading
from concurrent.futures import CancelledError
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libffgb.so"

FFGB_C64 = 0
FFGB_C128 = 1

_ERRORS = {
    1: ValueError,
    2: TypeError,
    3: MemoryError,
    4: RuntimeError,
    5: TimeoutError,
    6: NotImplementedError,
    7: ArithmeticError,
    8: CancelledError,
}

_c_void_p = ctypes.c_void_p
_c_int = ctypes.c_int
_c_double = ctypes.c_double
_c_size_t = ctypes.c_size_t
_c_ll = ctypes.c_longlong
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

# name -> argtypes (all return int status except where noted)
SIGNATURES = {
    "ffgb_version": [],
    "ffgb_last_error": [],
    "ffgb_launch_count": [],
    "ffgb_device_alloc_count": [],
    "ffgb_debug_fma_rate": [_c_int, _dp, _c_void_p],
    "ffgb_givens_decomposition": [_dp, _c_int, _c_double, _dp, _ip, _ip, _dp],
    "ffgb_eigh": [_dp, _c_int, _dp, _dp],
    "ffgb_debug_plan": [_dp, _c_int, _c_int, _dp, _c_int, _ip],
    "ffgb_debug_stage": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _c_int, _c_void_p],
    "ffgb_scratch_bytes": [_c_int, _c_int, _c_int, _c_int, _c_int],
    "ffgb_apply_givens_rotation": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_double,
                                   _c_double, _c_double, _c_int, _c_int, _c_void_p],
    "ffgb_apply_phase_shift": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_double,
                               _c_double, _c_int, _c_void_p],
    "ffgb_apply_excitation": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _c_int,
                              _c_void_p],
    "ffgb_apply_orbital_rotation": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _dp, _c_void_p,
                                    _c_size_t, _c_void_p],
    "ffgb_apply_diag_coulomb_evolution": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _dp, _dp,
                                          _c_double, _c_int, _dp, _dp, _c_void_p, _c_size_t,
                                          _c_void_p],
    "ffgb_apply_num_op_sum_evolution": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _dp,
                                        _c_double, _dp, _dp, _c_void_p, _c_size_t, _c_void_p],
    "ffgb_ucj_spin_balanced_apply": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _dp, _dp,
                                     _dp, _c_void_p, _c_size_t, _c_void_p],
    "ffgb_contract_diag_coulomb": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _dp,
                                   _dp, _c_int, _c_int, _c_void_p],
    "ffgb_contract_diag_coulomb_static": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp,
                                          _dp, _dp, _c_int, _c_int, _c_void_p],
    "ffgb_contract_num_op_sum": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _c_int,
                                 _c_void_p],
    "ffgb_rotated_diag_matvec": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _dp,
                                 _c_int, _dp, _c_int, _c_void_p, _c_size_t, _c_void_p],
    "ffgb_df_matvec": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _c_int, _dp, _dp,
                       _c_double, _c_int, _c_void_p, _c_size_t, _c_void_p],
    "ffgb_df_expectation": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _c_int, _dp, _dp,
                            _c_double, _c_int, _dp, _dp, _c_void_p, _c_size_t, _c_void_p],
    "ffgb_lucj_energy": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _dp, _dp, _dp,
                         _dp, _c_int, _dp, _dp, _c_double, _dp, _c_void_p, _c_size_t, _c_void_p],
    "ffgb_batch_scratch_bytes": [_c_int, _c_int, _c_int, _c_int, _c_int, _c_ll],
    "ffgb_batch_lucj_energy": [_c_void_p, _c_ll, _c_int, _c_int, _c_int, _c_int, _c_int, _dp, _dp, _dp, _dp, _c_int,
                               _dp, _dp, _c_double, _dp, _c_void_p, _c_size_t, _c_void_p, _c_void_p],
    "ffgb_batch_df_matvec": [_c_void_p, _c_void_p, _c_ll, _c_int, _c_int, _c_int, _c_int, _dp, _c_int, _dp, _dp,
                             _c_double, _c_int, _c_void_p, _c_size_t, _c_void_p, _c_void_p],
    "ffgb_transition_rdm1": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _c_void_p, _c_size_t,
                             _c_void_p],
    "ffgb_pair_density": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _dp, _c_void_p, _c_size_t,
                          _c_void_p],
    "ffgb_gate_densities": [_c_void_p, _c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _c_void_p, _c_void_p,
                            _c_size_t, _c_void_p],
    "ffgb_vdot": [_c_void_p, _c_void_p, _c_int, _c_ll, _dp, _c_void_p],
    "ffgb_hartree_fock": [_c_void_p, _c_int, _c_ll, _c_void_p],
    "ffgb_resident_open": [_c_int, _c_int, _c_double, ctypes.POINTER(_c_void_p)],
    "ffgb_resident_hamiltonian": [_c_void_p, _c_int, _dp, _c_int, _dp, _dp, _c_double, _c_int, _ip],
    "ffgb_resident_submit": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _dp, _dp, _dp,
                             ctypes.POINTER(_c_ll)],
    "ffgb_resident_poll": [_c_void_p, _c_ll, _dp],
    "ffgb_resident_submit_grad": [_c_void_p, _c_int, _c_int, _c_int, _c_int, _c_int, _dp, _dp,
                                  ctypes.POINTER(_c_ll)],
    "ffgb_resident_poll_densities": [_c_void_p, _c_ll, _dp, _dp],
    "ffgb_resident_cancel": [_c_void_p, _c_ll],
    "ffgb_resident_start": [_c_void_p],
    "ffgb_resident_status": [_c_void_p, _ip, _ip],
    "ffgb_resident_close": [_c_void_p],
}

FFGB_PENDING = 9

class Control(ctypes.Structure):
    """``ffgb_control`` of a batch call: a cancellation flag that another
    thread sets with ``request_cancel()`` and a deadline in seconds (<= 0:
    none).  Pass ``control.ptr``."""

    _fields_ = [("cancel", ctypes.POINTER(ctypes.c_int)), ("timeout_s", ctypes.c_double)]

    def __init__(self, timeout_s: float = 0.0):
        super().__init__()
        self._flag = ctypes.c_int(0)
        self.cancel = ctypes.pointer(self._flag)
        self.timeout_s = float(timeout_s)

    def request_cancel(self) -> None:
        self._flag.value = 1

    @property
    def ptr(self):
        return ctypes.byref(self)


_lock = threading.Lock()
_lib = None


def load() -> ctypes.CDLL:
    """Load libffgb.so (raises ImportError if it has not been built)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing; build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(ffsim_gb300 has no CPU fallback)"
            )
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _c_int
        lib.ffgb_last_error.restype = ctypes.c_char_p
        lib.ffgb_scratch_bytes.restype = _c_size_t
        lib.ffgb_batch_scratch_bytes.restype = _c_size_t
        lib.ffgb_launch_count.restype = _c_ll
        lib.ffgb_device_alloc_count.restype = _c_ll
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != 0:
        msg = load().ffgb_last_error().decode(errors="replace")
        raise _ERRORS.get(status, RuntimeError)(msg or f"ffgb status {status}")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def dptr(arr: np.ndarray | None):
    """Pointer to the data of a contiguous float64/complex128 numpy array (or NULL)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(_dp)


def _checked(arr: np.ndarray, shape, what: str) -> np.ndarray:
    """The library reads exactly ``shape`` elements through the pointer, so a
    mis-sized array is rejected here instead of read past its end."""
    if shape is not None and arr.shape != tuple(shape):
        raise ValueError(f"{what} must have shape {tuple(shape)}, got {arr.shape}")
    return arr


def cmat(mat, shape=None, what: str = "matrix") -> np.ndarray | None:
    """Contiguous complex128 copy of ``mat`` (None stays None), optionally shape-checked."""
    if mat is None:
        return None
    return _checked(np.ascontiguousarray(np.asarray(mat, dtype=np.complex128)), shape, what)


def rmat(mat, shape=None, what: str = "matrix") -> np.ndarray | None:
    """Contiguous float64 copy of ``mat`` (None stays None), optionally shape-checked."""
    if mat is None:
        return None
    return _checked(np.ascontiguousarray(np.asarray(mat, dtype=np.float64)), shape, what)
