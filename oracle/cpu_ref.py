"""Driver for the C restatement of the reference CPU path (oracle/cpu_ref.c).

TEST/BASELINE INFRASTRUCTURE ONLY: timed as the CPU baseline by bench.py
(``cpu_baseline`` and ``--impl reference``).  The orchestration follows the
reference Python drivers (python/ffsim/gates/orbital_rotation.py:117-199,
gates/diag_coulomb.py:156-220, contract/diag_coulomb.py:133-192,
hamiltonians/double_factorized_hamiltonian.py:244-275): per-Givens row-pair
sweeps over cached index tables, a contiguous transposed copy for the beta
sector, and the three-phase diagonal kernels, with OpenMP threads in place of
rayon.
"""

from __future__ import annotations

import ctypes
import math
import os
import subprocess
from pathlib import Path

import numpy as np

from oracle import ffsim_oracle as o

HERE = Path(__file__).resolve().parent
LIB = HERE / "libcpu_ref.so"
_lib = None

_zp = ctypes.c_void_p


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "libcpu_ref.so"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = ctypes.CDLL(str(LIB))
        L = _lib
        L.ref_givens_rows.argtypes = [_zp, ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      _zp, _zp, ctypes.c_long]
        L.ref_phase_rows.argtypes = [_zp, ctypes.c_long, ctypes.c_double, ctypes.c_double, _zp, ctypes.c_long]
        L.ref_diag_coulomb_num.argtypes = [_zp, ctypes.c_long, ctypes.c_long, ctypes.c_int, _zp, _zp, _zp,
                                           _zp, ctypes.c_int, _zp, ctypes.c_int]
        L.ref_contract_dc_num.argtypes = [_zp, _zp, ctypes.c_long, ctypes.c_long, ctypes.c_int, _zp, _zp, _zp,
                                          _zp, ctypes.c_int, _zp, ctypes.c_int]
        L.ref_num_op_sum_rows.argtypes = [_zp, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                          _zp, _zp, ctypes.c_int]
        L.ref_contract_nos_rows.argtypes = [_zp, _zp, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                                            ctypes.c_long, _zp, _zp, ctypes.c_int]
    return _lib


def threads() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


_tables: dict = {}


def _pairs(norb, nocc, i, j):
    key = ("p", norb, nocc, i, j)
    if key not in _tables:
        idx = np.ascontiguousarray(o.zero_one_subspace_indices(norb, nocc, (i, j)).astype(np.int64))
        _tables[key] = (idx[: len(idx) // 2].copy(), idx[len(idx) // 2 :].copy())
    return _tables[key]


def _ones(norb, nocc, i):
    key = ("o", norb, nocc, i)
    if key not in _tables:
        _tables[key] = np.ascontiguousarray(o.one_subspace_indices(norb, nocc, (i,)).astype(np.int64))
    return _tables[key]


def init_cache(norb, nelec):
    """Pre-build the index tables (python/ffsim/init_cache.py:25-41)."""
    for nocc in set(nelec):
        for i in range(norb - 1):
            _pairs(norb, nocc, i, i + 1)
            _pairs(norb, nocc, i + 1, i)
        for i in range(norb):
            _ones(norb, nocc, i)
        o.gen_occslst(norb, nocc)


def _rotate_rows(v2d, decomp, norb, nocc):
    L = lib()
    rots, phases = decomp
    dim_b = v2d.shape[1]
    for c, s, i, j in rots:
        s1, s2 = _pairs(norb, nocc, i, j)
        sc = complex(s).conjugate()
        L.ref_givens_rows(v2d.ctypes.data, dim_b, float(c), sc.real, sc.imag, s1.ctypes.data, s2.ctypes.data,
                          len(s1))
    for i, ph in enumerate(phases):
        rows = _ones(norb, nocc, i)
        L.ref_phase_rows(v2d.ctypes.data, dim_b, ph.real, ph.imag, rows.ctypes.data, len(rows))


def apply_orbital_rotation(vec, mat, norb, nelec):
    """orbital_rotation.py:117-154 with the C kernels (same matrix for both spins)."""
    na, nb = nelec
    decomp = o.givens_decomposition(mat)
    v = np.array(vec, dtype=complex).reshape(math.comb(norb, na), math.comb(norb, nb))
    _rotate_rows(v, decomp, norb, na)
    v = np.ascontiguousarray(v.T)
    _rotate_rows(v, decomp, norb, nb)
    return np.ascontiguousarray(v.T).reshape(-1)


def apply_diag_coulomb_evolution(vec, mat, time, norb, nelec):
    """diag_coulomb.py:156-220 (number representation, single matrix)."""
    na, nb = nelec
    eaa, eab, ebb = o.get_mat_exp(mat, time, norb, False)
    eaa, eab, ebb = (np.ascontiguousarray(x) for x in (eaa, eab, ebb))
    oa = np.ascontiguousarray(o.gen_occslst(norb, na).astype(np.int64))
    ob = np.ascontiguousarray(o.gen_occslst(norb, nb).astype(np.int64))
    v = np.array(vec, dtype=complex).reshape(len(oa), len(ob))
    lib().ref_diag_coulomb_num(v.ctypes.data, len(oa), len(ob), norb, eaa.ctypes.data, eab.ctypes.data,
                               ebb.ctypes.data, oa.ctypes.data, na, ob.ctypes.data, nb)
    return v.reshape(-1)


def contract_diag_coulomb(vec, mat, norb, nelec):
    na, nb = nelec
    aa, ab, bb = (np.ascontiguousarray(x) for x in o.get_mats(mat, norb, False))
    oa = np.ascontiguousarray(o.gen_occslst(norb, na).astype(np.int64))
    ob = np.ascontiguousarray(o.gen_occslst(norb, nb).astype(np.int64))
    v = np.ascontiguousarray(vec.reshape(len(oa), len(ob)))
    out = np.zeros_like(v)
    lib().ref_contract_dc_num(v.ctypes.data, out.ctypes.data, len(oa), len(ob), norb, aa.ctypes.data,
                              ab.ctypes.data, bb.ctypes.data, oa.ctypes.data, na, ob.ctypes.data, nb)
    return out.reshape(-1)


def df_term_matvec(vec, mat, rot, norb, nelec):
    """diag_coulomb_linop matvec (contract/diag_coulomb.py:245-268)."""
    v = apply_orbital_rotation(vec, rot.T.conj(), norb, nelec)
    v = contract_diag_coulomb(v, mat, norb, nelec)
    return apply_orbital_rotation(v, rot, norb, nelec)
