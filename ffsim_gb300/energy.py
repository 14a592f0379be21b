"""Fused LUCJ energy: the UCJ circuit applied to a state (Hartree-Fock by
default) followed by the double-factorized Hamiltonian expectation, with the
circuit's last orbital rotation merged into every Hamiltonian term.

Equals ``np.vdot(psi, H @ psi).real`` with ``psi = apply_unitary(hf, ucj)``
(tests/python/variational/ucj_spin_balanced_test.py:152-158 in the reference).
"""

from __future__ import annotations

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import dim, scratch
from ffsim_gb300.hamiltonians import DoubleFactorizedHamiltonian
from ffsim_gb300.variational import UCJOpSpinBalanced


class LUCJEnergy:
    """Reusable LUCJ energy evaluator holding its device buffers."""

    def __init__(self, norb: int, nelec: tuple[int, int], *, dtype=torch.complex64, device="cuda"):
        self.norb = norb
        self.nelec = tuple(nelec)
        self.dtype = dtype
        self.code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
        self.work = torch.empty(dim(norb, nelec), dtype=dtype, device=device)
        self.buf, self.nbytes = scratch(self.work, 2, norb, *self.nelec)
        self.stream = None

    def __call__(self, ucj: UCJOpSpinBalanced, ham: DoubleFactorizedHamiltonian, vec=None) -> float:
        n_alpha, n_beta = self.nelec
        norb = self.norb
        if ucj.norb != norb or ham.norb != norb:
            raise ValueError(f"the evaluator is for {norb} orbitals; got an operator on {ucj.norb} "
                             f"and a Hamiltonian on {ham.norb}")
        dcm = _lib.rmat(ucj.diag_coulomb_mats, (ucj.n_reps, 2, norb, norb), "diag_coulomb_mats")
        rots = _lib.cmat(ucj.orbital_rotations, (ucj.n_reps, norb, norb), "orbital_rotations")
        final = _lib.cmat(ucj.final_orbital_rotation, (norb, norb), "final_orbital_rotation")
        if ham.z_representation:
            ham = ham.to_number_representation()
        one_body, hdcm, hrots = ham._arrays()
        e = np.zeros(1)
        vin = None
        if vec is not None:
            vin = vec.contiguous()
            if vin.dtype != self.dtype:
                raise TypeError("vec dtype must match the evaluator dtype")
            if vin.device != self.work.device or vin.numel() != self.work.numel():
                raise ValueError(f"vec must be a tensor of {self.work.numel()} entries on {self.work.device}")
        stream = torch.cuda.current_stream(self.work.device).cuda_stream
        _lib.call("ffgb_lucj_energy", None if vin is None else vin.data_ptr(), self.work.data_ptr(),
                  self.code, self.norb, n_alpha, n_beta, ucj.n_reps, _lib.dptr(dcm),
                  rots.ctypes.data_as(_lib._dp), _lib.dptr(final), _lib.dptr(one_body), hdcm.shape[0],
                  _lib.dptr(hdcm), hrots.ctypes.data_as(_lib._dp), float(ham.constant), _lib.dptr(e),
                  self.buf.data_ptr(), self.nbytes, stream)
        return float(e[0])


def lucj_energy(ucj: UCJOpSpinBalanced, ham: DoubleFactorizedHamiltonian, norb: int,
                nelec: tuple[int, int], *, dtype=torch.complex64, vec=None) -> float:
    """One LUCJ energy evaluation (allocates its buffers; use LUCJEnergy to reuse them)."""
    return LUCJEnergy(norb, nelec, dtype=dtype)(ucj, ham, vec)


class BatchLUCJEnergy:
    """LUCJ energies of many parameter sets of one shape under one
    double-factorized Hamiltonian (``ffgb_batch_lucj_energy``): each UCJ
    circuit runs on its own state, then every Hamiltonian term runs once over
    all the states.  Holds device buffers for up to ``max_states`` states.

    Per state the energy equals ``LUCJEnergy`` to rounding; the reference
    evaluates such energies one parameter vector at a time
    (python/ffsim/optimize/linear_method.py:181-243).
    """

    def __init__(self, norb: int, nelec: tuple[int, int], max_states: int, *, dtype=torch.complex64,
                 device="cuda"):
        if max_states < 1:
            raise ValueError("max_states must be positive")
        self.norb = norb
        self.nelec = tuple(nelec)
        self.dtype = dtype
        self.max_states = max_states
        self.code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
        self.work = torch.empty((max_states, dim(norb, nelec)), dtype=dtype, device=device)
        self.nbytes = _lib.load().ffgb_batch_scratch_bytes(0, self.code, norb, *self.nelec, max_states)
        self.buf = torch.empty(self.nbytes, dtype=torch.uint8, device=device)

    def close(self) -> None:
        """Release the device buffers now."""
        self.work = self.buf = None

    def __call__(self, ucjs: list[UCJOpSpinBalanced], ham: DoubleFactorizedHamiltonian,
                 control: _lib.Control | None = None) -> np.ndarray:
        """Energies of the operators; ``control`` (optional) can cancel the
        batch from another thread or give it a deadline (CancelledError /
        TimeoutError, checked between states and Hamiltonian terms)."""
        n = len(ucjs)
        norb = self.norb
        if not 1 <= n <= self.max_states:
            raise ValueError(f"between 1 and {self.max_states} operators are accepted, got {n}")
        n_reps = ucjs[0].n_reps
        for u in ucjs:
            if u.norb != norb or u.n_reps != n_reps:
                raise ValueError("every operator of a batch must have the evaluator's norb and the same n_reps")
        if ham.norb != norb:
            raise ValueError(f"the evaluator is for {norb} orbitals; got a Hamiltonian on {ham.norb}")
        dcm = np.ascontiguousarray(np.stack([_lib.rmat(u.diag_coulomb_mats, (n_reps, 2, norb, norb),
                                                       "diag_coulomb_mats") for u in ucjs]))
        rots = np.ascontiguousarray(np.stack([_lib.cmat(u.orbital_rotations, (n_reps, norb, norb),
                                                        "orbital_rotations") for u in ucjs]))
        final = None
        if any(u.final_orbital_rotation is not None for u in ucjs):
            eye = np.eye(norb, dtype=complex)
            final = np.ascontiguousarray(np.stack([
                _lib.cmat(u.final_orbital_rotation if u.final_orbital_rotation is not None else eye,
                          (norb, norb), "final_orbital_rotation") for u in ucjs]))
        if ham.z_representation:
            ham = ham.to_number_representation()
        one_body, hdcm, hrots = ham._arrays()
        e = np.zeros(n)
        stream = torch.cuda.current_stream(self.work.device).cuda_stream
        _lib.call("ffgb_batch_lucj_energy", self.work.data_ptr(), n, self.code, norb, *self.nelec, n_reps,
                  _lib.dptr(dcm), rots.ctypes.data_as(_lib._dp), None if final is None else final.ctypes.data_as(_lib._dp),
                  _lib.dptr(one_body), hdcm.shape[0], _lib.dptr(hdcm), hrots.ctypes.data_as(_lib._dp),
                  float(ham.constant), _lib.dptr(e), self.buf.data_ptr(), self.nbytes,
                  None if control is None else control.ptr, stream)
        return e


def lucj_energies(ucjs: list[UCJOpSpinBalanced], ham: DoubleFactorizedHamiltonian, norb: int,
                  nelec: tuple[int, int], *, dtype=torch.complex64) -> np.ndarray:
    """Energies of several UCJ operators under one Hamiltonian in one batch."""
    return BatchLUCJEnergy(norb, nelec, len(ucjs), dtype=dtype)(ucjs, ham)
