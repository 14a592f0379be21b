"""Resident evaluator: LUCJ energies and gradients of small shapes served by a persistent kernel.

``ResidentEvaluator`` wraps the ``ffgb_resident_*`` entry points.  One
persistent kernel takes requests from a queue in host-mapped memory; each of
its CTAs evaluates one request at a time end to end -- the spin-balanced UCJ
circuit from Hartree-Fock, then every term of the request's
double-factorized Hamiltonian -- with the state (norb <= 8: at most 4,900
complex64 amplitudes) in shared memory, and writes the FP64 energy back to the
request's slot.  Requests of different shapes and Hamiltonians share the
queue.  The batch path (``BatchLUCJEnergy``) launches a few hundred kernels
per evaluation, which at these sizes costs more than the arithmetic.

The kernel's wait for work is bounded: after ``idle_seconds`` without a
request its CTAs exit and ``status()`` reports ``FFGB_ERR_TIMEOUT`` (the wait
ran out); the next ``submit`` launches it again.  ``cancel`` stops a request
between gates.  Equals ``np.vdot(psi, H @ psi).real`` with ``psi =
apply_unitary(hf, ucj)`` (tests/python/variational/ucj_spin_balanced_test.py:152-158
in the reference).
"""

from __future__ import annotations

import ctypes
import time
from concurrent.futures import CancelledError

import numpy as np

from ffsim_gb300 import _lib
from ffsim_gb300.hamiltonians import DoubleFactorizedHamiltonian
from ffsim_gb300.variational import UCJOpSpinBalanced

MAX_NORB = 8
MAX_REPS = 4


def accepts(norb: int, n_reps: int) -> bool:
    """Whether the resident kernel takes requests of this shape."""
    return 1 <= norb <= MAX_NORB and 1 <= n_reps <= MAX_REPS


class ResidentEvaluator:
    """Queue of ``n_slots`` requests served by ``n_ctas`` CTAs (one request
    per CTA at a time) on the current CUDA device."""

    def __init__(self, n_slots: int = 256, n_ctas: int = 8, idle_seconds: float = 1.0):
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.ffgb_resident_open(int(n_slots), int(n_ctas), float(idle_seconds), ctypes.byref(h)))
        self._h = h
        self._hams: dict[int, tuple[int, object]] = {}  # id(ham) -> (ham_id, ham kept alive)
        self._grad_hosts: dict = {}  # norb -> GradientHost
        self._grad_jobs: dict = {}  # ticket -> what the chain rule needs at collection

    def _ham_id(self, ham: DoubleFactorizedHamiltonian) -> int:
        got = self._hams.get(id(ham))
        if got is not None:
            return got[0]
        h = ham.to_number_representation() if ham.z_representation else ham
        one_body, dcm, rots = h._arrays()
        hid = ctypes.c_int(-1)
        _lib.call("ffgb_resident_hamiltonian", self._h, h.norb, _lib.dptr(one_body), dcm.shape[0], _lib.dptr(dcm),
                  rots.ctypes.data_as(_lib._dp), float(h.constant), 0, ctypes.byref(hid))
        self._hams[id(ham)] = (hid.value, ham)
        return hid.value

    def submit(self, ucj: UCJOpSpinBalanced, ham: DoubleFactorizedHamiltonian, nelec: tuple[int, int]) -> int:
        """Queue the energy of ``ucj`` applied to Hartree-Fock under ``ham``;
        returns the request's ticket (MemoryError when the queue is full of
        uncollected results)."""
        norb = ucj.norb
        if ham.norb != norb:
            raise ValueError(f"the operator acts on {norb} orbitals, the Hamiltonian on {ham.norb}")
        if not accepts(norb, ucj.n_reps):
            raise NotImplementedError(f"the resident kernel takes norb <= {MAX_NORB} and n_reps <= {MAX_REPS}")
        dcm = _lib.rmat(ucj.diag_coulomb_mats, (ucj.n_reps, 2, norb, norb), "diag_coulomb_mats")
        rots = _lib.cmat(ucj.orbital_rotations, (ucj.n_reps, norb, norb), "orbital_rotations")
        final = _lib.cmat(ucj.final_orbital_rotation, (norb, norb), "final_orbital_rotation")
        ticket = ctypes.c_longlong(-1)
        _lib.call("ffgb_resident_submit", self._h, self._ham_id(ham), norb, int(nelec[0]), int(nelec[1]),
                  ucj.n_reps, _lib.dptr(dcm), rots.ctypes.data_as(_lib._dp), _lib.dptr(final),
                  ctypes.byref(ticket))
        return ticket.value

    def poll(self, ticket: int) -> float | None:
        """The energy once the request has finished (its slot is then free),
        None while it runs; CancelledError if it was cancelled."""
        e = ctypes.c_double(0.0)
        status = _lib.load().ffgb_resident_poll(self._h, int(ticket), ctypes.byref(e))
        if status == _lib.FFGB_PENDING:
            return None
        _lib.check(status)
        return e.value

    def wait(self, ticket: int, timeout: float = 60.0) -> float:
        """Poll until the request finishes (TimeoutError after ``timeout`` s)."""
        deadline = time.perf_counter() + timeout
        while True:
            e = self.poll(ticket)
            if e is not None:
                return e
            if time.perf_counter() > deadline:
                raise TimeoutError(f"resident request {ticket} did not finish within {timeout} s")
            time.sleep(20e-6)

    def energies(self, ucjs: list[UCJOpSpinBalanced], ham: DoubleFactorizedHamiltonian, nelec: tuple[int, int],
                 timeout: float = 60.0) -> np.ndarray:
        """Submit every operator, then wait for all the energies."""
        tickets = [self.submit(u, ham, nelec) for u in ucjs]
        return np.array([self.wait(t, timeout) for t in tickets])

    # -- gradients -----------------------------------------------------------
    def _host(self, norb: int):
        from ffsim_gb300.gradient import GradientHost

        h = self._grad_hosts.get(norb)
        if h is None:
            h = self._grad_hosts[norb] = GradientHost(norb)
        return h

    def submit_grad(self, params: np.ndarray, n_reps: int, ham: DoubleFactorizedHamiltonian,
                    nelec: tuple[int, int], *, with_final_orbital_rotation: bool = False) -> int:
        """Queue the energy and adjoint gradient of the spin-balanced UCJ
        operator with these parameters (the ``from_parameters`` layout) under
        ``ham``; collect with ``poll_grad``.  The kernel runs the circuit, the
        Hamiltonian matvec and the backward pass with its densities; the chain
        rule to the parameters runs on the host at collection."""
        norb = ham.norb
        if not accepts(norb, n_reps):
            raise NotImplementedError(f"the resident kernel takes norb <= {MAX_NORB} and n_reps <= {MAX_REPS}")
        params = np.asarray(params, dtype=float)
        n = UCJOpSpinBalanced.n_params(norb, n_reps, with_final_orbital_rotation=with_final_orbital_rotation)
        if params.shape != (n,):
            raise ValueError(f"expected {n} parameters, got shape {params.shape}")
        circ = self._host(norb)._circuits(params[None, :], n_reps, with_final_orbital_rotation)[0]
        V = np.ascontiguousarray(np.stack(circ[2][1:]), dtype=np.complex128)
        J = np.ascontiguousarray(np.stack([np.stack([circ[3][k], circ[4][k]]) for k in range(1, n_reps + 1)]),
                                 dtype=np.float64)
        ticket = ctypes.c_longlong(-1)
        _lib.call("ffgb_resident_submit_grad", self._h, self._ham_id(ham), norb, int(nelec[0]), int(nelec[1]),
                  n_reps, V.ctypes.data_as(_lib._dp), _lib.dptr(J), ctypes.byref(ticket))
        self._grad_jobs[ticket.value] = (n, n_reps, with_final_orbital_rotation, circ, norb)
        return ticket.value

    def poll_grad(self, ticket: int) -> tuple[float, np.ndarray] | None:
        """(energy, gradient) once the gradient request has finished, None
        while it runs; CancelledError if it was cancelled."""
        n, L, with_final, circ, norb = self._grad_jobs[ticket]
        e = ctypes.c_double(0.0)
        dens = np.zeros(2 * (L + 1) * 5 * norb * norb)
        status = _lib.load().ffgb_resident_poll_densities(self._h, int(ticket), ctypes.byref(e), _lib.dptr(dens))
        if status == _lib.FFGB_PENDING:
            return None
        del self._grad_jobs[ticket]
        _lib.check(status)
        blocks = dens.view(np.complex128).reshape(L + 1, 5, norb, norb)
        gamma = [None] + [blocks[j - 1, 0] + blocks[j - 1, 1] for j in range(1, L + 2)]
        pdens = [None] + [blocks[j, 2:5].copy() for j in range(1, L + 1)]
        grad = self._host(norb)._chains(n, [circ], [(gamma, pdens)], L, with_final)[0]
        return e.value, grad

    def wait_grad(self, ticket: int, timeout: float = 60.0) -> tuple[float, np.ndarray]:
        deadline = time.perf_counter() + timeout
        while True:
            got = self.poll_grad(ticket)
            if got is not None:
                return got
            if time.perf_counter() > deadline:
                raise TimeoutError(f"resident request {ticket} did not finish within {timeout} s")
            time.sleep(20e-6)

    def cancel(self, ticket: int) -> None:
        _lib.call("ffgb_resident_cancel", self._h, int(ticket))

    def start(self) -> None:
        """Launch the kernel now if it is not running."""
        _lib.call("ffgb_resident_start", self._h)

    def status(self) -> tuple[bool, int]:
        """(running, kernel status): FFGB_ERR_TIMEOUT (5) once the kernel has
        exited because no request came within its idle limit."""
        running, st = ctypes.c_int(0), ctypes.c_int(0)
        _lib.call("ffgb_resident_status", self._h, ctypes.byref(running), ctypes.byref(st))
        return bool(running.value), st.value

    def close(self) -> None:
        """Stop the kernel and free the queue (uncollected results are lost)."""
        if self._h is not None:
            h, self._h = self._h, None
            _lib.call("ffgb_resident_close", h)

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


__all__ = ["ResidentEvaluator", "accepts", "CancelledError"]
