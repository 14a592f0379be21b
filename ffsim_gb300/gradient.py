"""Adjoint gradient of the LUCJ energy with respect to the parameters of a
spin-balanced UCJ operator (``UCJOpSpinBalanced.from_parameters`` layout).

With the UCJ rotations merged as in ``_apply_unitary_``
(python/ffsim/variational/ucj_spin_balanced.py:657-696 in the reference)::

    psi = W(V_{L+1}) D_L W(V_L) ... D_1 W(V_1) |HF>,
    V_1 = U_1^dag, V_k = U_k^dag U_{k-1}, V_{L+1} = U_final U_L,
    D_k = exp(i f_k),  f_k = sum_{i<=j} w_ij J^aa_ij (n_ia n_ja + n_ib n_jb) + sum_ij J^ab_ij n_ia n_jb

the energy E = <psi|H|psi> is differentiated by reverse accumulation: with
lambda = H psi, the gates are undone one by one on both psi and lambda (the
circuit is uncomputed, nothing is stored), and at each gate

* an orbital rotation W(V) perturbed as V exp(t G) contributes
  2 Re sum_pq G_pq <lambda| a+_p a_q |phi> (phi, lambda taken just below the
  gate): the transition one-body density, ffgb_transition_rdm1;
* a diagonal phase exp(i f) contributes -2 Im <lambda| df |phi>: the diagonal
  pair densities, ffgb_pair_density.

The generator gradients are mapped to the antihermitian parameters of each
U_k = exp(K_k) (python/ffsim/linalg/util.py:93-124) through the derivative of
the matrix exponential in the eigenbasis of K_k, in FP64 on the host.  The
states run in complex64 or complex128 on the GPU.  The reference has no
gradient; the result is checked against central finite differences of the
energy.
"""

from __future__ import annotations

import itertools
import threading
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from ffsim_gb300 import _lib
from ffsim_gb300._state import dim
from ffsim_gb300.hamiltonians import DoubleFactorizedHamiltonian
from ffsim_gb300.linalg import antihermitians_from_parameters
from ffsim_gb300.variational import UCJOpSpinBalanced


def _antihermitian_basis(norb: int) -> np.ndarray:
    """dK/dtheta for every one of the norb**2 rotation parameters."""
    eye = np.eye(norb * norb)
    return antihermitians_from_parameters(eye.reshape(-1), norb, norb * norb)


def _dexp(K: np.ndarray, dK: np.ndarray) -> np.ndarray:
    """d exp(K)[dK] for antihermitian K and a batch dK (n, norb, norb)."""
    w, W = np.linalg.eigh(-1j * K)  # K = W diag(i w) W^dag
    e = np.exp(1j * w)
    diff = 1j * (w[:, None] - w[None, :])
    with np.errstate(divide="ignore", invalid="ignore"):
        phi = (e[:, None] - e[None, :]) / diff
    close = np.abs(diff) < 1e-12
    phi[close] = np.broadcast_to(e[:, None], phi.shape)[close]
    Wd = W.conj().T
    M = Wd @ dK @ W
    return W @ (M * phi[None]) @ Wd


def _dexp_adjoint(K: np.ndarray, gam: np.ndarray) -> np.ndarray:
    """The matrix G with Re <dexp(K)[dK], gam> = Re <dK, G> for every dK
    (<X, Y> = sum_pq X_pq Y_pq): the adjoint of _dexp.  With K = W diag(i w)
    W^dag and dexp(K)[dK] = W ((W^dag dK W) o Phi) W^dag, G = conj(W)
    (Phi o (W^T gam conj(W))) W^T."""
    w, W = np.linalg.eigh(-1j * K)
    e = np.exp(1j * w)
    diff = 1j * (w[:, None] - w[None, :])
    with np.errstate(divide="ignore", invalid="ignore"):
        phi = (e[:, None] - e[None, :]) / diff
    close = np.abs(diff) < 1e-12
    phi[close] = np.broadcast_to(e[:, None], phi.shape)[close]
    Wc = W.conj()
    return Wc @ (phi * (W.T @ gam @ Wc)) @ W.T


class LUCJGradient:
    """Energy and gradient of the LUCJ ansatz for one (norb, nelec) shape,
    holding its device buffers (two states and scratch)."""

    def __init__(self, norb: int, nelec: tuple[int, int], *, dtype=torch.complex64, device="cuda",
                 workers: int = 4):
        self.norb = norb
        # batches: per-state gates run on `workers` host threads, each with its
        # own CUDA stream and scratch, so that their launches and host syncs
        # overlap; the Hamiltonian matvec runs once over the whole batch
        self.workers = max(1, int(workers))
        self._tls = threading.local()
        self._lanes = None
        self._pool = None
        self.nelec = tuple(nelec)
        self.dtype = dtype
        self.code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
        d = dim(norb, nelec)
        self.cur = torch.empty(d, dtype=dtype, device=device)
        self.lam = torch.empty(d, dtype=dtype, device=device)
        need = max(_lib.load().ffgb_scratch_bytes(op, self.code, norb, *self.nelec) for op in (0, 1, 3))
        self.buf = torch.empty(need, dtype=torch.uint8, device=device)
        self.nbytes = need
        self.basis = _antihermitian_basis(norb)
        # upper-triangle index pairs (i <= j) in the parameter order of from_parameters
        self._triu = tuple(np.array(v) for v in zip(*itertools.combinations_with_replacement(range(norb), 2)))

    # -- device helpers ----------------------------------------------------
    def _stream(self):
        return torch.cuda.current_stream(self.cur.device).cuda_stream

    def _buf(self) -> int:
        """Scratch of the calling thread (a batch lane's own, else the evaluator's)."""
        b = getattr(self._tls, "buf", None)
        return (self.buf if b is None else b).data_ptr()

    def _rotate(self, vec: torch.Tensor, mat: np.ndarray) -> None:
        m = _lib.cmat(mat)
        na, nb = self.nelec
        _lib.call("ffgb_apply_orbital_rotation", vec.data_ptr(), self.code, self.norb, na, nb, _lib.dptr(m),
                  _lib.dptr(m), self._buf(), self.nbytes, self._stream())

    def _phase(self, vec: torch.Tensor, jaa: np.ndarray, jab: np.ndarray, time: float) -> None:
        aa, ab = _lib.rmat(jaa), _lib.rmat(jab)
        na, nb = self.nelec
        _lib.call("ffgb_apply_diag_coulomb_evolution", vec.data_ptr(), self.code, self.norb, na, nb,
                  _lib.dptr(aa), _lib.dptr(ab), _lib.dptr(aa), float(time), 0, None, None, self._buf(),
                  self.nbytes, self._stream())

    def _density(self, name: str, x: torch.Tensor, y: torch.Tensor, blocks: int) -> np.ndarray:
        out = np.zeros(2 * blocks * self.norb * self.norb)
        na, nb = self.nelec
        _lib.call(name, x.data_ptr(), y.data_ptr(), self.code, self.norb, na, nb, _lib.dptr(out),
                  self._buf(), self.nbytes, self._stream())
        return out.view(np.complex128).reshape(blocks, self.norb, self.norb)

    # -- energy and gradient -------------------------------------------------
    def _circuit(self, params: np.ndarray, n_reps: int, with_final: bool):
        """The merged rotations V_j and diagonal matrices of the circuit."""
        norb = self.norb
        ucj = UCJOpSpinBalanced.from_parameters(params, norb=norb, n_reps=n_reps,
                                                with_final_orbital_rotation=with_final)
        L = n_reps
        U = [np.eye(norb, dtype=complex)] + [np.asarray(u) for u in ucj.orbital_rotations]
        Uf = (np.asarray(ucj.final_orbital_rotation) if ucj.final_orbital_rotation is not None
              else np.eye(norb, dtype=complex))
        V = [None] + [U[k].conj().T @ U[k - 1] for k in range(1, L + 1)] + [Uf @ U[L]]
        jaa = [None] + [ucj.diag_coulomb_mats[k, 0] for k in range(L)]
        jab = [None] + [ucj.diag_coulomb_mats[k, 1] for k in range(L)]
        return U, Uf, V, jaa, jab

    def _forward(self, cur: torch.Tensor, V, jaa, jab, L: int) -> None:
        """psi from the Hartree-Fock state."""
        _lib.call("ffgb_hartree_fock", cur.data_ptr(), self.code, cur.numel(), self._stream())
        for k in range(1, L + 1):
            self._rotate(cur, V[k])
            self._phase(cur, jaa[k], jab[k], -1.0)
        self._rotate(cur, V[L + 1])

    def _backward(self, cur: torch.Tensor, lam: torch.Tensor, V, jaa, jab, L: int):
        """Undo the gates on psi and lambda; generator gradients of the V_j and
        pair densities at the D_k.  Every gate's densities go to one device
        buffer (ffgb_gate_densities, no synchronization) that is read back
        once at the end."""
        norb = self.norb
        na, nb = self.nelec
        n2 = norb * norb
        dens = torch.empty((L + 2, 10 * n2), dtype=torch.float64, device=cur.device)
        for j in range(L + 1, 0, -1):
            vd = V[j].conj().T
            self._rotate(cur, vd)
            self._rotate(lam, vd)
            _lib.call("ffgb_gate_densities", lam.data_ptr(), cur.data_ptr(), self.code, norb, na, nb, int(j > 1),
                      dens[j].data_ptr(), self._buf(), self.nbytes, self._stream())
            if j > 1:
                k = j - 1
                self._phase(cur, jaa[k], jab[k], 1.0)
                self._phase(lam, jaa[k], jab[k], 1.0)
        h = dens.cpu().numpy()
        gamma = [None] * (L + 2)
        pdens = [None] * (L + 1)
        for j in range(1, L + 2):
            blk = h[j].view(np.complex128).reshape(5, norb, norb)
            gamma[j] = blk[0] + blk[1]
            if j > 1:
                pdens[j - 1] = blk[2:5].copy()
        return gamma, pdens

    def _chain(self, params: np.ndarray, U, Uf, gamma, pdens, L: int, with_final: bool) -> np.ndarray:
        """Chain rule from the generator gradients to the parameters."""
        norb = self.norb
        grad = np.zeros_like(params)
        ti, tj = self._triu
        n_triu = len(ti)
        diag = ti == tj
        index = 0
        for k in range(1, L + 1):
            Kk = antihermitians_from_parameters(params[index: index + norb * norb], norb, 1)[0]
            # V_k = U_k^dag U_{k-1} is perturbed as A dU_k^dag C (A = U_{k-1}^dag U_k,
            # C = U_{k-1}) and V_{k+1} = U_{k+1}^dag U_k (or U_final U_L) as D dU_k
            # (D = U_k^dag); sum_pq (A X C)_pq g_pq = <X, A^T g C^T>, so both
            # contributions are 2 Re <dU_k, Gam> with one matrix Gam
            A = U[k - 1].conj().T @ U[k]
            g1 = A.T @ gamma[k] @ U[k - 1].T
            gam = g1.conj().T + U[k].conj() @ gamma[k + 1]
            grad[index: index + norb * norb] = 2 * np.einsum(
                "nab,ab->n", self.basis, _dexp_adjoint(Kk, gam)).real
            index += norb * norb
            P = pdens[k]
            # same-spin: the pair (i, j) of both sectors, halved on the diagonal;
            # opposite-spin: both orders of (i, j), once on the diagonal
            daa = np.where(diag, 0.5, 1.0) * (P[0, ti, tj] + P[2, ti, tj])
            dab = np.where(diag, P[1, ti, tj], P[1, ti, tj] + P[1, tj, ti])
            grad[index: index + n_triu] = -2 * daa.imag
            grad[index + n_triu: index + 2 * n_triu] = -2 * dab.imag
            index += 2 * n_triu
        if with_final:
            Kf = antihermitians_from_parameters(params[index:], norb, 1)[0]
            # V_{L+1} = U_final U_L perturbed as A dU_final C (A = U_L^dag U_final^dag, C = U_L)
            A = U[L].conj().T @ Uf.conj().T
            gam = A.T @ gamma[L + 1] @ U[L].T
            grad[index:] = 2 * np.einsum("nab,ab->n", self.basis, _dexp_adjoint(Kf, gam)).real
        return grad

    def _vdot(self, x: torch.Tensor, y: torch.Tensor) -> float:
        e = np.zeros(2)
        _lib.call("ffgb_vdot", x.data_ptr(), y.data_ptr(), self.code, x.numel(), _lib.dptr(e), self._stream())
        return float(e[0])

    @staticmethod
    def _ham_arrays(ham: DoubleFactorizedHamiltonian):
        # lambda = (H - c) psi: the constant c changes neither the gradient (the
        # gates keep the norm) nor needs the states' precision, so it is added
        # to the energy exactly: E = c + <psi|lambda>
        if ham.z_representation:
            ham = ham.to_number_representation()
        return ham, ham._arrays()

    def value_and_grad(self, params: np.ndarray, n_reps: int, ham: DoubleFactorizedHamiltonian, *,
                       with_final_orbital_rotation: bool = False) -> tuple[float, np.ndarray]:
        norb = self.norb
        na, nb = self.nelec
        if ham.norb != norb:
            raise ValueError(f"the evaluator is for {norb} orbitals; got a Hamiltonian on {ham.norb}")
        params = np.asarray(params, dtype=float)
        L = n_reps
        U, Uf, V, jaa, jab = self._circuit(params, n_reps, with_final_orbital_rotation)
        self._forward(self.cur, V, jaa, jab, L)
        ham, (one_body, hdcm, hrots) = self._ham_arrays(ham)
        _lib.call("ffgb_df_matvec", self.cur.data_ptr(), self.lam.data_ptr(), self.code, norb, na, nb,
                  _lib.dptr(one_body), hdcm.shape[0], _lib.dptr(hdcm), hrots.ctypes.data_as(_lib._dp),
                  0.0, 0, self._buf(), self.nbytes, self._stream())
        energy = float(ham.constant) + self._vdot(self.cur, self.lam)
        gamma, pdens = self._backward(self.cur, self.lam, V, jaa, jab, L)
        return energy, self._chain(params, U, Uf, gamma, pdens, L, with_final_orbital_rotation)

    def value_and_grad_batch(self, params: np.ndarray, n_reps: int, ham: DoubleFactorizedHamiltonian, *,
                             with_final_orbital_rotation: bool = False,
                             control: _lib.Control | None = None) -> tuple[np.ndarray, np.ndarray]:
        """Energies and gradients of a batch of parameter vectors (rows of
        ``params``).  The Hamiltonian matvec -- every term's rotations and
        diagonal pass, most of the work -- runs once over all the states of
        the batch (ffgb_batch_df_matvec); the circuit's gates run per state.
        ``control`` (optional) can cancel the matvec from another thread or give
        it a deadline.  Returns (energies (batch,), gradients (batch, n_params))."""
        norb = self.norb
        na, nb = self.nelec
        if ham.norb != norb:
            raise ValueError(f"the evaluator is for {norb} orbitals; got a Hamiltonian on {ham.norb}")
        params = np.atleast_2d(np.asarray(params, dtype=float))
        B = params.shape[0]
        L = n_reps
        self._ensure_batch(B)
        cur, lam = self._bcur[:B], self._blam[:B]
        circuits = [self._circuit(p, n_reps, with_final_orbital_rotation) for p in params]

        def forward(b):
            _, _, V, jaa, jab = circuits[b]
            self._forward(cur[b], V, jaa, jab, L)

        self._on_lanes(forward, B)
        ham, (one_body, hdcm, hrots) = self._ham_arrays(ham)
        _lib.call("ffgb_batch_df_matvec", cur.data_ptr(), lam.data_ptr(), B, self.code, norb, na, nb,
                  _lib.dptr(one_body), hdcm.shape[0], _lib.dptr(hdcm), hrots.ctypes.data_as(_lib._dp), 0.0, 0,
                  self._bbuf.data_ptr(), self._bbytes, None if control is None else control.ptr, self._stream())

        def backward(b):
            U, Uf, V, jaa, jab = circuits[b]
            e = float(ham.constant) + self._vdot(cur[b], lam[b])
            gamma, pdens = self._backward(cur[b], lam[b], V, jaa, jab, L)
            return e, self._chain(params[b], U, Uf, gamma, pdens, L, with_final_orbital_rotation)

        out = self._on_lanes(backward, B)
        return np.array([o[0] for o in out]), np.stack([o[1] for o in out])

    def _on_lanes(self, fn, n: int) -> list:
        """fn(0), ..., fn(n - 1), spread over the worker lanes (state b on lane
        b mod workers, in order), each lane on its own stream after the work
        already queued on the current stream; the current stream then waits
        for every lane."""
        dev = self.cur.device
        main = torch.cuda.current_stream(dev)
        if self._lanes is None:
            self._lanes = [(torch.cuda.Stream(dev), torch.empty(self.nbytes, dtype=torch.uint8, device=dev))
                           for _ in range(self.workers)]
            self._pool = ThreadPoolExecutor(self.workers, thread_name_prefix="lucj-grad")
        W = len(self._lanes)

        def lane(i):
            stream, buf = self._lanes[i]
            self._tls.buf = buf
            stream.wait_stream(main)
            with torch.cuda.stream(stream):
                return [(b, fn(b)) for b in range(i, n, W)]

        results = [None] * n
        for part in self._pool.map(lane, range(min(W, n))):
            for b, r in part:
                results[b] = r
        for stream, _ in self._lanes:
            main.wait_stream(stream)
        return results

    def close(self) -> None:
        """Release the device buffers and the worker lanes now (instead of
        when the object is collected)."""
        if self._pool is not None:
            self._pool.shutdown(wait=True)
            self._pool = None
        self._lanes = None
        for name in ("_bcur", "_blam", "_bbuf"):
            if hasattr(self, name):
                delattr(self, name)
        self._bcap = 0
        self.cur = self.lam = self.buf = None

    def _ensure_batch(self, B: int) -> None:
        """Device buffers for B states (kept for later batches of at most B)."""
        if getattr(self, "_bcap", 0) >= B:
            return
        d = self.cur.numel()
        dev = self.cur.device
        self._bcur = torch.empty((B, d), dtype=self.dtype, device=dev)
        self._blam = torch.empty((B, d), dtype=self.dtype, device=dev)
        self._bbytes = _lib.load().ffgb_batch_scratch_bytes(1, self.code, self.norb, *self.nelec, B)
        self._bbuf = torch.empty(self._bbytes, dtype=torch.uint8, device=dev)
        self._bcap = B


class LUCJEnergyFunction(torch.autograd.Function):
    """E(params) with the adjoint gradient as its backward.  params: float64
    tensor of shape (n_params,) or (batch, n_params); returns E of shape () or
    (batch,)."""

    @staticmethod
    def forward(ctx, params, evaluator: LUCJGradient, n_reps: int, ham: DoubleFactorizedHamiltonian,
                with_final_orbital_rotation: bool = False):
        p = params.detach().cpu().numpy().astype(float)
        batch = p.reshape(-1, p.shape[-1])
        if batch.shape[0] > 1:
            es, gs = evaluator.value_and_grad_batch(batch, n_reps, ham,
                                                    with_final_orbital_rotation=with_final_orbital_rotation)
        else:
            e, g = evaluator.value_and_grad(batch[0], n_reps, ham,
                                            with_final_orbital_rotation=with_final_orbital_rotation)
            es, gs = [e], [g]
        grad = torch.as_tensor(np.array(gs).reshape(p.shape), dtype=params.dtype, device=params.device)
        ctx.save_for_backward(grad)
        out = torch.as_tensor(np.array(es), dtype=params.dtype, device=params.device)
        return out.reshape(p.shape[:-1])

    @staticmethod
    def backward(ctx, grad_out):
        (grad,) = ctx.saved_tensors
        return grad_out.unsqueeze(-1) * grad, None, None, None, None


def lucj_energy_autograd(params: torch.Tensor, evaluator: LUCJGradient, n_reps: int,
                         ham: DoubleFactorizedHamiltonian, *, with_final_orbital_rotation: bool = False):
    """LUCJ energy as a differentiable function of the parameter tensor."""
    return LUCJEnergyFunction.apply(params, evaluator, n_reps, ham, with_final_orbital_rotation)
