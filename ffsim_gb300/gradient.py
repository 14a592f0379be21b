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


def _dexp_adjoint(w: np.ndarray, W: np.ndarray, gam: np.ndarray) -> np.ndarray:
    """For a stack of antihermitian K = W diag(i w) W^dag ((B, n), (B, n, n))
    and gam (B, n, n): the matrices G with Re <dexp(K)[dK], gam> = Re <dK, G>
    for every dK (<X, Y> = sum_pq X_pq Y_pq), the adjoint of _dexp.  With
    dexp(K)[dK] = W ((W^dag dK W) o Phi) W^dag, G = conj(W) (Phi o (W^T gam
    conj(W))) W^T."""
    e = np.exp(1j * w)
    diff = 1j * (w[:, :, None] - w[:, None, :])
    with np.errstate(divide="ignore", invalid="ignore"):
        phi = (e[:, :, None] - e[:, None, :]) / diff
    close = np.abs(diff) < 1e-12
    phi[close] = np.broadcast_to(e[:, :, None], phi.shape)[close]
    Wc = W.conj()
    WT = np.swapaxes(W, -1, -2)
    return Wc @ (phi * (WT @ gam @ Wc)) @ WT


class GradientHost:
    """The host side of the adjoint gradient for one norb: the circuits of
    parameter rows (the merged rotations, the diagonal gates and the
    eigendecompositions the chain rule reuses) and the chain rule from a
    circuit's gate densities to its parameters.  The device part (forward
    circuit, Hamiltonian matvec, backward pass with densities) is
    LUCJGradient's (batch path) or the resident kernel's (small shapes)."""

    def __init__(self, norb: int):
        self.norb = norb
        self.basis = _antihermitian_basis(norb)
        # upper-triangle index pairs (i <= j) in the parameter order of from_parameters
        self._triu = tuple(np.array(v) for v in zip(*itertools.combinations_with_replacement(range(norb), 2)))

    def _circuits(self, params: np.ndarray, n_reps: int, with_final: bool) -> list:
        """The circuits of a batch of parameter rows (B, n_params), computed
        together: per state (U, Uf, V, jaa, jab, eig) with U[k] the layer
        rotations (U[0] = 1), V[j] the merged rotations V_j, the diagonal
        matrices of each layer and eig[k] = (w, W) with U[k] = W diag(e^{iw}) W^dag
        (the eigendecomposition the chain rule reuses).  Every step acts on each
        state on its own (stacked LAPACK and GEMM calls), so a state's circuit
        does not depend on the batch."""
        norb = self.norb
        L = n_reps
        P = np.atleast_2d(np.asarray(params, dtype=float))
        B = P.shape[0]
        n2 = norb * norb
        ti, tj = self._triu
        nt = len(ti)
        per = n2 + 2 * nt
        body = P[:, : L * per].reshape(B, L, per)
        K = antihermitians_from_parameters(body[:, :, :n2].reshape(-1), norb, B * L).reshape(B, L, norb, norb)
        mats = [K[:, k] for k in range(L)]
        if with_final:
            mats.append(antihermitians_from_parameters(P[:, L * per:].reshape(-1), norb, B))
        w, W = np.linalg.eigh(-1j * np.stack(mats, axis=1))  # (B, L(+1), n), (B, L(+1), n, n)
        Us = W @ (np.exp(1j * w)[..., None] * np.swapaxes(W, -1, -2).conj())
        J = np.zeros((B, L, 2, norb, norb))
        for t in range(2):
            vals = body[:, :, n2 + t * nt: n2 + (t + 1) * nt]
            J[:, :, t, tj, ti] = vals
            J[:, :, t, ti, tj] = vals
        eye = np.eye(norb, dtype=complex)
        out = []
        for b in range(B):
            U = [eye] + [Us[b, k] for k in range(L)]
            Uf = Us[b, L] if with_final else eye
            V = [None] + [U[k].conj().T @ U[k - 1] for k in range(1, L + 1)] + [Uf @ U[L]]
            jaa = [None] + [J[b, k, 0] for k in range(L)]
            jab = [None] + [J[b, k, 1] for k in range(L)]
            eig = [None] + [(w[b, k], W[b, k]) for k in range(w.shape[1])]
            out.append((U, Uf, V, jaa, jab, eig))
        return out

    def _circuit(self, params: np.ndarray, n_reps: int, with_final: bool):
        """The merged rotations V_j and diagonal matrices of one circuit."""
        return self._circuits(np.asarray(params, dtype=float)[None, :], n_reps, with_final)[0]

    def _chains(self, n_params: int, circuits: list, dens: list, L: int, with_final: bool) -> np.ndarray:
        """Chain rule from the generator gradients to the parameters, for a
        batch: circuits[b] from _circuits, dens[b] = (gamma, pdens) from
        _backward.  Returns (B, n_params).  Per state the same operations in
        the same order whatever the batch (stacked small GEMMs, a per-state
        projection onto the parameter basis)."""
        norb = self.norb
        B = len(circuits)
        grad = np.zeros((B, n_params))
        ti, tj = self._triu
        n_triu = len(ti)
        diag = ti == tj
        basis_t = self.basis.reshape(norb * norb, norb * norb).T
        index = 0

        def project(eigs, gam):
            # 2 Re <basis_n, G> for every rotation parameter n
            G = _dexp_adjoint(np.stack([e[0] for e in eigs]), np.stack([e[1] for e in eigs]), gam)
            flat = G.reshape(B, -1)
            return np.stack([2 * (flat[b] @ basis_t).real for b in range(B)])

        for k in range(1, L + 1):
            Ukm1 = np.stack([c[0][k - 1] for c in circuits])
            Uk = np.stack([c[0][k] for c in circuits])
            gk = np.stack([d[0][k] for d in dens])
            gk1 = np.stack([d[0][k + 1] for d in dens])
            # V_k = U_k^dag U_{k-1} is perturbed as A dU_k^dag C (A = U_{k-1}^dag U_k,
            # C = U_{k-1}) and V_{k+1} = U_{k+1}^dag U_k (or U_final U_L) as D dU_k
            # (D = U_k^dag); sum_pq (A X C)_pq g_pq = <X, A^T g C^T>, so both
            # contributions are 2 Re <dU_k, Gam> with one matrix Gam
            A = np.swapaxes(Ukm1, -1, -2).conj() @ Uk
            g1 = np.swapaxes(A, -1, -2) @ gk @ np.swapaxes(Ukm1, -1, -2)
            gam = np.swapaxes(g1, -1, -2).conj() + Uk.conj() @ gk1
            grad[:, index: index + norb * norb] = project([c[5][k] for c in circuits], gam)
            index += norb * norb
            P = np.stack([d[1][k] for d in dens])
            # same-spin: the pair (i, j) of both sectors, halved on the diagonal;
            # opposite-spin: both orders of (i, j), once on the diagonal
            daa = np.where(diag, 0.5, 1.0) * (P[:, 0, ti, tj] + P[:, 2, ti, tj])
            dab = np.where(diag, P[:, 1, ti, tj], P[:, 1, ti, tj] + P[:, 1, tj, ti])
            grad[:, index: index + n_triu] = -2 * daa.imag
            grad[:, index + n_triu: index + 2 * n_triu] = -2 * dab.imag
            index += 2 * n_triu
        if with_final:
            UL = np.stack([c[0][L] for c in circuits])
            Uf = np.stack([c[1] for c in circuits])
            gL = np.stack([d[0][L + 1] for d in dens])
            # V_{L+1} = U_final U_L perturbed as A dU_final C (A = U_L^dag U_final^dag, C = U_L)
            A = np.swapaxes(UL, -1, -2).conj() @ np.swapaxes(Uf, -1, -2).conj()
            gam = np.swapaxes(A, -1, -2) @ gL @ np.swapaxes(UL, -1, -2)
            grad[:, index:] = project([c[5][L + 1] for c in circuits], gam)
        return grad


class LUCJGradient(GradientHost):
    """Energy and gradient of the LUCJ ansatz for one (norb, nelec) shape,
    holding its device buffers (two states and scratch)."""

    def __init__(self, norb: int, nelec: tuple[int, int], *, dtype=torch.complex64, device="cuda",
                 workers: int = 4):
        GradientHost.__init__(self, norb)
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
        circ = self._circuit(params, n_reps, with_final_orbital_rotation)
        V, jaa, jab = circ[2], circ[3], circ[4]
        self._forward(self.cur, V, jaa, jab, L)
        ham, (one_body, hdcm, hrots) = self._ham_arrays(ham)
        _lib.call("ffgb_df_matvec", self.cur.data_ptr(), self.lam.data_ptr(), self.code, norb, na, nb,
                  _lib.dptr(one_body), hdcm.shape[0], _lib.dptr(hdcm), hrots.ctypes.data_as(_lib._dp),
                  0.0, 0, self._buf(), self.nbytes, self._stream())
        energy = float(ham.constant) + self._vdot(self.cur, self.lam)
        dens = self._backward(self.cur, self.lam, V, jaa, jab, L)
        return energy, self._chains(params.size, [circ], [dens], L, with_final_orbital_rotation)[0]

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
        circuits = self._circuits(params, n_reps, with_final_orbital_rotation)

        def forward(b):
            V, jaa, jab = circuits[b][2], circuits[b][3], circuits[b][4]
            self._forward(cur[b], V, jaa, jab, L)

        self._on_lanes(forward, B)
        ham, (one_body, hdcm, hrots) = self._ham_arrays(ham)
        _lib.call("ffgb_batch_df_matvec", cur.data_ptr(), lam.data_ptr(), B, self.code, norb, na, nb,
                  _lib.dptr(one_body), hdcm.shape[0], _lib.dptr(hdcm), hrots.ctypes.data_as(_lib._dp), 0.0, 0,
                  self._bbuf.data_ptr(), self._bbytes, None if control is None else control.ptr, self._stream())

        def backward(b):
            V, jaa, jab = circuits[b][2], circuits[b][3], circuits[b][4]
            e = float(ham.constant) + self._vdot(cur[b], lam[b])
            return e, self._backward(cur[b], lam[b], V, jaa, jab, L)

        out = self._on_lanes(backward, B)
        grads = self._chains(params.shape[1], circuits, [o[1] for o in out], L, with_final_orbital_rotation)
        return np.array([o[0] for o in out]), grads

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

        # every lane finishes enqueueing, and the current stream waits for
        # all of them, before an error from one lane is raised: no lane's
        # work on the batch buffers outlives the call
        futures = [self._pool.submit(lane, i) for i in range(min(W, n))]
        results = [None] * n
        err = None
        for fut in futures:
            try:
                for b, r in fut.result():
                    results[b] = r
            except BaseException as exc:  # noqa: BLE001
                err = err or exc
        for stream, _ in self._lanes:
            main.wait_stream(stream)
        if err is not None:
            raise err
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
