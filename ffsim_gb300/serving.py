"""Serving loop for LUCJ energy and gradient requests of mixed shapes.

Continuous batching on one GPU: every worker thread owns a CUDA stream and
takes the oldest pending request that it can admit -- a free worker, and
device buffers for the request's shape either idle in the pool or allocatable
within the HBM budget.  Requests that arrive while others run are admitted as
workers and memory free up, so their kernels overlap on the device with the
ones already running.  Device buffers (states and scratch) stay resident in a
per-shape pool and are reused by later requests of the same shape; idle
buffers of other shapes are released when a new shape needs their memory.

The library calls release the Python interpreter lock while they run (ctypes
foreign calls), so the workers' host orchestration proceeds in parallel.
Results do not depend on what else runs: every kernel's reductions have a
fixed order and the coefficient dithering depends only on the request.
"""

from __future__ import annotations

import collections
import dataclasses
import statistics
import threading
import time
from typing import Callable

import numpy as np


@dataclasses.dataclass
class Request:
    """One evaluation: kind is "energy" or "gradient"; params in the
    ``UCJOpSpinBalanced.from_parameters`` layout for (norb, n_reps)."""

    rid: int
    kind: str
    norb: int
    nelec: tuple[int, int]
    n_reps: int
    params: np.ndarray
    ham: object
    arrival: float = 0.0


@dataclasses.dataclass
class Result:
    rid: int
    energy: float
    grad: np.ndarray | None
    arrival: float
    start: float
    end: float

    @property
    def latency(self) -> float:
        return self.end - self.arrival


class _Evaluator:
    """Device buffers of one (kind, shape) and the call that uses them."""

    def __init__(self, kind: str, norb: int, nelec: tuple[int, int], dtype):
        import torch

        from ffsim_gb300.energy import LUCJEnergy
        from ffsim_gb300.gradient import LUCJGradient

        self.key = (kind, norb, tuple(nelec))
        if kind == "energy":
            self.impl = LUCJEnergy(norb, nelec, dtype=dtype)
            self.nbytes = self.impl.work.numel() * self.impl.work.element_size() + self.impl.nbytes
        else:
            self.impl = LUCJGradient(norb, nelec, dtype=dtype)
            self.nbytes = 2 * self.impl.cur.numel() * self.impl.cur.element_size() + self.impl.nbytes
        self._torch = torch

    def run(self, req: Request) -> tuple[float, np.ndarray | None]:
        from ffsim_gb300.variational import UCJOpSpinBalanced

        if req.kind == "energy":
            op = UCJOpSpinBalanced.from_parameters(req.params, norb=req.norb, n_reps=req.n_reps)
            return self.impl(op, req.ham), None
        return self.impl.value_and_grad(req.params, req.n_reps, req.ham)


def evaluator_bytes(kind: str, norb: int, nelec: tuple[int, int], dtype) -> int:
    """Device bytes an evaluator of this shape holds (states + scratch)."""
    import torch

    from ffsim_gb300 import _lib
    from ffsim_gb300._state import dim

    code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
    el = 8 if dtype == torch.complex64 else 16
    lib = _lib.load()
    d = dim(norb, nelec)
    if kind == "energy":
        return d * el + lib.ffgb_scratch_bytes(2, code, norb, *nelec)
    return 2 * d * el + max(lib.ffgb_scratch_bytes(op, code, norb, *nelec) for op in (0, 1, 3))


class LUCJServer:
    """Continuous-batching server.

    workers: concurrent requests (one CUDA stream each).
    budget_bytes: device memory the pooled buffers may hold (default: 85% of
    the free HBM when the server starts).
    make_evaluator / size_of: injection points (the defaults build the GPU
    evaluators); tests substitute host-only fakes.
    """

    def __init__(self, workers: int = 6, *, dtype=None, budget_bytes: int | None = None,
                 make_evaluator: Callable | None = None, size_of: Callable | None = None,
                 use_streams: bool = True):
        import torch

        self.dtype = dtype if dtype is not None else torch.complex64
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            budget_bytes = int(0.85 * free)
        self.budget = int(budget_bytes)
        self.make_evaluator = make_evaluator or (lambda k, n, ne: _Evaluator(k, n, ne, self.dtype))
        self.size_of = size_of or (lambda k, n, ne: evaluator_bytes(k, n, ne, self.dtype))
        self.use_streams = use_streams
        self._cv = threading.Condition()
        self._pending: collections.deque[Request] = collections.deque()
        self._idle: dict[tuple, list] = collections.defaultdict(list)
        self._idle_order: collections.OrderedDict = collections.OrderedDict()  # id -> (key, ev), LRU
        self._in_use = 0  # bytes held by pooled + running evaluators
        self._results: list[Result] = []
        self._errors: list[BaseException] = []
        self._stop = False
        self.max_concurrent = 0
        self._running = 0
        self._threads = [threading.Thread(target=self._worker, args=(i,), daemon=True) for i in range(workers)]
        for t in self._threads:
            t.start()

    # -- client side -------------------------------------------------------
    def submit(self, req: Request) -> None:
        with self._cv:
            if not req.arrival:
                req.arrival = time.perf_counter()
            self._pending.append(req)
            self._cv.notify_all()

    def drain(self, n_expected: int, timeout: float = 3600.0) -> list[Result]:
        """Wait until n_expected results exist; returns them sorted by rid."""
        deadline = time.perf_counter() + timeout
        with self._cv:
            while len(self._results) + len(self._errors) < n_expected:
                left = deadline - time.perf_counter()
                if left <= 0:
                    raise TimeoutError(f"{len(self._results)} of {n_expected} requests finished")
                self._cv.wait(timeout=min(left, 1.0))
            if self._errors:
                raise self._errors[0]
            return sorted(self._results, key=lambda r: r.rid)

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join(timeout=60)

    # -- scheduling -----------------------------------------------------------
    def _take(self):
        """Under the lock: the oldest admissible request with its evaluator."""
        for i, req in enumerate(self._pending):
            key = (req.kind, req.norb, tuple(req.nelec))
            if self._idle[key]:
                ev = self._idle[key].pop()
                self._idle_order.pop(id(ev), None)
                del self._pending[i]
                return req, ev, 0
            need = self.size_of(*key)
            if need > self.budget:
                del self._pending[i]
                self._errors.append(MemoryError(f"request {req.rid} needs {need} bytes; the budget is "
                                                f"{self.budget}"))
                self._cv.notify_all()
                return self._take()
            # release idle buffers of other shapes (least recently used first)
            while self._in_use + need > self.budget and self._idle_order:
                _, (k2, ev2) = self._idle_order.popitem(last=False)
                self._idle[k2].remove(ev2)
                self._in_use -= ev2.nbytes
            if self._in_use + need <= self.budget:
                del self._pending[i]
                self._in_use += need  # reserved; replaced by the real size after allocation
                return req, None, need
        return None

    def _worker(self, index: int) -> None:
        import torch

        stream = torch.cuda.Stream() if self.use_streams else None
        while True:
            with self._cv:
                while True:
                    if self._stop:
                        return
                    got = self._take()
                    if got is not None:
                        break
                    self._cv.wait()
                self._running += 1
                self.max_concurrent = max(self.max_concurrent, self._running)
            req, ev, reserved = got
            try:
                start = time.perf_counter()
                if stream is not None:
                    with torch.cuda.stream(stream):
                        if ev is None:
                            ev = self.make_evaluator(req.kind, req.norb, tuple(req.nelec))
                        energy, grad = ev.run(req)
                        stream.synchronize()
                else:
                    if ev is None:
                        ev = self.make_evaluator(req.kind, req.norb, tuple(req.nelec))
                    energy, grad = ev.run(req)
                end = time.perf_counter()
                res = Result(req.rid, energy, grad, req.arrival, start, end)
                err = None
            except BaseException as exc:  # noqa: BLE001
                res, err = None, exc
            with self._cv:
                self._running -= 1
                if ev is not None:
                    if reserved:
                        self._in_use += ev.nbytes - reserved
                    key = (req.kind, req.norb, tuple(req.nelec))
                    self._idle[key].append(ev)
                    self._idle_order[id(ev)] = (key, ev)
                elif reserved:
                    self._in_use -= reserved
                if err is not None:
                    self._errors.append(err)
                else:
                    self._results.append(res)
                self._cv.notify_all()


def latency_stats(results: list[Result]) -> dict:
    lat = sorted(r.latency for r in results)
    t0 = min(r.arrival for r in results)
    t1 = max(r.end for r in results)
    return {
        "requests": len(results),
        "p50_ms": 1e3 * statistics.median(lat),
        "p99_ms": 1e3 * float(np.percentile(lat, 99)),
        "evals_per_s": len(results) / (t1 - t0),
        "span_s": t1 - t0,
    }


def synthetic_stream(n: int, *, rate: float, seed: int = 0, norbs=(8, 10, 12, 14, 16), reps=(1, 2, 3),
                     gradient_fraction: float = 0.2):
    """Requests with Poisson arrivals (mean rate per second): norb uniform over
    `norbs` at half filling, n_reps uniform over `reps`, parameters N(0, 0.1)
    (the scale of the workload's diag-Coulomb entries), an energy or (with
    probability gradient_fraction) a gradient, and a double-factorized
    Hamiltonian of rank 2 * norb per norb.  Returns (offsets in seconds, requests)."""
    from ffsim_gb300 import random as fr
    from ffsim_gb300.variational import UCJOpSpinBalanced

    rng = np.random.default_rng(seed)
    hams = {m: fr.random_df_hamiltonian_normal(m, rank=2 * m, seed=seed + m) for m in norbs}
    offsets = np.cumsum(rng.exponential(1.0 / rate, size=n))
    reqs = []
    for i in range(n):
        m = int(rng.choice(norbs))
        L = int(rng.choice(reps))
        kind = "gradient" if rng.random() < gradient_fraction else "energy"
        params = rng.normal(scale=0.1, size=UCJOpSpinBalanced.n_params(m, L))
        reqs.append(Request(i, kind, m, (m // 2, m - m // 2), L, params, hams[m]))
    return offsets, reqs


def replay(server: LUCJServer, offsets, reqs) -> list[Result]:
    """Submit the requests at their arrival offsets and wait for all results."""
    t0 = time.perf_counter()
    for off, req in zip(offsets, reqs):
        now = time.perf_counter() - t0
        if off > now:
            time.sleep(off - now)
        req.arrival = t0 + off
        server.submit(req)
    return server.drain(len(reqs))
