"""Serving loop for LUCJ energy and gradient requests of mixed shapes.

Continuous batching on one GPU.  Requests that share a batch key -- kind
(energy or gradient), shape (norb, nelec), n_reps and Hamiltonian -- are
evaluated together: every term of the Hamiltonian runs once over all the
states of the batch (``BatchLUCJEnergy``, ``LUCJGradient.value_and_grad_batch``).
Worker threads, each with its own CUDA stream, take the oldest pending request
together with every pending request of its key (up to ``max_batch``), so
requests that arrive while others run join the next batch of their key, and
batches of different keys overlap on the device.

Admission is by device memory: an engine (the device buffers of one key's
shape for ``capacity`` states) is taken idle from the pool or allocated within
the HBM budget, releasing the least recently used idle engines of other shapes
when needed (their memory is freed at once); an engine for a batch takes at
most its worker's share of the budget, and a batch shrinks to what fits.  The
budget is an estimate: if the device cannot hold a new engine after all (the
caching allocator's segments fragment), the budget shrinks to the memory the
device reports free and the batch waits for its turn again.

Every request gets its own result: a value, or the error that stopped it
(``ValueError`` for an invalid request, ``MemoryError`` when even one state
does not fit the budget, ``TimeoutError`` when its deadline passed while it
waited, ``CancelledError`` after ``cancel``, or what the engine raised).  An
engine whose call raised (other than a cancellation) is not reused.  A batch
whose requests are all cancelled stops within about two Hamiltonian terms
(``ffgb_control``).

Requests of small shapes (norb <= 8, n_reps <= 4), energies and gradients,
go instead to a resident evaluator (``resident.ResidentEvaluator``): one
persistent kernel that takes them from a queue in host-mapped memory and
evaluates each inside one CTA, next to the batches on the device (for a
gradient the kernel runs the circuit, the Hamiltonian matvec and the backward
pass with its densities; the chain rule runs on the host at collection).  A resident lane thread submits
them in arrival order while the queue has room and collects the results;
cancellation and deadlines apply to them as to the others.  A request the
resident kernel cannot plan falls back to the batch path, and so do all small
requests if the resident evaluator cannot be created.

Results do not depend on what else runs: a state's result is the same alone
and in any batch (the dithering of a state's coefficients and the order of
its reductions do not depend on its neighbours), and a resident request's
result is the same alone and in any queue.
"""

from __future__ import annotations

import collections
import dataclasses
import statistics
import threading
import time
from concurrent.futures import CancelledError
from typing import Callable

import numpy as np


@dataclasses.dataclass
class Request:
    """One evaluation: kind is "energy" or "gradient"; params in the
    ``UCJOpSpinBalanced.from_parameters`` layout for (norb, n_reps).
    deadline: seconds after arrival by which it must have started (None: no
    deadline)."""

    rid: int
    kind: str
    norb: int
    nelec: tuple[int, int]
    n_reps: int
    params: np.ndarray
    ham: object
    arrival: float = 0.0
    deadline: float | None = None


@dataclasses.dataclass
class Result:
    rid: int
    energy: float | None
    grad: np.ndarray | None
    arrival: float
    start: float
    end: float
    error: BaseException | None = None
    batch: int = 0  # size of the batch it ran in (0: it did not run)
    path: str = "batch"  # "batch" or "resident"

    @property
    def ok(self) -> bool:
        return self.error is None

    @property
    def latency(self) -> float:
        return self.end - self.arrival


def batch_key(req: Request) -> tuple:
    return (req.kind, req.norb, tuple(req.nelec), req.n_reps, id(req.ham))


def validate(req: Request) -> None:
    """Checks a request before it is queued (raises ValueError)."""
    from ffsim_gb300.variational import UCJOpSpinBalanced

    if req.kind not in ("energy", "gradient"):
        raise ValueError(f"request {req.rid}: kind must be 'energy' or 'gradient', got {req.kind!r}")
    if not 1 <= req.norb <= 18:
        raise ValueError(f"request {req.rid}: norb must be in [1, 18], got {req.norb}")
    nelec = tuple(req.nelec)
    if len(nelec) != 2 or not all(0 <= n <= req.norb for n in nelec):
        raise ValueError(f"request {req.rid}: nelec must be two occupations in [0, norb], got {req.nelec}")
    if req.n_reps < 1:
        raise ValueError(f"request {req.rid}: n_reps must be positive, got {req.n_reps}")
    n = UCJOpSpinBalanced.n_params(req.norb, req.n_reps)
    if np.shape(req.params) != (n,):
        raise ValueError(f"request {req.rid}: expected {n} parameters, got shape {np.shape(req.params)}")
    if getattr(req.ham, "norb", req.norb) != req.norb:
        raise ValueError(f"request {req.rid}: the Hamiltonian acts on {req.ham.norb} orbitals, not {req.norb}")


class _Engine:
    """Device buffers of one (kind, norb, nelec) for up to `capacity` states."""

    def __init__(self, kind: str, norb: int, nelec: tuple[int, int], capacity: int, dtype):
        from ffsim_gb300.energy import BatchLUCJEnergy
        from ffsim_gb300.gradient import LUCJGradient

        self.capacity = capacity
        self.kind = kind
        if kind == "energy":
            self.impl = BatchLUCJEnergy(norb, nelec, capacity, dtype=dtype)
        else:
            self.impl = LUCJGradient(norb, nelec, dtype=dtype)
            self.impl._ensure_batch(capacity)
        self.nbytes = engine_bytes(kind, norb, nelec, capacity, dtype)

    def close(self) -> None:
        """Release the device buffers now."""
        if self.impl is not None:
            self.impl.close()
            self.impl = None

    def run(self, reqs: list[Request], control) -> list[tuple[float, np.ndarray | None]]:
        from ffsim_gb300.variational import UCJOpSpinBalanced

        r0 = reqs[0]
        if self.kind == "energy":
            ops = [UCJOpSpinBalanced.from_parameters(r.params, norb=r.norb, n_reps=r.n_reps) for r in reqs]
            return [(float(e), None) for e in self.impl(ops, r0.ham, control)]
        params = np.stack([r.params for r in reqs])
        es, gs = self.impl.value_and_grad_batch(params, r0.n_reps, r0.ham, control=control)
        return [(float(e), g) for e, g in zip(es, gs)]


def engine_bytes(kind: str, norb: int, nelec: tuple[int, int], capacity: int, dtype) -> int:
    """Device bytes an engine of this shape and capacity holds."""
    import torch

    from ffsim_gb300 import _lib
    from ffsim_gb300._state import dim

    code = _lib.FFGB_C64 if dtype == torch.complex64 else _lib.FFGB_C128
    el = 8 if dtype == torch.complex64 else 16
    lib = _lib.load()
    d = dim(norb, nelec)
    if kind == "energy":
        return capacity * d * el + lib.ffgb_batch_scratch_bytes(0, code, norb, *nelec, capacity)
    per_state = max(lib.ffgb_scratch_bytes(op, code, norb, *nelec) for op in (0, 1, 3))
    workers = 4  # LUCJGradient's lanes, each with its own scratch
    return ((2 + 2 * capacity) * d * el + (1 + workers) * per_state
            + lib.ffgb_batch_scratch_bytes(1, code, norb, *nelec, capacity))


class LUCJServer:
    """Continuous-batching server.

    workers: batches in flight at once (one CUDA stream each).
    max_batch: states per batch (at most).
    budget_bytes: device memory the pooled engines may hold (default: 85% of
    the free HBM when the server starts).
    make_engine(kind, norb, nelec, capacity) / size_of(kind, norb, nelec,
    capacity): injection points (the defaults build GPU engines); tests
    substitute host-only fakes.
    resident: route small energy requests to a resident evaluator (default:
    when the engines are the GPU ones and the dtype is complex64);
    make_resident() builds it (injection point, like make_engine).
    """

    def __init__(self, workers: int = 2, *, max_batch: int = 64, dtype=None, budget_bytes: int | None = None,
                 make_engine: Callable | None = None, size_of: Callable | None = None, use_streams: bool = True,
                 resident: bool | None = None, make_resident: Callable | None = None):
        import torch

        self.dtype = dtype if dtype is not None else torch.complex64
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            budget_bytes = int(0.85 * free)
        self.budget = int(budget_bytes)
        # an engine for a batch (more than one state) may take at most its
        # worker's share of the budget, so that every worker can hold one
        self.engine_limit = self.budget // max(1, workers)
        self.max_batch = max(1, int(max_batch))
        self._default_make = lambda k, n, ne, c: _Engine(k, n, ne, c, self.dtype)
        self.make_engine = make_engine or self._default_make
        self._evicted = False  # idle engines were released since the last build
        self.oom_retries = 0  # engine builds that found less device memory than the budget
        self.size_of = size_of or (lambda k, n, ne, c: engine_bytes(k, n, ne, c, self.dtype))
        self.use_streams = use_streams
        self._cv = threading.Condition()
        self._pending: collections.deque[Request] = collections.deque()
        self._idle: dict[tuple, list] = collections.defaultdict(list)  # (kind, norb, nelec) -> engines
        self._idle_order: collections.OrderedDict = collections.OrderedDict()  # id -> (shape, engine), LRU
        self._in_use = 0  # bytes held by pooled and running engines
        self._results: dict[int, Result] = {}
        self._running: dict[int, tuple] = {}  # rid -> (batch requests, control)
        self._cancelled: set[int] = set()
        self._stop = False
        self.max_concurrent = 0
        self.batch_sizes: list[int] = []
        self._n_running = 0
        if resident is None:
            resident = make_resident is not None or (make_engine is None and self.dtype == torch.complex64)
        self.resident = bool(resident)
        self._make_resident = make_resident or (lambda: _default_resident())
        self._res_pending: collections.deque[Request] = collections.deque()
        self._res_inflight: dict[int, tuple[Request, float]] = {}  # ticket -> (request, start)
        self._res_ticket: dict[int, int] = {}  # rid -> ticket
        self.resident_served = 0
        self._threads = [threading.Thread(target=self._worker, daemon=True) for _ in range(workers)]
        if self.resident:
            self._threads.append(threading.Thread(target=self._resident_lane, daemon=True))
        for t in self._threads:
            t.start()

    # -- client side -------------------------------------------------------
    def submit(self, req: Request) -> None:
        """Queue a request; an invalid one gets its error result at once."""
        if not req.arrival:
            req.arrival = time.perf_counter()
        try:
            validate(req)
        except ValueError as exc:
            self._finish_one(req, None, exc, 0, time.perf_counter())
            return
        with self._cv:
            if self._for_resident(req):
                self._res_pending.append(req)
            else:
                self._pending.append(req)
            self._cv.notify_all()

    def _for_resident(self, req: Request) -> bool:
        from ffsim_gb300 import resident as res

        return self.resident and res.accepts(req.norb, req.n_reps)

    def cancel(self, rid: int) -> bool:
        """Cancel a request: a pending one is dropped at once, a running one
        gets a cancellation result (and its batch stops early when every
        request of the batch is cancelled).  False if it already finished."""
        with self._cv:
            if rid in self._results:
                return False
            for queue in (self._pending, self._res_pending):
                for i, req in enumerate(queue):
                    if req.rid == rid:
                        del queue[i]
                        self._record(req, None, CancelledError(f"request {rid} was cancelled"), 0,
                                     time.perf_counter())
                        return True
            self._cancelled.add(rid)
            self._cv.notify_all()
            if rid in self._running:
                batch, control = self._running[rid]
                if control is not None and all(r.rid in self._cancelled for r in batch):
                    control.request_cancel()
            return True

    def drain(self, n_expected: int, timeout: float = 3600.0) -> list[Result]:
        """Wait until n_expected results exist; returns them sorted by rid
        (each with its value or its error)."""
        deadline = time.perf_counter() + timeout
        with self._cv:
            while len(self._results) < n_expected:
                left = deadline - time.perf_counter()
                if left <= 0:
                    raise TimeoutError(f"{len(self._results)} of {n_expected} requests finished")
                self._cv.wait(timeout=min(left, 1.0))
            return sorted(self._results.values(), key=lambda r: r.rid)

    def close(self) -> None:
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        for t in self._threads:
            t.join(timeout=60)

    # -- scheduling -----------------------------------------------------------
    def _record(self, req: Request, value, error, batch: int, start: float, path: str = "batch") -> None:
        """Under the lock: the result of one request."""
        energy, grad = value if value is not None else (None, None)
        if req.rid in self._cancelled and error is None:
            error = CancelledError(f"request {req.rid} was cancelled")
        self._results[req.rid] = Result(req.rid, energy, grad, req.arrival, start, time.perf_counter(), error, batch,
                                        path)
        self._cv.notify_all()

    def _finish_one(self, req, value, error, batch, start) -> None:
        with self._cv:
            self._record(req, value, error, batch, start)

    def _expire(self, now: float) -> None:
        """Under the lock: pending requests past their deadline."""
        self._pending = self._expired(self._pending, now)

    def _expired(self, queue, now: float):
        keep = collections.deque()
        for req in queue:
            if req.deadline is not None and now > req.arrival + req.deadline:
                self._record(req, None, TimeoutError(f"request {req.rid} waited past its deadline"), 0, now)
            else:
                keep.append(req)
        return keep

    @staticmethod
    def _release(ev) -> None:
        """An engine leaves the pool: free its device memory now."""
        close = getattr(ev, "close", None)
        if close is not None:
            close()

    def _reserve(self, shape: tuple, cap: int) -> int:
        """Under the lock: bytes for a new engine of `shape` and capacity
        `cap`, releasing idle engines of other shapes (least recently used
        first) as needed; 0 if it does not fit."""
        need = self.size_of(shape[0], shape[1], shape[2], cap)
        if need > (self.engine_limit if cap > 1 else self.budget):
            return 0
        for oid, (s2, e2) in list(self._idle_order.items()):
            if self._in_use + need <= self.budget:
                break
            if s2 == shape:
                continue
            del self._idle_order[oid]
            self._idle[s2].remove(e2)
            self._in_use -= e2.nbytes
            self._release(e2)
            self._evicted = True
        if self._in_use + need > self.budget:
            return 0
        self._in_use += need
        return need

    def _take(self):
        """Under the lock: the oldest admissible request with the pending
        requests of its key that join it, and an idle engine or the bytes
        reserved for a new one: (group, engine or None, reserved bytes,
        capacity)."""
        self._expire(time.perf_counter())
        for req in list(self._pending):
            key = batch_key(req)
            shape = key[:3]
            group = [r for r in self._pending if batch_key(r) == key][: self.max_batch]
            idle = sorted(self._idle[shape], key=lambda e: e.capacity)
            fit = [e for e in idle if e.capacity >= len(group)]
            ev, reserved, cap = (fit[0] if fit else None), 0, 0
            if ev is None:
                # a new engine for the whole group (capacities are powers of two) ...
                cap = min(1 << (len(group) - 1).bit_length(), self.max_batch)
                reserved = self._reserve(shape, cap)
                if not reserved and idle:  # ... else the largest idle one
                    ev = idle[-1]
                while not reserved and ev is None and cap > 1:  # ... else a smaller new one
                    cap //= 2
                    reserved = self._reserve(shape, cap)
                if not reserved and ev is None:
                    if self.size_of(shape[0], shape[1], shape[2], 1) > self.budget:
                        self._pending.remove(req)
                        self._record(req, None, MemoryError(
                            f"request {req.rid} needs {self.size_of(shape[0], shape[1], shape[2], 1)} bytes; "
                            f"the budget is {self.budget}"), 0, time.perf_counter())
                        return self._take()
                    continue  # waits for memory held by running batches
            if ev is not None:
                self._idle[shape].remove(ev)
                self._idle_order.pop(id(ev), None)
                cap = ev.capacity
            group = group[:cap]
            for r in group:
                self._pending.remove(r)
            return group, ev, reserved, cap
        return None

    def _worker(self) -> None:
        import torch

        from ffsim_gb300 import _lib

        stream = torch.cuda.Stream() if self.use_streams else None
        while True:
            with self._cv:
                while True:
                    if self._stop:
                        return
                    got = self._take()
                    if got is not None:
                        break
                    self._cv.wait(timeout=0.5)
                group, ev, reserved, cap = got
                control = _lib.Control()
                for r in group:
                    self._running[r.rid] = (group, control)
                self._n_running += 1
                self.max_concurrent = max(self.max_concurrent, self._n_running)
                self.batch_sizes.append(len(group))
            start = time.perf_counter()
            values, err = None, None
            shape = batch_key(group[0])[:3]
            if ev is None:
                ev = self._build(shape, cap, reserved, group)
                if ev is None:  # no device memory after all: the group waits again
                    with self._cv:
                        self._n_running -= 1
                        for r in group:
                            self._running.pop(r.rid, None)
                    continue
            try:
                if stream is not None:
                    with torch.cuda.stream(stream):
                        values = ev.run(group, control)
                        stream.synchronize()
                else:
                    values = ev.run(group, control)
            except BaseException as exc:  # noqa: BLE001
                err = exc
            with self._cv:
                self._n_running -= 1
                for r in group:
                    self._running.pop(r.rid, None)
                keep = ev is not None and (err is None or isinstance(err, CancelledError))
                if keep:
                    if reserved:
                        self._in_use += ev.nbytes - reserved
                    self._idle[shape].append(ev)
                    self._idle_order[id(ev)] = (shape, ev)
                else:  # failed: its memory is released
                    self._in_use -= reserved if reserved else ev.nbytes
                    self._release(ev)
                    self._evicted = True
                    ev = None
                for i, r in enumerate(group):
                    self._record(r, None if err is not None else values[i], err, len(group), start)

    def _build(self, shape: tuple, cap: int, reserved: int, group: list[Request]):
        """A new engine for `group`, or None when the device cannot hold it
        now.  The caching allocator keeps released engines' memory unless it
        is emptied, so it is emptied after evictions.  If the allocation
        still fails, the budget shrinks to what the device really has, the
        reservation is returned and the group goes back to the front of the
        queue; after three such failures its requests fail with MemoryError."""
        import torch

        if self._evicted and self.make_engine is self._default_make:
            self._evicted = False
            torch.cuda.empty_cache()
        try:
            return self.make_engine(shape[0], shape[1], shape[2], cap)
        except BaseException as exc:  # noqa: BLE001
            oom = isinstance(exc, MemoryError) or type(exc).__name__ == "OutOfMemoryError"
            with self._cv:
                self._in_use -= reserved
                tries = max(getattr(r, "_oom_tries", 0) for r in group) + 1
                if not oom or tries >= 3:
                    for r in group:
                        self._record(r, None, exc, 0, time.perf_counter())
                    return None
                for r in group:
                    r._oom_tries = tries
                self._pending.extendleft(reversed(group))
                self.oom_retries += 1
            if self.make_engine is self._default_make:
                torch.cuda.empty_cache()
                free, _ = torch.cuda.mem_get_info()
                with self._cv:
                    self.budget = min(self.budget, self._in_use + int(0.9 * free))
                    self.engine_limit = min(self.engine_limit, self.budget)
                    self._cv.notify_all()
            return None

    def _resident_lane(self) -> None:
        """Feeds the resident evaluator in arrival order while its queue has
        room, forwards cancellations, and collects the results."""
        from ffsim_gb300.variational import UCJOpSpinBalanced

        ev = None
        try:
            while True:
                with self._cv:
                    if self._stop:
                        return
                    self._res_pending = self._expired(self._res_pending, time.perf_counter())
                    if not self._res_pending and not self._res_inflight:
                        self._cv.wait(timeout=0.5)
                        continue
                    # taken out of the pending queue under the lock: a cancel()
                    # from now on finds them through self._cancelled
                    todo = list(self._res_pending)
                    self._res_pending.clear()
                    cancel = [t for rid, t in self._res_ticket.items() if rid in self._cancelled]
                if ev is None:
                    try:
                        ev = self._make_resident()
                    except BaseException:  # noqa: BLE001
                        # no resident evaluator on this device: its requests,
                        # and every small one from now on, take the batch path
                        with self._cv:
                            self.resident = False
                            self._pending.extend(todo)
                            self._pending.extend(self._res_pending)
                            self._res_pending.clear()
                            self._cv.notify_all()
                        return
                for t in cancel:
                    ev.cancel(t)
                for i, req in enumerate(todo):
                    start = time.perf_counter()
                    try:
                        if req.kind == "gradient":
                            ticket = ev.submit_grad(req.params, req.n_reps, req.ham, req.nelec)
                        else:
                            op = UCJOpSpinBalanced.from_parameters(req.params, norb=req.norb, n_reps=req.n_reps)
                            ticket = ev.submit(op, req.ham, req.nelec)
                    except MemoryError:
                        with self._cv:  # the queue is full: the rest wait for collected results
                            self._res_pending.extendleft(reversed(todo[i:]))
                        break
                    except NotImplementedError:
                        with self._cv:  # the resident kernel cannot plan it: the batch path takes it
                            self._pending.append(req)
                            self._cv.notify_all()
                        continue
                    except BaseException as exc:  # noqa: BLE001
                        with self._cv:
                            self._record(req, None, exc, 0, start, "resident")
                        continue
                    with self._cv:
                        self._res_inflight[ticket] = (req, start)
                        self._res_ticket[req.rid] = ticket
                        cancelled = req.rid in self._cancelled
                    if cancelled:
                        ev.cancel(ticket)
                done = []
                for ticket, (req, start) in list(self._res_inflight.items()):
                    try:
                        if req.kind == "gradient":
                            got = ev.poll_grad(ticket)
                        else:
                            e = ev.poll(ticket)
                            got = None if e is None else (e, None)
                    except BaseException as exc:  # noqa: BLE001
                        done.append((ticket, req, start, None, exc))
                        continue
                    if got is not None:
                        done.append((ticket, req, start, got, None))
                if done:
                    with self._cv:
                        for ticket, req, start, value, err in done:
                            del self._res_inflight[ticket]
                            self._res_ticket.pop(req.rid, None)
                            self._record(req, value, err, 1, start, "resident")
                            self.resident_served += err is None
                else:
                    time.sleep(200e-6)
        finally:
            if ev is not None:
                ev.close()


def _default_resident():
    from ffsim_gb300.resident import ResidentEvaluator

    # the kernel lives only while requests come (it exits 5 ms after the
    # last), so between bursts it holds no SM resources the batches could use
    return ResidentEvaluator(n_slots=256, n_ctas=8, idle_seconds=0.005)


def latency_stats(results: list[Result]) -> dict:
    ok = [r for r in results if r.ok]
    lat = sorted(r.latency for r in ok)
    t0 = min(r.arrival for r in ok)
    t1 = max(r.end for r in ok)
    return {
        "requests": len(results),
        "completed": len(ok),
        "p50_ms": 1e3 * statistics.median(lat),
        "p99_ms": 1e3 * float(np.percentile(lat, 99)),
        "evals_per_s": len(ok) / (t1 - t0),
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
