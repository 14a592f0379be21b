"""LUCJ energy throughput on one GB300 (or N independent replicas).

Workload (the metric's configuration): norb=16, nelec=(8,8) (dim_a = dim_b =
12870, 1.656e8 amplitudes), spin-balanced UCJ with n_reps=2 applied to the
Hartree-Fock state (Haar orbital rotations, diag-Coulomb entries N(0,0.1)),
then <psi|H|psi> for a synthetic double-factorized Hamiltonian (Hermitian
one-body N(0,1)/16, rank 32, Haar term rotations, J_t entries N(0,0.05),
constant -100).  Inputs are seeded synthetic data (the reference publishes no
dataset).  A step is one batch: the energies of --batch-states (default 4)
UCJ parameter sets under the Hamiltonian, as the serving loop evaluates
them (BatchLUCJEnergy: every Hamiltonian term runs once over all the states).

Reported:
* value      complex64 evaluations/s, device time (CUDA events on the
             launching stream), inputs resident; max over ranks, summed over
             ranks (replicas).
* single     one evaluation per step (LUCJEnergy) beside it.
* served     the same workload through the continuous-batching serving loop,
             every request submitted at once (wall clock).
* e2e        the batch step through the public API ``BatchLUCJEnergy`` with
             host (numpy) inputs and the energies read back every step.
* complex128 the plain complex128 GPU path on the same GPU (fewer steps).
* roofline   the dominant kernel (one window stage of the stage-major
             rotation: 2 S algorithmic bytes, S the state size, timed with
             CUDA events through ffgb_debug_stage) against the measured copy
             bandwidth in MEASURED_PEAKS.json; the cross-half pass, a full
             orbital rotation (4 S) and the whole evaluation (S (6 L + 3 (R+1)),
             the final UCJ rotation merged into every term) beside it.
* cpu_baseline the C/OpenMP restatement of the reference CPU algorithm on a
             bounded sample (one orbital rotation + one diag-Coulomb evolution
             at norb=16, complex128), extrapolated to one evaluation.

``--impl reference`` times that CPU restatement alone as the reference arm.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

NORB, NELEC, N_REPS, RANK = 16, (8, 8), 2, 32
METRIC = "LUCJ energy evals/s norb=16 (8,8) c64 vs c128 at |dE|<=1e-6 Ha; p50/p99 ms"
WORKLOAD = "LUCJ n_reps=2 from HF + DF Hamiltonian rank 32 energy, norb=16, nelec=(8,8)"


def run_config(world: int, batch: int) -> dict:
    """The workload's config block, identical in both arms."""
    return {"workload": WORKLOAD, "norb": NORB, "nelec": list(NELEC), "n_reps": N_REPS, "df_rank": RANK,
            "batch_states": batch, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (state 1.32 GB in complex64, 2.65 GB in complex128)"}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(seed: int = 2026):
    import ffsim_gb300 as f

    ucj = f.random.random_ucj_op_spin_balanced(NORB, n_reps=N_REPS, diag_coulomb_normal=True,
                                               diag_coulomb_scale=0.1, seed=seed)
    ham = f.random.random_df_hamiltonian_normal(NORB, rank=RANK, seed=seed + 1)
    return ucj, ham


def time_energy(dtype, steps, warmup, ucj, ham, stream):
    """Per-step CUDA-event times (ms) of LUCJ energy evaluations on `stream`."""
    import torch

    import ffsim_gb300 as f

    ev = f.LUCJEnergy(NORB, NELEC, dtype=dtype)
    energies = []
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            energies.append(ev(ucj, ham))
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for k in range(steps):
            starts[k].record(stream)
            energies.append(ev(ucj, ham))
            ends[k].record(stream)
        torch.cuda.synchronize()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    del ev
    torch.cuda.empty_cache()
    return times, energies


def make_batch_ops(seed: int, n: int, first):
    """The operators of a batch step: the single-evaluation workload's
    operator first, then n - 1 more drawn the same way (other seeds)."""
    import ffsim_gb300 as f

    return [first] + [f.random.random_ucj_op_spin_balanced(NORB, n_reps=N_REPS, diag_coulomb_normal=True,
                                                           diag_coulomb_scale=0.1, seed=seed + 1000 * k)
                      for k in range(1, n)]


def time_batch_energy(dtype, steps, warmup, ops, ham, stream):
    """Per-step CUDA-event times (ms) of batched LUCJ energy evaluations (one
    step = the energies of every operator of `ops`, BatchLUCJEnergy) on
    `stream`; returns (times, energies of the last step)."""
    import torch

    import ffsim_gb300 as f

    ev = f.BatchLUCJEnergy(NORB, NELEC, len(ops), dtype=dtype)
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            energies = ev(ops, ham)
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for k in range(steps):
            starts[k].record(stream)
            energies = ev(ops, ham)
            ends[k].record(stream)
        torch.cuda.synchronize()
    times = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    del ev
    torch.cuda.empty_cache()
    return times, energies


def time_batch_e2e(steps, ops, ham):
    """Wall time per batch step through the public API (host parameter arrays
    in, energies read back)."""
    import torch

    import ffsim_gb300 as f

    ev = f.BatchLUCJEnergy(NORB, NELEC, len(ops), dtype=torch.complex64)
    ev(ops, ham)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ev(ops, ham)
    t1 = time.perf_counter()
    del ev
    torch.cuda.empty_cache()
    return (t1 - t0) / steps


def time_e2e(steps, ucj, ham):
    """Wall time per evaluation through the public API with host inputs."""
    import torch

    import ffsim_gb300 as f

    ev = f.LUCJEnergy(NORB, NELEC, dtype=torch.complex64)
    ev(ucj, ham)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        ev(ucj, ham)  # numpy inputs -> planning -> kernels -> energy read back (synchronizes)
    t1 = time.perf_counter()
    del ev
    torch.cuda.empty_cache()
    return (t1 - t0) / steps


def window_stage_traffic():
    """DRAM bytes (read + write) of one 8-orbital window stage at norb=16 (8,8)
    complex64: the sum over its class launches of dram__bytes_read.sum +
    dram__bytes_write.sum in the committed ncu capture
    profiles/window_stage_norb16_c64_traffic.txt (the command that made it is
    in its header).  None when that capture is absent."""
    p = ROOT / "profiles" / "window_stage_norb16_c64_traffic.txt"
    if not p.exists():
        return None, None
    total = 0.0
    for line in p.read_text().splitlines():  # kernel | time_us | dram_read_bytes | dram_write_bytes
        parts = [x.strip() for x in line.split("|")]
        if len(parts) >= 4 and parts[0].startswith("win_class_kernel"):
            total += float(parts[2]) + float(parts[3])
    return (total if total > 0 else None), str(p.relative_to(ROOT))


def eval_bytes_moved():
    """DRAM bytes (read + write) of one whole evaluation at norb=16 (8,8),
    summed over its launches in the committed ncu capture
    profiles/lucj_energy_norb16_c64_dram.txt.  None when absent."""
    p = ROOT / "profiles" / "lucj_energy_norb16_c64_dram.txt"
    if not p.exists():
        return None, None
    for line in p.read_text().splitlines():
        parts = [x.strip() for x in line.split("|")]
        if len(parts) >= 3 and parts[0] == "total":
            return float(parts[2]), str(p.relative_to(ROOT))
    return None, None


def window_stage_flops(norb: int, nocc: int, b: int = 8) -> float:
    """FP32 flops of one b-orbital window stage on the orbitals [0, b) of a
    sector with nocc of norb orbitals occupied, per column: a class with K
    electrons in the window has C(b, K) members per group, and each of the
    b (b - 1) / 2 rotations of its network takes the C(b-2, K-1) member pairs
    with exactly one of its two orbitals occupied, 12 FMA (24 flops) per pair."""
    out = 0.0
    for k in range(0, b + 1):
        groups = math.comb(norb - b, nocc - k)
        pairs = math.comb(b - 2, k - 1) if 1 <= k <= b - 1 else 0
        out += groups * (b * (b - 1) // 2) * pairs * 24
    return out


def rotation_flops(norb: int, nelec) -> float:
    """Floating-point operations of the complex128 two-sector rotation: the
    adjacent-Givens network has norb (norb - 1) / 2 rotations per sector, each
    touching the strings with exactly one of its two orbitals occupied
    (2 C(norb-2, n-1) of C(norb, n)) with 6 FMA = 12 flops per amplitude."""
    d = math.comb(norb, nelec[0]) * math.comb(norb, nelec[1])
    flops = 0.0
    for n in nelec:
        frac = 2 * math.comb(norb - 2, n - 1) / math.comb(norb, n)
        flops += norb * (norb - 1) / 2 * frac * d * 12
    return flops


def stage_rooflines(stream, reps: int = 8):
    """CUDA-event times of single stages and of a full orbital rotation on a
    resident norb=16 complex64 state, with their algorithmic bytes:
    a window stage or the cross-half pass reads and writes the state once
    (2 S); a two-sector orbital rotation is 4 S (one read and one write per
    sector)."""
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib
    from ffsim_gb300._state import scratch

    d = f.dim(NORB, NELEC)
    S = d * 8
    u = _lib.cmat(f.random.random_unitary(NORB, seed=99))
    out = {}
    with torch.cuda.stream(stream):
        v = torch.randn(d, dtype=torch.complex64, device="cuda")
        v /= torch.linalg.vector_norm(v)
        buf, nbytes = scratch(v, 0, NORB, *NELEC)
        sptr = stream.cuda_stream

        def timed(fn):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            return a.elapsed_time(b) / reps

        def stage(k):
            return lambda: _lib.call("ffgb_debug_stage", v.data_ptr(), _lib.FFGB_C64, NORB, NELEC[0], NELEC[1],
                                     _lib.dptr(u), k, sptr)

        def rot():
            _lib.call("ffgb_apply_orbital_rotation", v.data_ptr(), _lib.FFGB_C64, NORB, NELEC[0], NELEC[1],
                      _lib.dptr(u), _lib.dptr(u), buf.data_ptr(), nbytes, sptr)

        out["window_stage_ms"] = timed(stage(0))
        out["cross_half_stage_ms"] = timed(stage(2))  # all eight sites in one pass
        out["rotation_ms"] = timed(rot)
    del v, buf
    torch.cuda.empty_cache()
    out["S"] = S
    return out


def time_rotation_c128(stream, reps: int = 2) -> float:
    """CUDA-event time (ms) of one complex128 two-sector orbital rotation on a
    resident norb=16 (8,8) state."""
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib
    from ffsim_gb300._state import scratch

    d = f.dim(NORB, NELEC)
    u = _lib.cmat(f.random.random_unitary(NORB, seed=98))
    with torch.cuda.stream(stream):
        v = torch.randn(d, dtype=torch.complex128, device="cuda")
        v /= torch.linalg.vector_norm(v)
        buf, nbytes = scratch(v, 0, NORB, *NELEC)

        def rot():
            _lib.call("ffgb_apply_orbital_rotation", v.data_ptr(), _lib.FFGB_C128, NORB, NELEC[0], NELEC[1],
                      _lib.dptr(u), _lib.dptr(u), buf.data_ptr(), nbytes, stream.cuda_stream)

        rot()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            rot()
        b.record(stream)
        torch.cuda.synchronize()
    del v, buf
    torch.cuda.empty_cache()
    return a.elapsed_time(b) / reps


def run_profile_eval(args) -> None:
    """Two single LUCJ energy evaluations of the metric's workload shape at
    --norb (half filling), nothing timed: the second is the one a profiler
    captures (its launches follow the first's, the same number)."""
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib

    norb = args.norb
    nelec = (norb // 2, norb - norb // 2)
    ucj = f.random.random_ucj_op_spin_balanced(norb, n_reps=N_REPS, diag_coulomb_normal=True,
                                               diag_coulomb_scale=0.1, seed=2026)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=2 * norb, seed=2027)
    ev = f.LUCJEnergy(norb, nelec, dtype=torch.complex64)
    lib = _lib.load()
    counts = []
    for _ in range(2):
        n0 = lib.ffgb_launch_count()
        e = ev(ucj, ham)
        torch.cuda.synchronize()
        counts.append(lib.ffgb_launch_count() - n0)
    print(json.dumps({"profile_eval": norb, "energy": e, "launches_per_evaluation": counts,
                      "state_bytes": f.dim(norb, nelec) * 8, "df_rank": 2 * norb}), flush=True)


def run_ops(args) -> None:
    """Per-operation GB/s on a resident state (--ops): one JSON line per op,
    each against its algorithmic bytes (S = state bytes)."""
    import numpy as np
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300 import _lib
    from ffsim_gb300._state import scratch

    norb = args.norb
    nelec = (norb // 2, norb - norb // 2)
    d = f.dim(norb, nelec)
    dtype = torch.complex64 if args.dtype == "c64" else torch.complex128
    code = _lib.FFGB_C64 if args.dtype == "c64" else _lib.FFGB_C128
    el = 8 if args.dtype == "c64" else 16
    S = d * el
    peak, peak_kind = _peaks()
    rng = np.random.default_rng(7)
    u = _lib.cmat(f.random.random_unitary(norb, seed=rng))
    jm = np.asarray(f.random.random_symmetric_matrix_normal(norb, scale=0.1, seed=rng), dtype=np.float64)
    ham = f.random.random_df_hamiltonian_normal(norb, rank=norb, seed=11)
    ob, dcm, hrots = ham._arrays()
    eout = np.zeros(1)
    stream = torch.cuda.Stream()
    sptr = stream.cuda_stream
    with torch.cuda.stream(stream):
        v = torch.randn(d, dtype=dtype, device="cuda")
        v /= torch.linalg.vector_norm(v)
        out = torch.empty_like(v)
        buf, nbytes = scratch(v, 3, norb, *nelec)  # the largest: two states plus density partials

    def timed(fn):
        for _ in range(min(args.warmup, 2)):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / args.reps

    # stage sequences: three 8-orbital windows up to norb 12; windows on the
    # halves around the cross-half stage (index 2) up to 16; for 17 and 18 one
    # window and three overlapping windows on each side of it (index 4)
    cs_index = None if norb <= 12 else (2 if norb <= 16 else 4)
    ops = {
        "window_stage": (2 * S, lambda: _lib.call("ffgb_debug_stage", v.data_ptr(), code, norb, nelec[0], nelec[1],
                                                  _lib.dptr(u), 0, sptr)),
        "cross_half_stage": (2 * S, lambda: _lib.call("ffgb_debug_stage", v.data_ptr(), code, norb, nelec[0],
                                                      nelec[1], _lib.dptr(u), cs_index, sptr)),
        "orbital_rotation": (4 * S, lambda: _lib.call("ffgb_apply_orbital_rotation", v.data_ptr(), code, norb,
                                                      nelec[0], nelec[1], _lib.dptr(u), _lib.dptr(u),
                                                      buf.data_ptr(), nbytes, sptr)),
        "diag_coulomb_evolution": (2 * S, lambda: _lib.call(
            "ffgb_apply_diag_coulomb_evolution", v.data_ptr(), code, norb, nelec[0], nelec[1], _lib.dptr(jm),
            _lib.dptr(jm), _lib.dptr(jm), 1.0, 0, None, None, buf.data_ptr(), nbytes, sptr)),
        "rotated_diag_matvec": (9 * S, lambda: _lib.call(
            "ffgb_rotated_diag_matvec", v.data_ptr(), out.data_ptr(), code, norb, nelec[0], nelec[1], None,
            _lib.dptr(jm), 0, _lib.dptr(u), 1, buf.data_ptr(), nbytes, sptr)),
        # energy of a rank-norb double-factorized Hamiltonian: R + 1 terms, 3 S each
        f"df_energy_rank{norb}": (3 * S * (norb + 1), lambda: _lib.call(
            "ffgb_df_expectation", v.data_ptr(), code, norb, nelec[0], nelec[1], _lib.dptr(ob), dcm.shape[0],
            _lib.dptr(dcm), hrots.ctypes.data_as(_lib._dp), float(ham.constant), 0, None, _lib.dptr(eout),
            buf.data_ptr(), nbytes, sptr)),
    }
    if cs_index is None or args.dtype != "c64":
        del ops["cross_half_stage"]
    if args.dtype != "c64":  # the stage kernels are complex64
        del ops["window_stage"]

    # compositions on the same entry points: Trotter evolution, the
    # spin-unbalanced UCJ operator, 1-RDMs and a molecular Hamiltonian
    def on_stream(fn):
        def run():
            with torch.cuda.stream(stream):
                fn()
        return run

    ucju = f.UCJOpSpinUnbalanced.from_parameters(
        rng.uniform(-0.5, 0.5, size=f.UCJOpSpinUnbalanced.n_params(norb, 2)), norb=norb, n_reps=2)
    ops[f"trotter_step_rank{norb}"] = (norb * 6 * S + 4 * S, on_stream(
        lambda: f.simulate_trotter_double_factorized(v, ham, 0.1, norb=norb, nelec=nelec, copy=False)))
    ops["ucj_spin_unbalanced_apply_L2"] = (3 * 4 * S + 2 * 2 * S, on_stream(
        lambda: f.apply_unitary(v, ucju, norb, nelec, copy=False)))
    ops["rdm1"] = (S, on_stream(lambda: f.rdms(v, norb, nelec)))
    # the adjoint gradient's densities between two states (each reads both once)
    dens_out = np.zeros(2 * 3 * norb * norb)
    ops["density_transition_rdm1"] = (2 * S, lambda: _lib.call(
        "ffgb_transition_rdm1", v.data_ptr(), out.data_ptr(), code, norb, nelec[0], nelec[1], _lib.dptr(dens_out),
        buf.data_ptr(), nbytes, sptr))
    ops["density_pair"] = (2 * S, lambda: _lib.call(
        "ffgb_pair_density", v.data_ptr(), out.data_ptr(), code, norb, nelec[0], nelec[1], _lib.dptr(dens_out),
        buf.data_ptr(), nbytes, sptr))
    # split-operator step of a Hubbard chain (hopping 1, U 4): one rotation by
    # the banded near-identity exp(-i 0.1 h) and one diagonal evolution (the
    # closing rotation by the identity is skipped)
    hop = np.diag(-np.ones(norb - 1), 1)
    hub = f.DiagonalCoulombHamiltonian(hop + hop.T, np.stack([np.zeros((norb, norb)), 4.0 * np.eye(norb)]))
    ops[f"trotter_split_op_step_norb{norb}"] = (4 * S + 2 * S, on_stream(
        lambda: f.simulate_trotter_diag_coulomb_split_op(v, hub, 0.1, norb=norb, nelec=nelec, copy=False)))
    if norb == NORB:
        n12, ne12 = 12, (6, 6)
        g = rng.standard_normal((n12, n12)) + 1j * rng.standard_normal((n12, n12))
        mk = rng.standard_normal((n12 * n12, n12, n12)) + 1j * rng.standard_normal((n12 * n12, n12, n12))
        mk = mk + mk.transpose(0, 2, 1).conj()
        mol = f.MolecularHamiltonian((g + g.conj().T) / 2, np.tensordot(mk, mk, axes=(0, 0)) / n12**2, 0.5)
        lin12 = f.linear_operator(mol, n12, ne12)
        n_terms = mol.to_double_factorized().diag_coulomb_mats.shape[0] + 1
        with torch.cuda.stream(stream):
            v12 = torch.randn(f.dim(n12, ne12), dtype=dtype, device="cuda")
        ops[f"molecular_matvec_norb12_{n_terms}terms"] = (n_terms * 9 * v12.numel() * el,
                                                          on_stream(lambda: lin12 @ v12))
    for name, (nb, fn) in ops.items():
        if args.op and args.op not in name:
            continue
        try:
            ms = timed(fn)
            gbs = nb / (ms * 1e-3) / 1e9
            line = {"op": name, "norb": norb, "nelec": list(nelec), "dtype": args.dtype, "ms": ms,
                    "algorithmic_bytes": nb, "GB/s": gbs, "frac": gbs / peak, "peak": peak,
                    "peak_kind": peak_kind}
        except Exception as exc:  # noqa: BLE001
            line = {"op": name, "norb": norb, "dtype": args.dtype, "unsupported": str(exc)}
        print(json.dumps(line), flush=True)


def run_grad(args) -> None:
    """Gradient workload: norb=12 (6,6), UCJ n_reps=3, DF rank 24, a batch of
    parameter vectors: energies and adjoint gradients per second.  The batch
    runs the Hamiltonian matvec once over all its states
    (LUCJGradient.value_and_grad_batch); one vector at a time beside it.  The
    directional derivative of one vector is checked against central finite
    differences of the complex128 energy (h = 1e-5)."""
    import numpy as np
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300.gradient import LUCJGradient

    norb, nelec, L, R, B = 12, (6, 6), 3, 24, args.batch
    rng = np.random.default_rng(2026)
    n = f.UCJOpSpinBalanced.n_params(norb, L)
    base = f.random.random_ucj_op_spin_balanced(norb, n_reps=L, diag_coulomb_normal=True,
                                                diag_coulomb_scale=0.1, seed=2026).to_parameters()
    batch = base[None, :] + 0.05 * rng.normal(size=(B, n))
    ham = f.random.random_df_hamiltonian_normal(norb, rank=R, seed=2027)
    ev = LUCJGradient(norb, nelec, dtype=torch.complex64, workers=args.grad_workers)
    for row in batch[:2]:
        ev.value_and_grad(row, L, ham)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grads = [ev.value_and_grad(row, L, ham)[1] for row in batch]
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    ev.value_and_grad_batch(batch, L, ham)  # warm: buffers and tables of the batch shape
    torch.cuda.synchronize()
    times = []
    for _ in range(max(args.steps, 1)):
        t0 = time.perf_counter()
        _, gb = ev.value_and_grad_batch(batch, L, ham)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t_batch = statistics.median(times)
    same = max(float(np.max(np.abs(gb[i] - grads[i]))) for i in range(B))
    # accuracy: directional derivative against FD of the complex128 energy
    d = rng.normal(size=n)
    d /= np.linalg.norm(d)
    h = 1e-5

    def e128(p):
        op = f.UCJOpSpinBalanced.from_parameters(p, norb=norb, n_reps=L)
        return f.lucj_energy(op, ham, norb, nelec, dtype=torch.complex128)

    fd = (e128(batch[0] + h * d) - e128(batch[0] - h * d)) / (2 * h)
    rel = abs(gb[0] @ d - fd) / abs(fd)
    print(json.dumps({
        "metric": "LUCJ energy+gradient evals/s norb=12 (6,6) n_reps=3 rank 24 (complex64, FP64 reductions)",
        "value": B / t_batch, "unit": "evals/s", "batch": B, "lanes": args.grad_workers, "n_params": n, "dtype": "c64",
        "ms_per_batch": 1e3 * t_batch, "sequential_evals_per_s": B / t_seq,
        "max_abs_diff_batched_vs_sequential": same,
        "fd_check": {"h": h, "directional_rel_err": rel, "bar": 1e-4},
        "data": "synthetic (seeded UCJ parameters near a random operator; Haar term rotations)"}), flush=True)


def run_serve(args) -> None:
    """Serving workload: Poisson arrivals of LUCJ energy (80%) and gradient
    (20%) requests, norb uniform over {8,10,12,14,16} at half filling,
    n_reps in {1,2,3}, DF rank 2*norb (one Hamiltonian per norb); p50/p99
    latency and served evaluations per second."""
    import torch

    from ffsim_gb300.serving import LUCJServer, latency_stats, replay, synthetic_stream

    offsets, reqs = synthetic_stream(args.requests, rate=args.rate, seed=2026)
    # warm the shapes (plans, string tables, kernels) outside the measurement
    warm = LUCJServer(workers=1, max_batch=2)
    _, wreqs = synthetic_stream(15, rate=1e6, seed=7)
    for r in wreqs:
        warm.submit(r)
    warm.drain(len(wreqs))
    warm.close()
    del warm
    torch.cuda.empty_cache()
    torch.cuda.synchronize()
    srv = LUCJServer(workers=args.workers, max_batch=args.max_batch, resident=not args.no_resident)
    res = replay(srv, offsets, reqs)
    srv.close()
    st = latency_stats(res)
    n_grad = sum(r.kind == "gradient" for r in reqs)
    by_norb, errors = {}, {}
    for r, q in zip(res, reqs):
        if r.ok:
            by_norb.setdefault(q.norb, []).append(r.latency)
        else:
            key = f"{type(r.error).__name__} ({q.kind}, norb {q.norb})"
            e = errors.setdefault(key, {"count": 0, "first": str(r.error)[:200]})
            e["count"] += 1
    print(json.dumps({
        "metric": "LUCJ serving evals/s, mixed norb {8..16} half filling, n_reps {1,2,3}, 80% energy / 20% "
                  "gradient, Poisson arrivals; p50/p99 ms",
        "value": st["evals_per_s"], "unit": "evals/s", "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
        "requests": len(reqs), "completed": st["completed"], "gradients": n_grad,
        "arrival_rate_per_s": args.rate, "workers": args.workers, "max_batch": args.max_batch,
        "resident": not args.no_resident, "oom_retries": srv.oom_retries,
        "allocator": os.environ.get("PYTORCH_ALLOC_CONF", os.environ.get("PYTORCH_CUDA_ALLOC_CONF", "")),
        "mean_batch": statistics.mean(srv.batch_sizes), "max_concurrent": srv.max_concurrent,
        "span_s": st["span_s"], "resident_served": srv.resident_served,
        "p50_ms_by_norb": {m: 1e3 * statistics.median(v) for m, v in sorted(by_norb.items())},
        "errors": errors,
        "dtype": "c64", "sample": f"{len(reqs)} requests of the stream (seed 2026)",
        "data": "synthetic"}), flush=True)


def run_resident(args) -> None:
    """Small-shape energies through the resident kernel against the batch
    path: norb=--norb (default 8) at half filling, n_reps=2, one DF
    Hamiltonian of rank 2*norb; --requests requests submitted at once, then
    collected (evaluations per second from the first submission to the last
    result, p50/p99 latency); the batch path evaluates the same operators in
    batches of --max-batch (BatchLUCJEnergy), and one at a time (LUCJEnergy)."""
    import numpy as np
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300.resident import ResidentEvaluator

    norb = args.norb if args.norb != NORB else 8
    nelec = (norb // 2, norb - norb // 2)
    n = args.requests
    ham = f.random.random_df_hamiltonian_normal(norb, rank=2 * norb, seed=17)
    ops = [f.random.random_ucj_op_spin_balanced(norb, n_reps=2, diag_coulomb_normal=True, diag_coulomb_scale=0.1,
                                                seed=100 + i) for i in range(n)]
    ev = ResidentEvaluator(n_slots=max(n, 16), n_ctas=args.resident_ctas, idle_seconds=2.0)
    ev.energies(ops[:16], ham, nelec)  # plans, kernel launch and Hamiltonian upload outside the timing
    t0 = time.perf_counter()
    tickets = [(ev.submit(op, ham, nelec), time.perf_counter()) for op in ops]
    lat, energies = [], []
    for t, t_sub in tickets:
        energies.append(ev.wait(t))
        lat.append(time.perf_counter() - t_sub)
    t1 = time.perf_counter()
    ev.close()
    res_rate = n / (t1 - t0)
    batch = f.BatchLUCJEnergy(norb, nelec, args.max_batch)
    batch(ops[: args.max_batch], ham)
    torch.cuda.synchronize()
    b0 = time.perf_counter()
    eb = []
    for i in range(0, n, args.max_batch):
        eb.extend(batch(ops[i:i + args.max_batch], ham))
    torch.cuda.synchronize()
    b1 = time.perf_counter()
    single = f.LUCJEnergy(norb, nelec)
    m = min(n, 64)
    s0 = time.perf_counter()
    for op in ops[:m]:
        single(op, ham)
    torch.cuda.synchronize()
    s1 = time.perf_counter()
    e128 = [f.lucj_energy(op, ham, norb, nelec, dtype=torch.complex128) for op in ops[:8]]
    # gradients: the resident kernel (the chain rule on the host at collection)
    # against LUCJGradient's batch path, on the same parameter vectors
    from ffsim_gb300.gradient import LUCJGradient

    m_grad = min(n, 256)
    params = [op.to_parameters() for op in ops[:m_grad]]
    ev = ResidentEvaluator(n_slots=max(m_grad, 16), n_ctas=args.resident_ctas, idle_seconds=2.0)
    ev.wait_grad(ev.submit_grad(params[0], 2, ham, nelec))
    g0 = time.perf_counter()
    gt = [ev.submit_grad(p, 2, ham, nelec) for p in params]
    grads = [ev.wait_grad(t)[1] for t in gt]
    g1 = time.perf_counter()
    ev.close()
    lg = LUCJGradient(norb, nelec)
    lg.value_and_grad_batch(np.stack(params[: args.max_batch]), 2, ham)
    torch.cuda.synchronize()
    b2 = time.perf_counter()
    gb = []
    for i in range(0, m_grad, args.max_batch):
        gb.extend(lg.value_and_grad_batch(np.stack(params[i:i + args.max_batch]), 2, ham)[1])
    torch.cuda.synchronize()
    b3 = time.perf_counter()
    lg.close()
    grad_rel = max(float(np.linalg.norm(a - b) / np.linalg.norm(b)) for a, b in zip(grads, gb))
    print(json.dumps({
        "metric": f"resident-kernel LUCJ energy evals/s, norb={norb} {nelec}, n_reps=2, DF rank {2 * norb}",
        "value": res_rate, "unit": "evals/s", "requests": n, "ctas": args.resident_ctas,
        "p50_ms": 1e3 * float(np.median(lat)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
        "batch_path_evals_per_s": n / (b1 - b0), "batch_states": args.max_batch,
        "single_path_evals_per_s": m / (s1 - s0),
        "max_abs_dE_vs_c128": float(max(abs(a - b) for a, b in zip(energies[:8], e128))),
        "max_abs_dE_vs_batch_c64": float(np.max(np.abs(np.array(energies) - np.array(eb)))),
        "gradient": {"resident_evals_per_s": m_grad / (g1 - g0), "batch_path_evals_per_s": m_grad / (b3 - b2),
                     "requests": m_grad, "max_rel_diff_vs_batch_path": grad_rel},
        "dtype": "c64", "data": "synthetic"}), flush=True)


def time_served(ucj_seed: int, n_requests: int, workers: int, max_batch: int) -> dict:
    """Served complex64 LUCJ energies of the metric's workload (norb=16, (8,8),
    n_reps=2, one rank-32 Hamiltonian) through the serving loop, every request
    submitted at once (the server saturated): evaluations per second from the
    first submission to the last result, with p50/p99 latency."""
    import numpy as np
    import torch

    import ffsim_gb300 as f
    from ffsim_gb300.serving import LUCJServer, Request, latency_stats

    ham = f.random.random_df_hamiltonian_normal(NORB, rank=RANK, seed=ucj_seed + 1)
    base = f.random.random_ucj_op_spin_balanced(NORB, n_reps=N_REPS, diag_coulomb_normal=True,
                                                diag_coulomb_scale=0.1, seed=ucj_seed).to_parameters()
    rng = np.random.default_rng(ucj_seed)
    srv = LUCJServer(workers=workers, max_batch=max_batch)
    warm = [Request(-1 - i, "energy", NORB, NELEC, N_REPS, base, ham) for i in range(max_batch)]
    for r in warm:
        srv.submit(r)
    srv.drain(len(warm))
    torch.cuda.synchronize()
    srv._results.clear()
    srv.batch_sizes.clear()
    reqs = [Request(i, "energy", NORB, NELEC, N_REPS, base + 0.01 * rng.normal(size=base.size), ham)
            for i in range(n_requests)]
    t0 = time.perf_counter()
    for r in reqs:
        srv.submit(r)
    res = srv.drain(n_requests)
    t1 = time.perf_counter()
    srv.close()
    del srv
    torch.cuda.empty_cache()
    st = latency_stats(res)
    return {"value": n_requests / (t1 - t0), "unit": "evals/s", "requests": n_requests, "workers": workers,
            "max_batch": max_batch, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
            "completed": st["completed"]}


def cpu_reference_sample(threads: int | None = None):
    """Time the C restatement of the reference on one orbital rotation and one
    diag-Coulomb evolution at norb=16 (complex128) and extrapolate one LUCJ
    energy evaluation: (L+1) rotations + L evolutions + (R+1) DF terms, each term
    2 rotations + 1 contraction (about one evolution's cost)."""
    import numpy as np

    from oracle import cpu_ref, ffsim_oracle as o

    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    cpu_ref.lib()
    cpu_ref.init_cache(NORB, NELEC)
    d = o.dim(NORB, NELEC)
    rng = np.random.default_rng(5)
    vec = (rng.standard_normal(d) + 1j * rng.standard_normal(d)) / math.sqrt(2 * d)
    u = o.random_unitary(NORB, seed=rng)
    j = o.random_symmetric_normal(NORB, scale=0.1, seed=rng)
    t0 = time.perf_counter()
    w = cpu_ref.apply_orbital_rotation(vec, u, NORB, NELEC)
    t1 = time.perf_counter()
    cpu_ref.apply_diag_coulomb_evolution(w, j, -1.0, NORB, NELEC)
    t2 = time.perf_counter()
    t_rot, t_dc = t1 - t0, t2 - t1
    t_eval = (N_REPS + 1) * t_rot + N_REPS * t_dc + (RANK + 1) * (2 * t_rot + t_dc)
    return t_eval, t_rot, t_dc


def run_reference(args, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    samples, step_s = [], []
    t_rot = t_dc = None
    for k in range(args.warmup + args.steps):
        t_eval, t_rot, t_dc = cpu_reference_sample(cores)
        if k >= args.warmup:
            samples.append(t_eval)
            step_s.append(t_rot + t_dc)
    t = statistics.median(samples)
    val = 1.0 / t
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        # a step is the bounded sample (one rotation + one evolution); the
        # evaluation time it extrapolates to is ms_per_eval
        "ms_per_step": 1e3 * statistics.median(step_s), "ms_per_eval": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": run_config(world, args.batch_states),
        "cpu_baseline": {"value": val, "unit": "evals/s", "cores": cores, "kind": "port",
                         "sample": f"one orbital rotation ({t_rot:.2f} s) + one diag-Coulomb evolution "
                                   f"({t_dc:.2f} s) at norb=16 complex128 per step, extrapolated to "
                                   f"{N_REPS + 1} rotations + {N_REPS} evolutions + {RANK + 1} DF terms"},
        "e2e": {"value": val, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def replica_max_ms(local_ms: float, dist, device: str) -> float:
    """The slowest replica's time: the job ends when every rank has finished
    its K steps (a max all-reduce; the only collective, none on the data path)."""
    if dist is None:
        return float(local_ms)
    import torch

    t = torch.tensor([float(local_ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, steps: int, max_ms: float) -> float:
    """Whole-job evaluations per second: every replica runs its own `steps`
    evaluations (weak scaling), timed by the slowest one."""
    return world * steps / (max_ms * 1e-3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--c128-steps", type=int, default=2)
    ap.add_argument("--ops", action="store_true", help="per-operation GB/s lines instead of the energy metric")
    ap.add_argument("--norb", type=int, default=NORB, help="--ops: orbitals (half filling)")
    ap.add_argument("--dtype", default="c64", choices=["c64", "c128"], help="--ops: state dtype")
    ap.add_argument("--reps", type=int, default=5, help="--ops: timed repetitions per op")
    ap.add_argument("--op", default="", help="--ops: only the ops whose name contains this text")
    ap.add_argument("--profile-eval", action="store_true",
                    help="two single evaluations at --norb, untimed (for a profiler's launch list)")
    ap.add_argument("--grad", action="store_true", help="gradient workload (norb=12, batch of parameters)")
    ap.add_argument("--batch", type=int, default=64, help="--grad: parameter vectors")
    ap.add_argument("--grad-workers", type=int, default=4, help="--grad: host lanes (streams) of a batch")
    ap.add_argument("--serve", action="store_true", help="serving workload (mixed requests, Poisson arrivals)")
    ap.add_argument("--resident", action="store_true",
                    help="small-shape energies through the resident kernel (--norb, --requests, --max-batch)")
    ap.add_argument("--resident-ctas", type=int, default=8, help="--resident: CTAs of the resident kernel")
    ap.add_argument("--no-resident", action="store_true",
                    help="--serve: every request through the batch path (no resident kernel)")
    ap.add_argument("--requests", type=int, default=300, help="--serve: requests")
    ap.add_argument("--rate", type=float, default=4.0, help="--serve: mean arrivals per second")
    ap.add_argument("--workers", type=int, default=2, help="--serve: batches in flight")
    ap.add_argument("--max-batch", type=int, default=16, help="--serve: states per batch")
    ap.add_argument("--served", type=int, default=8, help="norb-16 requests of the served measurement (0: skip)")
    ap.add_argument("--batch-states", type=int, default=4, help="evaluations per step (one batch)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.serve and "PYTORCH_ALLOC_CONF" not in os.environ and "PYTORCH_CUDA_ALLOC_CONF" not in os.environ:
        # engines of many shapes come and go: expandable segments let the
        # caching allocator return a released engine's pages to the device
        # instead of keeping partly used segments
        os.environ["PYTORCH_ALLOC_CONF"] = "expandable_segments:True"
    if args.ops:
        run_ops(args)
        return
    if args.profile_eval:
        run_profile_eval(args)
        return
    if args.grad:
        run_grad(args)
        return
    if args.resident:
        run_resident(args)
        return
    if args.serve:
        run_serve(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    from ffsim_gb300 import _lib

    lib = _lib.load()
    ucj, ham = make_inputs(2026 + rank)
    stream = torch.cuda.Stream()

    # complex64 batches of B evaluations: the headline (a step is one batch)
    B = args.batch_states
    ops = make_batch_ops(2026 + rank, B, ucj)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    n0 = lib.ffgb_launch_count()
    t_wall0 = time.perf_counter()
    times64, energies64 = time_batch_energy(torch.complex64, args.steps, args.warmup, ops, ham, stream)
    t_wall1 = time.perf_counter()
    launches = (lib.ffgb_launch_count() - n0) // (args.steps + args.warmup)
    clk = clocks.stop()
    barrier()
    total_ms = replica_max_ms(sum(times64), dist, "cuda")
    value = replica_throughput(world, args.steps * B, total_ms)

    # one evaluation per step (LUCJEnergy), the complex128 path on the same GPU
    times1, energies1 = time_energy(torch.complex64, args.steps, args.warmup, ucj, ham, stream)
    times128, energies128 = time_energy(torch.complex128, args.c128_steps, 1, ucj, ham, stream)
    e64, e64_single, e128 = float(energies64[0]), energies1[-1], energies128[-1]

    # end to end through the public API (host inputs, energies read back each step)
    e2e_s = time_batch_e2e(max(2, min(args.steps, 5)), ops, ham)
    h2d = sum(np.asarray(x).nbytes for o in ops for x in (o.diag_coulomb_mats, o.orbital_rotations)) + sum(
        np.asarray(x).nbytes for x in (ham.one_body_tensor, ham.diag_coulomb_mats, ham.orbital_rotations))

    # served through the continuous-batching loop (the same workload, saturated)
    served = time_served(2026 + rank, args.served, workers=2, max_batch=4) if args.served > 0 else None

    # dominant kernel roofline
    st = stage_rooflines(stream)
    traffic, traffic_src = window_stage_traffic()
    moved, moved_src = eval_bytes_moved()
    # the complex128 path against the measured FP64 FMA rate
    fp = np.zeros(2)
    lib.ffgb_debug_fma_rate(1, _lib.dptr(fp[:1]), stream.cuda_stream)
    lib.ffgb_debug_fma_rate(0, _lib.dptr(fp[1:]), stream.cuda_stream)
    rot128_ms = time_rotation_c128(stream)
    S = st["S"]
    peak, peak_kind = _peaks()
    gbs = 2 * S / (st["window_stage_ms"] * 1e-3) / 1e9
    eval_bytes = (6 * N_REPS + 3 * (RANK + 1)) * S
    win_flops = window_stage_flops(NORB, NELEC[0]) * math.comb(NORB, NELEC[1])

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            t_eval, t_rot, t_dc = cpu_reference_sample(os.cpu_count())
            cpu = {"value": 1.0 / t_eval, "unit": "evals/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"C/OpenMP restatement of the reference kernels: one orbital rotation "
                             f"({t_rot:.2f} s) + one diag-Coulomb evolution ({t_dc:.2f} s) at norb=16 "
                             f"complex128, extrapolated to one evaluation "
                             f"({N_REPS + 1} rotations + {N_REPS} evolutions + {RANK + 1} DF terms)"}
        except Exception as exc:  # noqa: BLE001
            cpu = {"value": None, "unit": "evals/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {exc!r}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": run_config(world, args.batch_states),
            "batch_states": B,
            "p50_ms": statistics.median(times64),
            "p99_ms": float(np.percentile(times64, 99)),
            "energy_c64": e64, "energy_c128": e128, "abs_dE_c64_vs_c128": abs(e64 - e128),
            "energy_c64_single": e64_single, "abs_dE_c64_single_vs_c128": abs(e64_single - e128),
            "single": {"value": 1e3 / statistics.mean(times1), "unit": "evals/s",
                       "ms_per_step": statistics.mean(times1), "p50_ms": statistics.median(times1),
                       "p99_ms": float(np.percentile(times1, 99)), "steps": len(times1),
                       "note": "one evaluation per step (LUCJEnergy), the final UCJ rotation merged into every term"},
            "c128": {"value": 1e3 / statistics.mean(times128), "unit": "evals/s",
                     "ms_per_step": statistics.mean(times128), "steps": len(times128),
                     "bound": "fp64",
                     "fp64_peak_tflops": fp[0], "fp64_peak_kind": "measured in-run (FMA-chain kernel, CUDA events)",
                     "rotation_ms": rot128_ms, "rotation_tflops": rotation_flops(NORB, NELEC) / rot128_ms / 1e9,
                     "rotation_frac_of_fp64": rotation_flops(NORB, NELEC) / rot128_ms / 1e9 / fp[0]},
            "fp32_peak_tflops": fp[1],
            "served": served,
            "e2e": {"value": world * B / e2e_s, "unit": "evals/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": 8 * B},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                         "frac": gbs / peak, "traffic": traffic, "traffic_source": traffic_src,
                         # the window stage is bound by FP32 as much as by HBM: its
                         # Givens network's FMA work against the measured FP32 rate
                         "fp32_tflops": win_flops / (st["window_stage_ms"] * 1e-3) / 1e12,
                         "fp32_frac": (win_flops / (st["window_stage_ms"] * 1e-3) / 1e12 / fp[1]) if fp[1] else None,
                         "kernel": "win_class_kernel: one 8-orbital window stage (one launch per electron-count "
                                   "class), 2 S algorithmic bytes",
                         "algorithmic_bytes": 2 * S, "ms": st["window_stage_ms"],
                         "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "others": {
                             "cross_half_stage": {"ms": st["cross_half_stage_ms"],
                                                  "GB/s": 2 * S / (st["cross_half_stage_ms"] * 1e-3) / 1e9},
                             "orbital_rotation": {"ms": st["rotation_ms"], "algorithmic_bytes": 4 * S,
                                                  "GB/s": 4 * S / (st["rotation_ms"] * 1e-3) / 1e9},
                             "energy_eval": {"ms": total_ms / args.steps / B, "algorithmic_bytes": eval_bytes,
                                             "bytes_moved_single": moved, "bytes_moved_source": moved_src,
                                             "GB/s": B * eval_bytes / (total_ms / args.steps * 1e-3) / 1e9,
                                             "frac": B * eval_bytes / (total_ms / args.steps * 1e-3) / 1e9 / peak}}},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
            "wall_s_c64": t_wall1 - t_wall0,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
