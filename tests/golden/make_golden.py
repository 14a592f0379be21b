"""Generate golden vectors by running the reference's own Python code.

Run in a container that has the ffsim source tree (read-only) at
``FFSIM_REF`` (required: the root of the ffsim source tree)::

    FFSIM_REF=/path/to/ffsim python tests/golden/make_golden.py

The reference package cannot be imported whole here: its Rust extension
``ffsim._lib`` is not built (no Rust toolchain) and ``pyscf`` / ``jax`` are not
installed.  This script therefore loads the individual reference modules on
the hot path from their source files and satisfies their imports with:

* ``ffsim._lib`` -> the reference's own pure-Python kernel restatements in
  ``python/ffsim/_slow/`` (which the reference's tests assert equal to the
  Rust kernels), plus a one-line phase shift (``src/gates/phase_shift.rs``)
  and the oracle's restatement of ``givens_decomposition`` (Rust-only in the
  reference; pinned separately by reconstruction and determinant checks);
* ``pyscf.fci.cistring`` -> ``make_strings`` / ``gen_occslst`` restated from
  their combinatorial definition (subsets of the orbital list in colexicographic
  order of positions, which gives ascending integers for ``range(norb)``), and
  ``str2addr`` / ``addrs2str`` / ``strs2addr`` as lookups in those tables;
* ``jax`` / ``opt_einsum`` / ``pyscf.ci`` / ``pyscf.fci.direct_nosym`` /
  ``pyscf.fci.direct_uhf``, the FermionOperator names, the two-body
  contraction and the single-factorized Hamiltonian -> inert placeholders
  (imported by the loaded modules, never called by the cases here).

Everything above the kernels -- reshapes, transposes, the ``s.conjugate()``
convention, pair slices, diagonal halving, ``None`` handling, linear operator
composition, UCJ rotation merging, and the Hamiltonian, ansatz, decomposition,
random, Slater, bitstring, gate and Wick modules -- is the reference's own
code.  The outputs are written to ``tests/golden/golden.npz``; each new group
of cases uses its own seed, so regenerating leaves earlier arrays unchanged.
"""

from __future__ import annotations

import importlib.util
import itertools
import math
import os
import sys
import types
from pathlib import Path

# Reproducible summation order, and so every output bit: one BLAS thread, and a
# fixed string-hash seed (einsum's contraction-path search iterates sets of
# index letters).  The hash seed only takes effect at start-up, so re-execute.
for _var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
    os.environ.setdefault(_var, "1")
if __name__ == "__main__" and os.environ.get("PYTHONHASHSEED") != "0":
    os.environ["PYTHONHASHSEED"] = "0"
    os.execv(sys.executable, [sys.executable, *sys.argv])

import numpy as np  # noqa: E402
import scipy.linalg  # noqa: E402

if "FFSIM_REF" not in os.environ:
    raise SystemExit("set FFSIM_REF to the root of an ffsim source checkout "
                     "(the directory holding python/ffsim), e.g. FFSIM_REF=/path/to/ffsim python make_golden.py")
REF = Path(os.environ["FFSIM_REF"])
PKG = REF / "python" / "ffsim"
HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import ffsim_oracle as orc  # noqa: E402  (givens restatement only)


def _module(name: str, attrs: dict | None = None, is_pkg: bool = False):
    mod = types.ModuleType(name)
    if is_pkg:
        mod.__path__ = []
    for k, v in (attrs or {}).items():
        setattr(mod, k, v)
    sys.modules[name] = mod
    parent, _, child = name.rpartition(".")
    if parent and parent in sys.modules:
        setattr(sys.modules[parent], child, mod)
    return mod


def _load(name: str, relpath: str):
    spec = importlib.util.spec_from_file_location(name, PKG / relpath)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    parent, _, child = name.rpartition(".")
    if parent in sys.modules:
        setattr(sys.modules[parent], child, mod)
    return mod


# ---- pyscf.fci.cistring (combinatorial definition) -------------------------


def _make_strings(orb_list, nocc):
    orb_list = list(orb_list)
    m = len(orb_list)
    if nocc == 0:
        return np.asarray([0], dtype=np.int64)
    if nocc > m:
        return np.asarray([], dtype=np.int64)
    subsets = sorted(
        itertools.combinations(range(m), nocc), key=lambda c: sum(1 << p for p in c)
    )
    return np.asarray(
        [sum(1 << int(orb_list[p]) for p in c) for c in subsets], dtype=np.int64
    )


def _gen_occslst(orb_list, nocc):
    strings = _make_strings(orb_list, nocc)
    occ = [[i for i in range(64) if (int(s) >> i) & 1] for s in strings]
    return np.asarray(occ, dtype=np.int32).reshape(len(strings), nocc)


def _str2addr(norb, nocc, string):
    """Address of a bitstring: its rank among the ascending strings of its popcount."""
    return int(np.searchsorted(_make_strings(range(norb), nocc), int(string)))


def _addrs2str(norb, nelec, addrs):
    return _make_strings(range(norb), nelec)[np.asarray(addrs, dtype=np.int64)]


def _strs2addr(norb, nelec, strings):
    return np.searchsorted(_make_strings(range(norb), nelec), np.asarray(strings, dtype=np.int64)).astype(np.int32)


def install_stubs():
    _module("pyscf", is_pkg=True)
    _module("pyscf.fci", is_pkg=True)
    _module("pyscf.fci.cistring", {"make_strings": _make_strings, "gen_occslst": _gen_occslst,
                                   "str2addr": _str2addr, "addrs2str": _addrs2str, "strs2addr": _strs2addr})
    _module("pyscf.ci", is_pkg=True)
    jax = _module("jax", {"config": types.SimpleNamespace(update=lambda *a, **k: None)})
    jax.numpy = _module("jax.numpy")
    if importlib.util.find_spec("opt_einsum") is None:
        _module("opt_einsum", {"contract": np.einsum})

    ffsim = _module("ffsim", is_pkg=True)
    ffsim.__path__ = [str(PKG)]
    # _slow kernels (reference's own restatements of the Rust kernels)
    _module("ffsim.gates", is_pkg=True)
    _module("ffsim.gates.basic_gates", {"_apply_phase_shift": None})
    slow_orb = _load("ffsim_slow_orb", "_slow/gates/orbital_rotation.py")
    slow_dc = _load("ffsim_slow_dc", "_slow/gates/diag_coulomb.py")
    slow_nos = _load("ffsim_slow_nos", "_slow/gates/num_op_sum.py")
    slow_cdc = _load("ffsim_slow_cdc", "_slow/contract/diag_coulomb.py")
    slow_cnos = _load("ffsim_slow_cnos", "_slow/contract/num_op_sum.py")

    def apply_phase_shift_in_place(vec, phase, indices):
        vec[indices] *= phase

    lib = _module(
        "ffsim._lib",
        {
            "apply_givens_rotation_in_place": slow_orb.apply_givens_rotation_in_place_slow,
            "apply_phase_shift_in_place": apply_phase_shift_in_place,
            "apply_num_op_sum_evolution_in_place": slow_nos.apply_num_op_sum_evolution_in_place_slow,
            "apply_diag_coulomb_evolution_in_place_num_rep": slow_dc.apply_diag_coulomb_evolution_in_place_num_rep_slow,
            "apply_diag_coulomb_evolution_in_place_z_rep": slow_dc.apply_diag_coulomb_evolution_in_place_z_rep_slow,
            "contract_diag_coulomb_into_buffer_num_rep": slow_cdc.contract_diag_coulomb_into_buffer_num_rep_slow,
            "contract_diag_coulomb_into_buffer_z_rep": slow_cdc.contract_diag_coulomb_into_buffer_z_rep_slow,
            "contract_num_op_sum_spin_into_buffer": slow_cnos.contract_num_op_sum_spin_into_buffer_slow,
            "givens_decomposition": lambda mat, tol=1e-12: orc.givens_decomposition(mat, tol),
        },
    )
    _module("ffsim.linalg", is_pkg=True)
    givens = types.SimpleNamespace()
    sys.modules["ffsim.linalg"].givens_decomposition = lambda mat, tol=1e-12: lib.givens_decomposition(
        np.asarray(mat, dtype=complex), tol
    )
    del givens
    _load("ffsim._cistring", "_cistring.py")
    _load("ffsim.states_dimensions", "states/dimensions.py")
    gor = _load("ffsim.gates.orbital_rotation", "gates/orbital_rotation.py")
    gdc = _load("ffsim.gates.diag_coulomb", "gates/diag_coulomb.py")
    gnos = _load("ffsim.gates.num_op_sum", "gates/num_op_sum.py")
    sys.modules["ffsim.gates"].apply_orbital_rotation = gor.apply_orbital_rotation
    sys.modules["ffsim.gates"].apply_diag_coulomb_evolution = gdc.apply_diag_coulomb_evolution
    sys.modules["ffsim.gates"].apply_num_op_sum_evolution = gnos.apply_num_op_sum_evolution
    _module("ffsim.contract", is_pkg=True)
    cdc = _load("ffsim.contract.diag_coulomb", "contract/diag_coulomb.py")
    cnos = _load("ffsim.contract.num_op_sum", "contract/num_op_sum.py")
    _load("ffsim.linalg.util", "linalg/util.py")
    pred = _load("ffsim.linalg.predicates", "linalg/predicates.py")
    sys.modules["ffsim.linalg"].is_real_symmetric = pred.is_real_symmetric
    sys.modules["ffsim.linalg"].is_unitary = pred.is_unitary
    _module("ffsim.variational", is_pkg=True)
    _load("ffsim.variational.util", "variational/util.py")
    proto = _module("ffsim.protocols", is_pkg=True)
    proto.SupportsApplyUnitary = type("SupportsApplyUnitary", (), {})
    proto.SupportsApproximateEquality = type("SupportsApproximateEquality", (), {})
    ffsim.gates = sys.modules["ffsim.gates"]
    ffsim.linalg = sys.modules["ffsim.linalg"]
    ffsim.protocols = proto
    ucj = _load("ffsim.variational.ucj_spin_balanced", "variational/ucj_spin_balanced.py")
    ucju = _load("ffsim.variational.ucj_spin_unbalanced", "variational/ucj_spin_unbalanced.py")
    ucjs = _load("ffsim.variational.ucj_spinless", "variational/ucj_spinless.py")
    giv = _load("ffsim.variational.givens", "variational/givens.py")
    # Trotter: the reference's step iterator and double-factorized evolution
    # (the Hamiltonian class is only a type annotation there)
    _module("ffsim.hamiltonians", {"DoubleFactorizedHamiltonian": types.SimpleNamespace,
                                   "DiagonalCoulombHamiltonian": types.SimpleNamespace})
    _module("ffsim.trotter", is_pkg=True)
    _load("ffsim.trotter._util", "trotter/_util.py")
    tdf = _load("ffsim.trotter.double_factorized", "trotter/double_factorized.py")
    tsplit = _load("ffsim.trotter.diagonal_coulomb_split_op", "trotter/diagonal_coulomb_split_op.py")
    # the diagonal Coulomb Hamiltonian dataclass itself: its FermionOperator
    # methods (Rust-backed) are never called, so the operator names are inert
    for name in ("SupportsDiagonal", "SupportsFermionOperator", "SupportsLinearOperator"):
        setattr(proto, name, type(name, (), {}))
    _module("ffsim.operators", {k: None for k in ("FermionOperator", "cre_a", "cre_b", "des_a", "des_b")})
    if "ffsim.states" not in sys.modules:
        _module("ffsim.states", is_pkg=True)
    _load("ffsim.states.dimensions", "states/dimensions.py")
    dch = _load("ffsim.hamiltonians.diagonal_coulomb_hamiltonian", "hamiltonians/diagonal_coulomb_hamiltonian.py")
    # the molecular and double-factorized Hamiltonian dataclasses and the
    # explicit double factorization; pyscf's make_hdiag and the two-body
    # contraction (pyscf-backed) are never called
    _module("pyscf.fci.direct_nosym", {"make_hdiag": None})
    _module("pyscf.fci.direct_uhf", {"make_hdiag": None})
    _module("ffsim.contract.two_body", {"two_body_linop": None, "two_body_linop_unrestricted": None})
    sys.modules["ffsim.operators"].FermionAction = None
    ldf = _load("ffsim.linalg.double_factorized_decomposition", "linalg/double_factorized_decomposition.py")
    sys.modules["ffsim.linalg"].double_factorized = ldf.double_factorized
    sys.modules["ffsim.linalg"].double_factorized_t2 = ldf.double_factorized_t2
    mol = _load("ffsim.hamiltonians.molecular_hamiltonian", "hamiltonians/molecular_hamiltonian.py")
    dfh = _load("ffsim.hamiltonians.double_factorized_hamiltonian", "hamiltonians/double_factorized_hamiltonian.py")
    # the seeded random constructors, over the real dataclasses
    for name, cls in [("DiagonalCoulombHamiltonian", dch.DiagonalCoulombHamiltonian),
                      ("DoubleFactorizedHamiltonian", dfh.DoubleFactorizedHamiltonian),
                      ("MolecularHamiltonian", mol.MolecularHamiltonian)]:
        setattr(sys.modules["ffsim.hamiltonians"], name, cls)
    for name, cls in [("UCJOpSpinBalanced", ucj.UCJOpSpinBalanced), ("UCJOpSpinUnbalanced", ucju.UCJOpSpinUnbalanced),
                      ("UCJOpSpinless", ucjs.UCJOpSpinless)]:
        setattr(sys.modules["ffsim.variational"], name, cls)
    rnd = _load("ffsim.random_module", "random/random.py")
    sys.modules["ffsim.linalg"].one_hot = _load("ffsim.linalg.linalg", "linalg/linalg.py").one_hot
    _load("ffsim.states.bitstring", "states/bitstring.py")
    slater = _load("ffsim.states.slater", "states/slater.py")
    spin_mod = _load("ffsim.states.spin", "states/spin.py")
    bits = sys.modules["ffsim.states.bitstring"]
    bg = _load("ffsim.gates.basic_gates", "gates/basic_gates.py")
    qh = _load("ffsim.gates.quad_ham", "gates/quad_ham.py")
    sys.modules["ffsim.gates"].apply_hop_gate = bg.apply_hop_gate
    nn = _load("ffsim.variational.num_num", "variational/num_num.py")
    hop = _load("ffsim.variational.hopgate", "variational/hopgate.py")
    # multireference states: the single-factorized Hamiltonian, product states
    # and the FermionOperator conversion it imports are never called here
    _module("ffsim.hamiltonians.single_factorized_hamiltonian", {"SingleFactorizedHamiltonian": type("SF", (), {})})
    _module("ffsim.operators.fermion_operator", {"_fermion_operator_to_linear_operator": None})
    _load("ffsim.protocols.apply_unitary_protocol", "protocols/apply_unitary_protocol.py")
    _load("ffsim.protocols.linear_operator_protocol", "protocols/linear_operator_protocol.py")
    sys.modules["ffsim.states"].slater_determinant = slater.slater_determinant
    sys.modules["ffsim.states"].ProductStateSum = types.SimpleNamespace
    mref = _load("ffsim.variational.multireference", "variational/multireference.py")
    proto.apply_unitary = sys.modules["ffsim.protocols.apply_unitary_protocol"].apply_unitary
    proto.approx_eq = _load("ffsim.protocols.approximate_equality_protocol",
                            "protocols/approximate_equality_protocol.py").approx_eq
    angles = _load("ffsim.variational.ucj_angles_spin_balanced", "variational/ucj_angles_spin_balanced.py")
    wick = _load("ffsim.states.wick", "states/wick.py")
    return types.SimpleNamespace(
        random=rnd,
        bitstring=bits,
        Spin=spin_mod.Spin,
        basic_gates=bg,
        apply_quad_ham_evolution=qh.apply_quad_ham_evolution,
        NumNumAnsatzOpSpinBalanced=nn.NumNumAnsatzOpSpinBalanced,
        HopGateAnsatzOperator=hop.HopGateAnsatzOperator,
        multireference_state=mref.multireference_state,
        UCJAnglesOpSpinBalanced=angles.UCJAnglesOpSpinBalanced,
        wick=wick,
        slater=slater,
        double_factorized_t2=ldf.double_factorized_t2,
        orbital_rotation_from_t1_amplitudes=sys.modules["ffsim.variational.util"].orbital_rotation_from_t1_amplitudes,
        modified_cholesky=ldf.modified_cholesky,
        double_factorized=ldf.double_factorized,
        MolecularHamiltonian=mol.MolecularHamiltonian,
        DoubleFactorizedHamiltonian=dfh.DoubleFactorizedHamiltonian,
        simulate_trotter_double_factorized=tdf.simulate_trotter_double_factorized,
        simulate_trotter_diag_coulomb_split_op=tsplit.simulate_trotter_diag_coulomb_split_op,
        DiagonalCoulombHamiltonian=dch.DiagonalCoulombHamiltonian,
        apply_orbital_rotation=gor.apply_orbital_rotation,
        apply_diag_coulomb_evolution=gdc.apply_diag_coulomb_evolution,
        apply_num_op_sum_evolution=gnos.apply_num_op_sum_evolution,
        contract_diag_coulomb=cdc.contract_diag_coulomb,
        diag_coulomb_linop=cdc.diag_coulomb_linop,
        contract_num_op_sum=cnos.contract_num_op_sum,
        num_op_sum_linop=cnos.num_op_sum_linop,
        zero_one_subspace_indices=gor._zero_one_subspace_indices,
        one_subspace_indices=gor._one_subspace_indices,
        UCJOpSpinBalanced=ucj.UCJOpSpinBalanced,
        UCJOpSpinUnbalanced=ucju.UCJOpSpinUnbalanced,
        UCJOpSpinless=ucjs.UCJOpSpinless,
        GivensAnsatzOp=giv.GivensAnsatzOp,
    )


def df_matvec(ref, one_body, dcm, rots, constant, norb, nelec, z_rep):
    """Body of DoubleFactorizedHamiltonian._linear_operator_
    (hamiltonians/double_factorized_hamiltonian.py:244-275) over the
    reference's own linear operators."""
    eigs, vecs = scipy.linalg.eigh(one_body)
    num_linop = ref.num_op_sum_linop(eigs, norb, nelec, orbital_rotation=vecs)
    linops = [
        ref.diag_coulomb_linop(m, norb, nelec, orbital_rotation=u, z_representation=z_rep)
        for m, u in zip(dcm, rots)
    ]

    def matvec(vec):
        vec = vec.astype(complex, copy=False)
        result = constant * vec
        result += num_linop @ vec
        for linop in linops:
            result += linop @ vec
        return result

    return matvec


def main():
    ref = install_stubs()
    rng = np.random.default_rng(20260603)
    out: dict[str, np.ndarray] = {}

    # pair / occupied index subsets
    for norb, nocc, orbs in [(5, 2, (1, 2)), (5, 3, (3, 2)), (6, 3, (0, 1)), (4, 2, (2, 3))]:
        key = f"zero_one_{norb}_{nocc}_{orbs[0]}{orbs[1]}"
        out[key] = np.asarray(ref.zero_one_subspace_indices(norb, nocc, orbs), dtype=np.int64)
    for norb, nocc, i in [(5, 2, 0), (5, 3, 4), (6, 3, 2)]:
        out[f"one_{norb}_{nocc}_{i}"] = np.asarray(
            ref.one_subspace_indices(norb, nocc, (i,)), dtype=np.int64
        )

    # orbital rotations
    cases = [(5, (3, 2)), (5, (2, 3)), (6, (3, 3)), (4, (3, 2)), (3, (2, 1)), (2, (1, 1)),
             (1, (1, 0)), (1, (0, 1)), (2, (2, 2)), (7, (3, 4))]
    for idx, (norb, nelec) in enumerate(cases):
        d = orc.dim(norb, nelec)
        vec = orc.random_state_vector(d, seed=rng)
        ua = orc.random_unitary(norb, seed=rng)
        ub = orc.random_unitary(norb, seed=rng)
        out[f"rot{idx}_in"] = vec
        out[f"rot{idx}_ua"] = ua
        out[f"rot{idx}_ub"] = ub
        out[f"rot{idx}_same"] = ref.apply_orbital_rotation(vec, ua, norb, nelec)
        out[f"rot{idx}_pair"] = ref.apply_orbital_rotation(vec, (ua, ub), norb, nelec)
        out[f"rot{idx}_aonly"] = ref.apply_orbital_rotation(vec, (ua, None), norb, nelec)
        out[f"rot{idx}_bonly"] = ref.apply_orbital_rotation(vec, (None, ub), norb, nelec)
    out["rot_cases"] = np.asarray([[n, a, b] for n, (a, b) in cases])

    # spinless rotation
    vec = orc.random_state_vector(math.comb(6, 2), seed=rng)
    u = orc.random_unitary(6, seed=rng)
    out["rotsl_in"], out["rotsl_u"] = vec, u
    out["rotsl_out"] = ref.apply_orbital_rotation(vec, u, 6, 2)

    # diag-Coulomb evolution, number and Z representations, with rotations
    dc_cases = [(5, (3, 2)), (4, (2, 2)), (6, (3, 2)), (3, (1, 2))]
    for idx, (norb, nelec) in enumerate(dc_cases):
        d = orc.dim(norb, nelec)
        vec = orc.random_state_vector(d, seed=rng)
        jaa = orc.random_symmetric_normal(norb, scale=0.7, seed=rng)
        jab = rng.standard_normal((norb, norb))
        jbb = orc.random_symmetric_normal(norb, scale=0.7, seed=rng)
        t = float(rng.uniform(-2, 2))
        u = orc.random_unitary(norb, seed=rng)
        out[f"dc{idx}_in"], out[f"dc{idx}_jaa"], out[f"dc{idx}_jab"] = vec, jaa, jab
        out[f"dc{idx}_jbb"], out[f"dc{idx}_t"], out[f"dc{idx}_u"] = jbb, np.asarray(t), u
        out[f"dc{idx}_num"] = ref.apply_diag_coulomb_evolution(vec, (jaa, jab, jbb), t, norb, nelec)
        out[f"dc{idx}_z"] = ref.apply_diag_coulomb_evolution(
            vec, (jaa, jab, jbb), t, norb, nelec, z_representation=True
        )
        out[f"dc{idx}_single"] = ref.apply_diag_coulomb_evolution(vec, jaa, t, norb, nelec)
        out[f"dc{idx}_none"] = ref.apply_diag_coulomb_evolution(vec, (None, jab, None), t, norb, nelec)
        out[f"dc{idx}_rot"] = ref.apply_diag_coulomb_evolution(
            vec, (jaa, jab, jbb), t, norb, nelec, orbital_rotation=u
        )
        out[f"dc{idx}_zrot"] = ref.apply_diag_coulomb_evolution(
            vec, jaa, t, norb, nelec, orbital_rotation=u, z_representation=True
        )
        # contractions
        out[f"dc{idx}_cnum"] = ref.contract_diag_coulomb(vec, (jaa, jab, jbb), norb, nelec)
        out[f"dc{idx}_cz"] = ref.contract_diag_coulomb(
            vec, (jaa, jab, jbb), norb, nelec, z_representation=True
        )
        out[f"dc{idx}_csingle"] = ref.contract_diag_coulomb(vec, jaa, norb, nelec)
        out[f"dc{idx}_linop"] = ref.diag_coulomb_linop(jaa, norb, nelec, orbital_rotation=u) @ vec
    out["dc_cases"] = np.asarray([[n, a, b] for n, (a, b) in dc_cases])

    # spinless diag-Coulomb
    vec = orc.random_state_vector(math.comb(5, 2), seed=rng)
    j = orc.random_symmetric_normal(5, seed=rng)
    out["dcsl_in"], out["dcsl_j"] = vec, j
    out["dcsl_out"] = ref.apply_diag_coulomb_evolution(vec, j, 0.3, 5, 2)

    # num-op-sum evolution and contraction
    for idx, (norb, nelec) in enumerate([(5, (3, 2)), (4, (1, 3))]):
        d = orc.dim(norb, nelec)
        vec = orc.random_state_vector(d, seed=rng)
        ca = rng.standard_normal(norb)
        cb = rng.standard_normal(norb)
        u = orc.random_unitary(norb, seed=rng)
        t = float(rng.uniform(-2, 2))
        out[f"nos{idx}_in"], out[f"nos{idx}_ca"], out[f"nos{idx}_cb"] = vec, ca, cb
        out[f"nos{idx}_u"], out[f"nos{idx}_t"] = u, np.asarray(t)
        out[f"nos{idx}_pair"] = ref.apply_num_op_sum_evolution(vec, (ca, cb), t, norb, nelec)
        out[f"nos{idx}_rot"] = ref.apply_num_op_sum_evolution(vec, ca, t, norb, nelec, orbital_rotation=u)
        out[f"nos{idx}_bonly"] = ref.apply_num_op_sum_evolution(vec, (None, cb), t, norb, nelec)
        out[f"nos{idx}_contract"] = ref.contract_num_op_sum(vec, ca, norb, nelec)
        out[f"nos{idx}_linop"] = ref.num_op_sum_linop(ca, norb, nelec, orbital_rotation=u) @ vec

    # double-factorized Hamiltonian matvec and energy
    for idx, (norb, nelec, n_terms, z_rep) in enumerate([(4, (2, 2), 3, False), (5, (3, 2), 2, False),
                                                         (4, (2, 1), 2, True)]):
        d = orc.dim(norb, nelec)
        vec = orc.random_state_vector(d, seed=rng)
        g = rng.standard_normal((norb, norb)) + 1j * rng.standard_normal((norb, norb))
        one_body = (g + g.conj().T) / 2
        dcm = np.stack([orc.random_symmetric_normal(norb, seed=rng) for _ in range(n_terms)])
        rots = np.stack([orc.random_unitary(norb, seed=rng) for _ in range(n_terms)])
        const = float(rng.standard_normal())
        mv = df_matvec(ref, one_body, dcm, rots, const, norb, nelec, z_rep)
        hv = mv(vec)
        out[f"df{idx}_in"], out[f"df{idx}_h1"], out[f"df{idx}_dcm"] = vec, one_body, dcm
        out[f"df{idx}_rots"], out[f"df{idx}_const"] = rots, np.asarray(const)
        out[f"df{idx}_z"] = np.asarray(z_rep)
        out[f"df{idx}_hv"] = hv
        out[f"df{idx}_energy"] = np.asarray(np.vdot(vec, hv).real)
    out["df_cases"] = np.asarray([[4, 2, 2, 3], [5, 3, 2, 2], [4, 2, 1, 2]])

    # UCJ spin-balanced apply_unitary (reference dataclass method)
    for idx, (norb, nelec, n_reps, final) in enumerate([(4, (2, 2), 2, False), (5, (3, 2), 1, True),
                                                        (6, (3, 3), 3, False)]):
        d = orc.dim(norb, nelec)
        n_params = n_reps * (norb * (norb + 1) + norb**2) + (norb**2 if final else 0)
        params = rng.uniform(-1, 1, size=n_params)
        op = ref.UCJOpSpinBalanced.from_parameters(
            params, norb=norb, n_reps=n_reps, with_final_orbital_rotation=final
        )
        vec = orc.random_state_vector(d, seed=rng)
        hf = orc.hartree_fock_state(norb, nelec)
        out[f"ucj{idx}_params"] = params
        out[f"ucj{idx}_dcm"] = op.diag_coulomb_mats
        out[f"ucj{idx}_rots"] = op.orbital_rotations
        out[f"ucj{idx}_final"] = (
            op.final_orbital_rotation if final else np.zeros((0, 0), dtype=complex)
        )
        out[f"ucj{idx}_in"] = vec
        out[f"ucj{idx}_out"] = op._apply_unitary_(vec, norb, nelec, copy=True)
        out[f"ucj{idx}_hf_out"] = op._apply_unitary_(hf, norb, nelec, copy=True)
    out["ucj_cases"] = np.asarray([[4, 2, 2, 2, 0], [5, 3, 2, 1, 1], [6, 3, 3, 3, 0]])

    # synthetic configuration 0: norb=8, (4,4), rotation then diag-Coulomb t=0.7
    r0 = np.random.default_rng(0)
    vec = orc.random_state_vector(4900, seed=r0)
    u = orc.random_unitary(8, seed=r0)
    j = orc.random_symmetric_normal(8, scale=0.5, seed=r0)
    mid = ref.apply_orbital_rotation(vec, u, 8, (4, 4))
    out["cfg0_in"], out["cfg0_u"], out["cfg0_j"] = vec, u, j
    out["cfg0_out"] = ref.apply_diag_coulomb_evolution(mid, j, 0.7, 8, (4, 4))

    # reference fixture: tests/python/test_data/orbital_rotation-0.npy on HF (8, (5, 5))
    mat = np.load(REF / "tests" / "python" / "test_data" / "orbital_rotation-0.npy")
    hf = orc.hartree_fock_state(8, (5, 5))
    out["fix_mat"] = mat
    out["fix_out"] = ref.apply_orbital_rotation(hf, mat, 8, (5, 5))

    # double-factorized Trotter evolution (trotter/double_factorized.py:25-127)
    rt = np.random.default_rng(20261204)
    trotter_cases = [(4, (2, 2), 0.3, 2, 0, False), (4, (2, 1), 0.2, 1, 2, True), (5, (3, 2), 0.25, 3, 1, False),
                     (3, (1, 1), 0.1, 2, 1, True)]
    for idx, (norb, nelec, t, n_steps, order, z_rep) in enumerate(trotter_cases):
        d = orc.dim(norb, nelec)
        vec = orc.random_state_vector(d, seed=rt)
        g = rt.standard_normal((norb, norb)) + 1j * rt.standard_normal((norb, norb))
        one_body = (g + g.conj().T) / 2
        n_terms = norb
        dcm = np.stack([orc.random_symmetric_normal(norb, seed=rt) for _ in range(n_terms)])
        rots = np.stack([orc.random_unitary(norb, seed=rt) for _ in range(n_terms)])
        const = float(rt.standard_normal())
        ham = types.SimpleNamespace(one_body_tensor=one_body, diag_coulomb_mats=dcm, orbital_rotations=rots,
                                    constant=const, z_representation=z_rep)
        out[f"trot{idx}_in"], out[f"trot{idx}_h1"], out[f"trot{idx}_dcm"] = vec, one_body, dcm
        out[f"trot{idx}_rots"], out[f"trot{idx}_const"] = rots, np.asarray(const)
        out[f"trot{idx}_out"] = ref.simulate_trotter_double_factorized(
            vec, ham, t, norb=norb, nelec=nelec, n_steps=n_steps, order=order)
    out["trot_cases"] = np.asarray([[n, a, b, t, s, o, int(z)] for n, (a, b), t, s, o, z in trotter_cases])

    # spin-unbalanced and spinless UCJ operators (reference dataclass methods)
    ru = np.random.default_rng(20261205)
    other_cases = [("ucju", 4, (2, 1), 2, False), ("ucju", 5, (2, 2), 1, True), ("ucjs", 4, (2, 2), 2, True),
                   ("ucjs", 5, 2, 2, False)]
    for idx, (kind, norb, nelec, n_reps, final) in enumerate(other_cases):
        cls = ref.UCJOpSpinUnbalanced if kind == "ucju" else ref.UCJOpSpinless
        n_params = cls.n_params(norb, n_reps, with_final_orbital_rotation=final)
        params = ru.uniform(-1, 1, size=n_params)
        op = cls.from_parameters(params, norb=norb, n_reps=n_reps, with_final_orbital_rotation=final)
        d = orc.dim(norb, nelec)
        vec = orc.random_state_vector(d, seed=ru)
        out[f"ucjx{idx}_params"] = params
        out[f"ucjx{idx}_dcm"] = op.diag_coulomb_mats
        out[f"ucjx{idx}_rots"] = op.orbital_rotations
        out[f"ucjx{idx}_in"] = vec
        out[f"ucjx{idx}_out"] = op._apply_unitary_(vec, norb, nelec, copy=True)
    out["ucjx_cases"] = np.asarray([[0 if k == "ucju" else 1, n, *(ne if isinstance(ne, tuple) else (ne, -1)), r,
                                     int(fi)] for k, n, ne, r, fi in other_cases])

    # Givens rotation ansatz (variational/givens.py): from parameters and from a rotation
    rg = np.random.default_rng(20261206)
    giv_cases = [(4, (2, 1), [(0, 1), (2, 3), (1, 2), (0, 1)], True, True),
                 (5, (2, 2), [(1, 2), (3, 4), (0, 1), (2, 3)], False, True),
                 (4, (1, 2), [(2, 3), (1, 2)], True, False)]
    for idx, (norb, nelec, pairs, with_phis, with_angles) in enumerate(giv_cases):
        n = ref.GivensAnsatzOp.n_params(norb, pairs, with_phis=with_phis, with_phase_angles=with_angles)
        params = rg.uniform(-np.pi, np.pi, size=n)
        op = ref.GivensAnsatzOp.from_parameters(params, norb, pairs, with_phis=with_phis,
                                                 with_phase_angles=with_angles)
        vec = orc.random_state_vector(orc.dim(norb, nelec), seed=rg)
        out[f"giv{idx}_params"], out[f"giv{idx}_pairs"] = params, np.asarray(pairs)
        out[f"giv{idx}_rot"] = op.to_orbital_rotation()
        out[f"giv{idx}_in"] = vec
        out[f"giv{idx}_out"] = op._apply_unitary_(vec, norb, nelec, copy=True)
    out["giv_cases"] = np.asarray([[n, a, b, int(p), int(q)] for n, (a, b), _, p, q in giv_cases])
    for norb in (4, 5):
        u = orc.random_unitary(norb, seed=rg)
        op = ref.GivensAnsatzOp.from_orbital_rotation(u)
        out[f"givu{norb}_u"] = u
        out[f"givu{norb}_pairs"] = np.asarray(op.interaction_pairs)
        out[f"givu{norb}_thetas"] = np.asarray(op.thetas)
        out[f"givu{norb}_phis"] = np.asarray(op.phis)
        out[f"givu{norb}_angles"] = np.asarray(op.phase_angles)

    # UCJ parameter maps with restricted interaction pairs (local UCJ)
    rp = np.random.default_rng(20261207)
    pair_cases = [
        ("bal", 4, 2, ([(0, 0), (1, 1), (0, 1), (2, 3)], [(0, 0), (1, 2), (3, 3)]), True),
        ("bal", 5, 1, (None, [(p, p) for p in range(5)]), False),
        ("unb", 4, 2, ([(0, 1), (2, 2)], [(1, 0), (0, 1), (3, 2)], None), True),
        ("unb", 4, 1, ([], [(2, 2)], [(0, 3)]), False),
        ("sl", 4, 2, [(0, 0), (1, 3), (2, 3)], True),
    ]
    for idx, (kind, norb, n_reps, pairs, final) in enumerate(pair_cases):
        cls = {"bal": ref.UCJOpSpinBalanced, "unb": ref.UCJOpSpinUnbalanced, "sl": ref.UCJOpSpinless}[kind]
        n = cls.n_params(norb, n_reps, interaction_pairs=pairs, with_final_orbital_rotation=final)
        params = rp.uniform(-1, 1, size=n)
        op = cls.from_parameters(params, norb=norb, n_reps=n_reps, interaction_pairs=pairs,
                                 with_final_orbital_rotation=final)
        out[f"pairs{idx}_params"] = params
        out[f"pairs{idx}_dcm"] = op.diag_coulomb_mats
        out[f"pairs{idx}_rots"] = op.orbital_rotations
        out[f"pairs{idx}_to"] = op.to_parameters(interaction_pairs=pairs)

    # diagonal Coulomb Hamiltonian: linear operator and diagonal
    # (hamiltonians/diagonal_coulomb_hamiltonian.py:67-97,208-238), and its
    # split-operator Trotter evolution (trotter/diagonal_coulomb_split_op.py:25-122).
    # Case 0 of the evolution is a 1-D Fermi-Hubbard chain with hopping 1,
    # interaction 4, chemical potential 0.5 and nearest-neighbour repulsion 0.3.
    rd = np.random.default_rng(20261208)
    dch_cases = [(4, (2, 2)), (5, (3, 1)), (6, (2, 3)), (3, (0, 2))]
    for idx, (norb, nelec) in enumerate(dch_cases):
        g = rd.standard_normal((norb, norb)) + 1j * rd.standard_normal((norb, norb))
        one_body = (g + g.conj().T) / 2
        dcm = np.stack([orc.random_symmetric_normal(norb, seed=rd), orc.random_symmetric_normal(norb, seed=rd)])
        const = float(rd.standard_normal())
        ham = ref.DiagonalCoulombHamiltonian(one_body, dcm, constant=const)
        vec = orc.random_state_vector(orc.dim(norb, nelec), seed=rd)
        out[f"dch{idx}_h1"], out[f"dch{idx}_dcm"], out[f"dch{idx}_const"] = one_body, dcm, np.asarray(const)
        out[f"dch{idx}_in"] = vec
        out[f"dch{idx}_matvec"] = ham._linear_operator_(norb, nelec) @ vec
        out[f"dch{idx}_diag"] = ham._diag_(norb, nelec)
    out["dch_cases"] = np.asarray([[n, a, b] for n, (a, b) in dch_cases])

    split_cases = [(4, (2, 2), 0.5, 3, 0), (4, (2, 1), 0.3, 2, 1), (5, (2, 2), 0.4, 1, 2), (3, (1, 2), 0.2, 2, 0)]
    for idx, (norb, nelec, t, n_steps, order) in enumerate(split_cases):
        if idx == 0:
            one_body = np.zeros((norb, norb), dtype=complex)
            for p in range(norb - 1):
                one_body[p, p + 1] = one_body[p + 1, p] = -1.0
            one_body -= 0.5 * np.eye(norb)
            aa = np.zeros((norb, norb))
            for p in range(norb - 1):
                aa[p, p + 1] = aa[p + 1, p] = 0.3
            ab = 4.0 * np.eye(norb) + aa
            dcm, const = np.stack([aa, ab]), 0.0
        else:
            g = rd.standard_normal((norb, norb)) + 1j * rd.standard_normal((norb, norb))
            one_body = (g + g.conj().T) / 2
            dcm = np.stack([orc.random_symmetric_normal(norb, seed=rd), orc.random_symmetric_normal(norb, seed=rd)])
            const = float(rd.standard_normal())
        ham = ref.DiagonalCoulombHamiltonian(one_body, dcm, constant=const)
        vec = orc.random_state_vector(orc.dim(norb, nelec), seed=rd)
        out[f"split{idx}_h1"], out[f"split{idx}_dcm"], out[f"split{idx}_const"] = one_body, dcm, np.asarray(const)
        out[f"split{idx}_in"] = vec
        out[f"split{idx}_out"] = ref.simulate_trotter_diag_coulomb_split_op(
            vec, ham, t, norb=norb, nelec=nelec, n_steps=n_steps, order=order)
    out["split_cases"] = np.asarray([[n, a, b, t, s, o] for n, (a, b), t, s, o in split_cases])

    # double factorization of molecular two-body tensors
    # (linalg/double_factorized_decomposition.py:70-309), the conversions of
    # hamiltonians/double_factorized_hamiltonian.py:140-242 and
    # MolecularHamiltonian.rotated (molecular_hamiltonian.py:119-144).  The
    # tensors are sums of L (x) L over real symmetric L: positive
    # semidefinite with the symmetries of molecular integrals.
    rm = np.random.default_rng(20261209)
    mol_norbs = [3, 4, 5]
    for idx, norb in enumerate(mol_norbs):
        g = rm.standard_normal((norb, norb))
        one_body = (g + g.T) / 2
        ls = [(x + x.T) / 2 for x in rm.standard_normal((norb + 1, norb, norb))]
        two_body = sum(np.einsum("pq,rs->pqrs", x, x) for x in ls)
        const = float(rm.standard_normal())
        mol = ref.MolecularHamiltonian(one_body, two_body, constant=const)
        out[f"mol{idx}_h1"], out[f"mol{idx}_h2"], out[f"mol{idx}_const"] = one_body, two_body, np.asarray(const)
        out[f"mol{idx}_chol"] = ref.modified_cholesky(two_body.reshape(norb**2, norb**2), tol=1e-8)
        out[f"mol{idx}_chol_max2"] = ref.modified_cholesky(two_body.reshape(norb**2, norb**2), tol=1e-8, max_vecs=2)
        for tag, kw in [("c", {}), ("c3", {"max_vecs": 3}), ("e", {"cholesky": False}),
                        ("e3", {"cholesky": False, "max_vecs": 3})]:
            mats, rots = ref.double_factorized(two_body, tol=1e-8, **kw)
            out[f"mol{idx}_df{tag}_mats"], out[f"mol{idx}_df{tag}_rots"] = mats, rots
        for z in (False, True):
            df = ref.DoubleFactorizedHamiltonian.from_molecular_hamiltonian(mol, z_representation=z)
            out[f"mol{idx}_from{int(z)}_h1"] = df.one_body_tensor
            out[f"mol{idx}_from{int(z)}_const"] = np.asarray(df.constant)
            out[f"mol{idx}_from{int(z)}_mats"] = df.diag_coulomb_mats
            back = df.to_molecular_hamiltonian()
            out[f"mol{idx}_back{int(z)}_h1"], out[f"mol{idx}_back{int(z)}_h2"] = back.one_body_tensor, back.two_body_tensor
        u = orc.random_unitary(norb, seed=rm)
        rot = mol.rotated(u)
        out[f"mol{idx}_u"], out[f"mol{idx}_rot_h1"], out[f"mol{idx}_rot_h2"] = u, rot.one_body_tensor, rot.two_body_tensor
    out["mol_cases"] = np.asarray(mol_norbs)

    # seeded random constructors (random/random.py): the same seed gives the
    # same inputs here and in the reference
    r = ref.random
    out["rnd_density"] = r.random_density_matrix(4, seed=1)
    out["rnd_orth"] = r.random_orthogonal(5, seed=2)
    out["rnd_sorth"] = r.random_special_orthogonal(5, seed=3)
    out["rnd_herm"] = r.random_hermitian(4, seed=4)
    out["rnd_antiherm"] = r.random_antihermitian(4, seed=5)
    out["rnd_tbt"] = r.random_two_body_tensor(3, seed=6)
    out["rnd_tbt_real_r2"] = r.random_two_body_tensor(3, rank=2, seed=7, dtype=float)
    for tag, dt in [("c", complex), ("r", float)]:
        m = r.random_molecular_hamiltonian(3, seed=8, dtype=dt)
        out[f"rnd_mol{tag}_h1"], out[f"rnd_mol{tag}_h2"] = m.one_body_tensor, m.two_body_tensor
        out[f"rnd_mol{tag}_const"] = np.asarray(m.constant)
    for tag, real in [("c", False), ("r", True)]:
        h = r.random_diagonal_coulomb_hamiltonian(4, real=real, seed=9)
        out[f"rnd_dch{tag}_h1"], out[f"rnd_dch{tag}_dcm"] = h.one_body_tensor, h.diag_coulomb_mats
        out[f"rnd_dch{tag}_const"] = np.asarray(h.constant)
        h = r.random_double_factorized_hamiltonian(3, rank=2, real=real, seed=10)
        out[f"rnd_df{tag}_h1"], out[f"rnd_df{tag}_dcm"] = h.one_body_tensor, h.diag_coulomb_mats
        out[f"rnd_df{tag}_rots"], out[f"rnd_df{tag}_const"] = h.orbital_rotations, np.asarray(h.constant)
    h = r.random_double_factorized_hamiltonian(3, seed=11, z_representation=True)
    out["rnd_dfz_rots"] = h.orbital_rotations
    ucj_kw = [dict(n_reps=2, seed=12), dict(n_reps=1, with_final_orbital_rotation=True, diag_coulomb_normal=True,
                                             diag_coulomb_scale=0.3, seed=13)]
    for k, kw in enumerate(ucj_kw):
        for tag, fn in [("bal", r.random_ucj_op_spin_balanced), ("unb", r.random_ucj_op_spin_unbalanced),
                        ("sl", r.random_ucj_op_spinless)]:
            op = fn(4, **kw)
            out[f"rnd_{tag}{k}_dcm"], out[f"rnd_{tag}{k}_rots"] = op.diag_coulomb_mats, op.orbital_rotations
            if op.final_orbital_rotation is not None:
                out[f"rnd_{tag}{k}_final"] = op.final_orbital_rotation
    op = r.random_ucj_op_spin_balanced(4, n_reps=2, interaction_pairs=([(0, 0), (1, 2)], [(0, 0), (3, 3)]), seed=14)
    out["rnd_balp_dcm"] = op.diag_coulomb_mats
    op = r.random_ucj_op_spin_unbalanced(4, interaction_pairs=([(0, 1)], [(2, 0), (1, 1)], []), seed=15)
    out["rnd_unbp_dcm"] = op.diag_coulomb_mats
    op = r.random_ucj_op_spinless(4, interaction_pairs=[(0, 3), (2, 2)], seed=16)
    out["rnd_slp_dcm"] = op.diag_coulomb_mats

    # UCJ from t amplitudes (variational/ucj_spin_balanced.py:377-532) over the
    # explicit t2 factorization (linalg/double_factorized_decomposition.py:467-659)
    t2_cases = [(5, 2, float, 17), (6, 3, float, 18), (5, 2, complex, 19)]
    for idx, (norb, nocc, dt, seed) in enumerate(t2_cases):
        t2 = r.random_t2_amplitudes(norb, nocc, seed=seed, dtype=dt)
        t1 = np.random.default_rng(seed).standard_normal((nocc, norb - nocc))
        out[f"t2{idx}_t2"], out[f"t2{idx}_t1"] = t2, t1
        mats, rots = ref.double_factorized_t2(t2)
        out[f"t2{idx}_mats"], out[f"t2{idx}_rots"] = mats, rots
        mats, rots = ref.double_factorized_t2(t2, max_terms=3)
        out[f"t2{idx}_mats3"] = mats
        out[f"t2{idx}_t1rot"] = ref.orbital_rotation_from_t1_amplitudes(t1)
        for tag, kw in [("a", {}), ("b", {"n_reps": 2, "t1": t1}), ("c", {"n_reps": 40}),
                        ("d", {"interaction_pairs": ([(0, 1), (1, 2)], [(0, 0)]), "n_reps": 3})]:
            op = ref.UCJOpSpinBalanced.from_t_amplitudes(t2, **kw)
            out[f"t2{idx}_op{tag}_dcm"], out[f"t2{idx}_op{tag}_rots"] = op.diag_coulomb_mats, op.orbital_rotations
            vec = orc.random_state_vector(orc.dim(norb, (nocc, nocc)), seed=seed)
            out[f"t2{idx}_op{tag}_in"] = vec
            out[f"t2{idx}_op{tag}_out"] = op._apply_unitary_(vec, norb, (nocc, nocc), copy=True)
    out["t2_cases"] = np.asarray([[n, o, int(d is complex), sd] for n, o, d, sd in t2_cases])

    # Slater determinants (states/slater.py:32-350): state vectors, closed-form
    # RDMs and amplitudes, spinful and spinless, with unsorted orbital lists
    rs = np.random.default_rng(20261210)
    sl = ref.slater
    u, v = orc.random_unitary(5, seed=rs), orc.random_unitary(5, seed=rs)
    out["sl_u"], out["sl_v"] = u, v
    out["sl_vec_plain"] = sl.slater_determinant(5, ([3, 0], [4, 1, 2]))
    out["sl_vec_plain_spinless"] = sl.slater_determinant(5, [2, 4, 0])
    out["sl_vec_rot"] = sl.slater_determinant(5, ([1, 3], [0, 4, 2]), u)
    out["sl_vec_pair"] = sl.slater_determinant(5, ([2, 0], [1]), (u, None))
    out["sl_vec_spinless_rot"] = sl.slater_determinant(5, [4, 1], v)
    for tag, occ, rot in [("a", ([0, 2], [1, 3, 4]), u), ("b", ([1], [0, 3]), (u, v)), ("c", [0, 3, 1], v),
                          ("d", ([0, 1], []), (None, v))]:
        for rank in (1, 2):
            for reorder in (True, False):
                res = sl.slater_determinant_rdms(5, occ, rot, rank=rank, reorder=reorder)
                if rank == 1:
                    out[f"sl_rdm_{tag}_1"] = res
                else:
                    out[f"sl_rdm_{tag}_2_{int(reorder)}"] = res[1]
    out["sl_amp_spinful"] = sl.slater_determinant_amplitudes(([0b00011, 0b10100], [0b01010, 0b11000]), 5,
                                                             ([0, 1], [2, 3]), (u, v))
    out["sl_amp_spinless"] = sl.slater_determinant_amplitudes([0b00111, 0b11010], 5, [0, 2, 4], v)

    # two-orbital gates (gates/basic_gates.py) and quadratic-Hamiltonian
    # evolution (gates/quad_ham.py), every spin selection
    rb = np.random.default_rng(20261211)
    bgm, spins = ref.basic_gates, [ref.Spin.ALPHA, ref.Spin.BETA, ref.Spin.ALPHA_AND_BETA]
    for tag, norb, nelec in [("s", 5, (2, 2)), ("u", 4, (2, 1)), ("l", 5, 3)]:
        vec = orc.random_state_vector(orc.dim(norb, nelec), seed=rb)
        out[f"bg{tag}_in"] = vec
        spin_list = spins if isinstance(nelec, tuple) else [ref.Spin.ALPHA_AND_BETA]
        for k, sp in enumerate(spin_list):
            out[f"bg{tag}_givens{k}"] = bgm.apply_givens_rotation(vec, 0.7, (0, 2), norb, nelec, sp, phi=0.3)
            out[f"bg{tag}_num{k}"] = bgm.apply_num_interaction(vec, 0.9, 1, norb, nelec, sp)
            out[f"bg{tag}_tunnel{k}"] = bgm.apply_tunneling_interaction(vec, 0.4, (3, 1), norb, nelec, sp)
            out[f"bg{tag}_numnum{k}"] = bgm.apply_num_num_interaction(vec, 1.1, (0, 3), norb, nelec, sp)
            out[f"bg{tag}_hop{k}"] = bgm.apply_hop_gate(vec, 0.5, (1, 2), norb, nelec, sp)
            out[f"bg{tag}_fsim{k}"] = bgm.apply_fsim_gate(vec, 0.6, 0.8, (2, 0), norb, nelec, sp)
            out[f"bg{tag}_fswap{k}"] = bgm.apply_fswap_gate(vec, (1, 3), norb, nelec, sp)
        m = rb.standard_normal((norb, norb)) + 1j * rb.standard_normal((norb, norb))
        m = (m + m.conj().T) / 2
        out[f"bg{tag}_qmat"] = m
        out[f"bg{tag}_quad"] = ref.apply_quad_ham_evolution(vec, m, 0.4, norb, nelec)
        if isinstance(nelec, tuple):
            out[f"bg{tag}_quadpair"] = ref.apply_quad_ham_evolution(vec, (m, None), 0.4, norb, nelec)
            out[f"bg{tag}_onsite"] = bgm.apply_on_site_interaction(vec, 0.8, 2, norb, nelec)
            for k, orbs in enumerate([((0, 2), (1,)), ((0, 1, 3), (2, 3)), ((), ()), ((1,), ()), ((0, 1), ()),
                                      ((), (2, 3)), ((0,), (1,)), ((0, 1, 2), ())]):
                out[f"bg{tag}_prod{k}"] = bgm.apply_num_op_prod_interaction(vec, 0.45, orbs, norb, nelec)

    # number-number and hop-gate ansatz operators (variational/num_num.py, hopgate.py)
    ra = np.random.default_rng(20261212)
    nn_pairs = ([(0, 1), (1, 3), (2, 2)], [(0, 0), (1, 2)])
    nn_params = ra.uniform(-1, 1, size=5)
    op = ref.NumNumAnsatzOpSpinBalanced.from_parameters(nn_params, norb=4, interaction_pairs=nn_pairs)
    vec = orc.random_state_vector(orc.dim(4, (2, 1)), seed=ra)
    out["nn_params"], out["nn_in"] = nn_params, vec
    out["nn_mats"] = op.to_diag_coulomb_mats()
    out["nn_out"] = op._apply_unitary_(vec, 4, (2, 1), copy=True)
    hop_pairs = [(0, 1), (2, 3), (1, 2)]
    for k, final in enumerate((False, True)):
        n = 5 + (16 if final else 0)
        params = ra.uniform(-1, 1, size=n)
        op = ref.HopGateAnsatzOperator.from_parameters(params, norb=4, interaction_pairs=hop_pairs,
                                                       with_final_orbital_rotation=final)
        vec = orc.random_state_vector(orc.dim(4, (2, 2)), seed=ra)
        out[f"hop{k}_params"], out[f"hop{k}_in"] = params, vec
        out[f"hop{k}_out"] = op._apply_unitary_(vec, 4, (2, 2), copy=True)
        out[f"hop{k}_to"] = op.to_parameters()

    # multireference state (variational/multireference.py:28-76): a UCJ ansatz on
    # three reference determinants, a double-factorized Hamiltonian's operator
    rmr = np.random.default_rng(20261213)
    ucj = ref.UCJOpSpinBalanced.from_parameters(rmr.uniform(-0.5, 0.5, size=ref.UCJOpSpinBalanced.n_params(4, 2)),
                                                norb=4, n_reps=2)
    g = rmr.standard_normal((4, 4)) + 1j * rmr.standard_normal((4, 4))
    dcm = np.stack([orc.random_symmetric_normal(4, seed=rmr) for _ in range(3)])
    rots = np.stack([orc.random_unitary(4, seed=rmr) for _ in range(3)])
    dfh = ref.DoubleFactorizedHamiltonian((g + g.conj().T) / 2, dcm, rots, constant=0.7)
    occs = [([0, 1], [0, 1]), ([0, 2], [0, 1]), ([0, 1], [1, 3])]
    out["mr_params"] = ucj.to_parameters()
    out["mr_h1"], out["mr_dcm"], out["mr_rots"] = dfh.one_body_tensor, dcm, rots
    for root in (0, 1):
        e, state = ref.multireference_state(dfh._linear_operator_(4, (2, 2)), ucj, occs, 4, (2, 2), root=root)
        out[f"mr{root}_energy"], out[f"mr{root}_state"] = np.asarray(e), state

    # UCJ operator parameterized by gate angles (variational/ucj_angles_spin_balanced.py)
    rua = np.random.default_rng(20261214)
    nn_pairs, giv_pairs = ([(0, 1), (2, 3)], [(0, 0), (1, 1), (0, 2)]), [(0, 1), (2, 3), (1, 2)]
    cls = ref.UCJAnglesOpSpinBalanced
    n = cls.n_params(4, 2, nn_pairs, giv_pairs, with_final_givens_ansatz_op=True)
    params = rua.uniform(-1, 1, size=n)
    op = cls.from_parameters(params, norb=4, n_reps=2, num_num_interaction_pairs=nn_pairs,
                             givens_interaction_pairs=giv_pairs, with_final_givens_ansatz_op=True)
    vec = orc.random_state_vector(orc.dim(4, (2, 2)), seed=rua)
    out["ang_params"], out["ang_in"] = params, vec
    out["ang_out"] = op._apply_unitary_(vec, 4, (2, 2), copy=True)
    out["ang_to"] = op.to_parameters()
    ucj = ref.UCJOpSpinBalanced.from_parameters(rua.uniform(-1, 1, size=ref.UCJOpSpinBalanced.n_params(
        4, 2, with_final_orbital_rotation=True)), norb=4, n_reps=2, with_final_orbital_rotation=True)
    out["ang_ucj_params"] = ucj.to_parameters()
    out["ang_from_ucj_to"] = cls.from_ucj_op(ucj).to_parameters()
    out["ang_from_ucj_out"] = cls.from_ucj_op(ucj)._apply_unitary_(vec, 4, (2, 2), copy=True)

    # Wick's theorem on a Slater determinant (states/wick.py)
    rw = np.random.default_rng(20261215)
    u = orc.random_unitary(6, seed=rw)
    rho = ref.slater.slater_determinant_rdms(6, [0, 2, 3], u)
    mats = [rw.standard_normal((6, 6)) + 1j * rw.standard_normal((6, 6)) for _ in range(4)]
    out["wick_rho"], out["wick_mats"] = rho, np.stack(mats)
    out["wick_prod"] = np.asarray([ref.wick.expectation_one_body_product(rho, mats[:k]) for k in range(5)])
    out["wick_pow"] = np.asarray([ref.wick.expectation_one_body_power(rho, mats[0], k) for k in range(4)])

    # addresses <-> bitstrings (states/bitstring.py:173-361), every representation
    bs = ref.bitstring
    addr_sets = {"s": (5, (2, 3), [0, 7, 42, 99]), "l": (6, 3, [0, 5, 19])}
    for tag, (norb, nelec, addrs) in addr_sets.items():
        out[f"bits{tag}_addrs"] = np.asarray(addrs)
        for t in bs.BitstringType:
            res = bs.addresses_to_strings(addrs, norb, nelec, bitstring_type=t)
            out[f"bits{tag}_{t.name}"] = np.asarray(res)
            if isinstance(nelec, tuple):
                a, b = bs.addresses_to_strings(addrs, norb, nelec, concatenate=False, bitstring_type=t)
                out[f"bits{tag}_{t.name}_a"], out[f"bits{tag}_{t.name}_b"] = np.asarray(a), np.asarray(b)
            back = bs.strings_to_addresses(res, norb, nelec)
            out[f"bits{tag}_{t.name}_back"] = np.asarray(back)

    np.savez_compressed(HERE / "golden.npz", **out)
    print(f"wrote {len(out)} arrays to {HERE / 'golden.npz'}")


if __name__ == "__main__":
    main()
