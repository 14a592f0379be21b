"""ffsim_gb300: the statevector gate path of ffsim on one GB300 GPU.

Drop-in counterparts of ``ffsim.apply_orbital_rotation``,
``ffsim.apply_diag_coulomb_evolution``, ``ffsim.apply_num_op_sum_evolution``,
``ffsim.apply_unitary`` for ``UCJOpSpinBalanced``,
``ffsim.linear_operator`` for ``DoubleFactorizedHamiltonian`` and
``ffsim.simulate_trotter_double_factorized``, running
hand-written sm_103a kernels through the C ABI in ``include/ffsim_gb300.h``.
"""

from ffsim_gb300 import contract, linalg, random, states
from ffsim_gb300._state import dim, dims
from ffsim_gb300.basic_gates import (
    Spin,
    apply_fsim_gate,
    apply_fswap_gate,
    apply_givens_rotation,
    apply_hop_gate,
    apply_num_interaction,
    apply_num_num_interaction,
    apply_num_op_prod_interaction,
    apply_on_site_interaction,
    apply_quad_ham_evolution,
    apply_tunneling_interaction,
    pair_for_spin,
)
from ffsim_gb300.bitstring import (
    BitstringType,
    addresses_to_strings,
    bitstring_to_occupied_orbitals,
    strings_to_addresses,
)
from ffsim_gb300.energy import BatchLUCJEnergy, LUCJEnergy, lucj_energies, lucj_energy
from ffsim_gb300.resident import ResidentEvaluator
from ffsim_gb300.gradient import LUCJGradient, lucj_energy_autograd
from ffsim_gb300.gates import (
    apply_diag_coulomb_evolution,
    apply_givens_rotation_in_place,
    apply_num_op_sum_evolution,
    apply_orbital_rotation,
    apply_phase_shift_in_place,
)
from ffsim_gb300.multireference import multireference_state
from ffsim_gb300.hamiltonians import DiagonalCoulombHamiltonian, DoubleFactorizedHamiltonian, MolecularHamiltonian
from ffsim_gb300.protocols import (
    LinearOperator,
    SupportsApplyUnitary,
    SupportsApproximateEquality,
    SupportsDiagonal,
    SupportsLinearOperator,
    SupportsTrace,
    apply_unitary,
    approx_eq,
    diag,
    linear_operator,
    trace,
)
from ffsim_gb300.rdm import rdms
from ffsim_gb300.states import (
    hartree_fock_state,
    init_cache,
    slater_determinant,
    slater_determinant_amplitudes,
    slater_determinant_rdms,
    spin_square,
    spinful_to_spinless_rdm1,
    spinful_to_spinless_rdm2,
    spinful_to_spinless_vec,
    vdot,
)
from ffsim_gb300.trotter import simulate_trotter_diag_coulomb_split_op, simulate_trotter_double_factorized
from ffsim_gb300.wick import expectation_one_body_power, expectation_one_body_product
from ffsim_gb300.variational import (
    GivensAnsatzOp,
    HopGateAnsatzOperator,
    NumNumAnsatzOpSpinBalanced,
    UCJAnglesOpSpinBalanced,
    UCJOpSpinBalanced,
    UCJOpSpinless,
    UCJOpSpinUnbalanced,
)

__all__ = [
    "LUCJGradient",
    "lucj_energy_autograd",
    "DiagonalCoulombHamiltonian",
    "DoubleFactorizedHamiltonian",
    "GivensAnsatzOp",
    "HopGateAnsatzOperator",
    "NumNumAnsatzOpSpinBalanced",
    "LUCJEnergy",
    "BatchLUCJEnergy",
    "ResidentEvaluator",
    "LinearOperator",
    "MolecularHamiltonian",
    "UCJAnglesOpSpinBalanced",
    "UCJOpSpinBalanced",
    "UCJOpSpinUnbalanced",
    "UCJOpSpinless",
    "BitstringType",
    "Spin",
    "SupportsApplyUnitary",
    "SupportsApproximateEquality",
    "SupportsDiagonal",
    "SupportsLinearOperator",
    "SupportsTrace",
    "addresses_to_strings",
    "bitstring_to_occupied_orbitals",
    "strings_to_addresses",
    "apply_diag_coulomb_evolution",
    "apply_fsim_gate",
    "apply_fswap_gate",
    "apply_givens_rotation",
    "apply_hop_gate",
    "apply_num_interaction",
    "apply_num_num_interaction",
    "apply_num_op_prod_interaction",
    "apply_on_site_interaction",
    "apply_quad_ham_evolution",
    "apply_tunneling_interaction",
    "pair_for_spin",
    "apply_givens_rotation_in_place",
    "apply_num_op_sum_evolution",
    "apply_orbital_rotation",
    "apply_phase_shift_in_place",
    "apply_unitary",
    "approx_eq",
    "rdms",
    "simulate_trotter_diag_coulomb_split_op",
    "simulate_trotter_double_factorized",
    "contract",
    "diag",
    "dim",
    "dims",
    "expectation_one_body_power",
    "expectation_one_body_product",
    "hartree_fock_state",
    "init_cache",
    "linalg",
    "linear_operator",
    "multireference_state",
    "lucj_energy",
    "lucj_energies",
    "random",
    "slater_determinant",
    "slater_determinant_amplitudes",
    "slater_determinant_rdms",
    "spin_square",
    "spinful_to_spinless_rdm1",
    "spinful_to_spinless_rdm2",
    "spinful_to_spinless_vec",
    "states",
    "trace",
    "vdot",
]
