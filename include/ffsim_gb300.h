/*
 * ffsim_gb300 -- C ABI of the GB300 (sm_103a) statevector gate path.
 *
 * Every entry point takes plain pointers and sizes, never throws, and
 * returns an ffgb_status.  Device pointers are owned by the caller; kernels
 * run asynchronously on the given CUDA stream (cudaStream_t passed as void*,
 * NULL = legacy default stream).  Complex arrays are interleaved
 * (re, im) pairs.  Host matrices are row-major complex128 (norb*norb*2
 * doubles) unless stated otherwise.  State, output and result buffers are
 * never optional (a state has at least one amplitude): NULL for any of them
 * returns FFGB_ERR_ARG before anything is launched; only the arguments
 * documented as "NULL = ..." may be NULL.
 *
 * State layout (identical to ffsim): a spinful state is a C-contiguous
 * (dim_a, dim_b) array; row = alpha string address, column = beta string
 * address; the address of an occupation bitstring is its rank in ascending
 * integer order among bitstrings with the same number of set bits.
 *
 * Scratch: entry points that need device scratch take (scratch,
 * scratch_bytes); ffgb_scratch_bytes() returns the required size.  The
 * library keeps only small per-device lookup tables (occupation strings),
 * created on first use for each (norb, nocc) with a synchronous copy; make
 * the first call for a shape outside stream capture.
 *
 * Reference interfaces replaced (paths inside the ffsim project):
 *   python/ffsim/_lib.pyi:36-123 and src/lib.rs:20-68 (PyO3 module ffsim._lib)
 */
#ifndef FFSIM_GB300_H
#define FFSIM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  FFGB_OK = 0,
  FFGB_ERR_ARG = 1,         /* invalid argument (maps to ValueError) */
  FFGB_ERR_DTYPE = 2,       /* unsupported dtype (TypeError) */
  FFGB_ERR_OOM = 3,         /* scratch too small / allocation failed (MemoryError) */
  FFGB_ERR_CUDA = 4,        /* CUDA runtime error (RuntimeError) */
  FFGB_ERR_TIMEOUT = 5,     /* a batch passed its deadline (TimeoutError) */
  FFGB_ERR_UNSUPPORTED = 6, /* shape not supported (NotImplementedError) */
  FFGB_ERR_NUMERIC = 7,     /* host factorization failed (ArithmeticError) */
  FFGB_ERR_CANCELLED = 8,   /* a batch was cancelled through its control (CancelledError) */
  FFGB_PENDING = 9          /* ffgb_resident_poll: the request has not finished yet (not an error) */
} ffgb_status;

/* Control of a long batch call (a NULL control pointer means none).
 * Between its states' circuits and between Hamiltonian terms the call reads
 * *cancel (when not NULL; written by another host thread) and the elapsed
 * time; it returns FFGB_ERR_CANCELLED once *cancel is nonzero and
 * FFGB_ERR_TIMEOUT once timeout_s seconds have passed since it started
 * (timeout_s <= 0: no deadline).  So that either acts promptly, the call then
 * keeps at most two such units of work queued on the stream ahead of the GPU.
 * After either error the stream stays usable and the outputs are undefined. */
typedef struct {
  const volatile int* cancel;
  double timeout_s;
} ffgb_control;

typedef enum { FFGB_C64 = 0, FFGB_C128 = 1 } ffgb_dtype;

/* Library version (major*10000 + minor*100 + patch). */
int ffgb_version(void);
/* Message of the last error raised on the calling thread ("" if none). */
const char* ffgb_last_error(void);
/* Number of CUDA kernels this library has launched in the process. */
long long ffgb_launch_count(void);
/* Number of device allocations (cudaMalloc, cudaMallocAsync) this library
 * has made in the process: its cached string and stage tables and the
 * temporary buffers of the entry points that take no workspace.  Test and
 * accounting aid; no counterpart in the reference. */
long long ffgb_device_alloc_count(void);
/* Measured fused multiply-add rate of the CUDA cores (TFLOP/s, 2 flops per
 * FMA): FP64 for FFGB_C128, FP32 for FFGB_C64.  Two launches of an
 * FMA-chain kernel over every SM on `stream`, the second timed with CUDA
 * events; about 10-20 ms.  The compute ceiling of the rotation kernels;
 * no counterpart in the reference. */
int ffgb_debug_fma_rate(int dtype, double* tflops, void* stream);

/* ------------------------------------------------------------------ */
/* Host-side linear algebra                                             */
/* ------------------------------------------------------------------ */

/* Givens decomposition U = D G_L^* ... G_1^* of a square unitary.
 * Replaces givens_decomposition (src/linalg/givens.rs:68-149,
 * python/ffsim/linalg/givens.py:59-156 exact path).
 * rot_cs: [n(n-1)/2][3] = (c, Re s, Im s); rot_ij: [n(n-1)/2][2];
 * *n_rot = number written; diag: [n][2]. */
int ffgb_givens_decomposition(const double* mat, int n, double tol, double* rot_cs, int* rot_ij,
                              int* n_rot, double* diag);

/* Hermitian eigendecomposition (ascending eigenvalues; eigenvectors in the
 * columns of vecs, row-major complex).  Host replacement of the
 * scipy.linalg.eigh call in double_factorized_hamiltonian.py:250. */
int ffgb_eigh(const double* mat, int n, double* eigvals, double* vecs);

/* Plan of W(mat) on one spin sector, serialized for inspection/tests:
 * out[0]=kind, out[1]=h, out[2]=max reconstruction error, then the plan
 * coefficients: the sector-kernel networks and phases, then the stage
 * sequence of the stage kernels (windows and cross-half rotations) with its
 * phases.  Returns the number of doubles written in *len. */
int ffgb_debug_plan(const double* mat, int norb, int use_windows, double* out, int cap, int* len);

/* One stage of the complex64 cosine-sine plan of W(mat) on the alpha sector of
 * vec, in place (stage 0/1: first lower/upper window, 2: cross-half pass,
 * 3/4: second lower/upper window).  A diagnostic for timing a single kernel
 * stage; the result alone is not a meaningful state.  No counterpart in the
 * reference. */
int ffgb_debug_stage(void* vec, int dtype, int norb, int n_alpha, int n_beta, const double* mat, int stage,
                     void* stream);

/* Scratch bytes needed by the functions below for a state of the given
 * shape (op: 0 = orbital rotation / evolutions, 1 = linear operator matvec,
 * 2 = expectation / energy, 3 = densities). */
size_t ffgb_scratch_bytes(int op, int dtype, int norb, int n_alpha, int n_beta);

/* ------------------------------------------------------------------ */
/* Gates (in place on vec)                                              */
/* ------------------------------------------------------------------ */

/* One adjacent Givens rotation on one spin sector (spin 0 = alpha rows,
 * 1 = beta columns): for every string pair x (i occupied, j empty) / y:
 * x <- c x + s y, y <- c y - conj(s) x.  Replaces
 * apply_givens_rotation_in_place (src/gates/orbital_rotation.rs:18-104)
 * with pair slices computed on the device.  |i - j| must be 1. */
int ffgb_apply_givens_rotation(void* vec, int dtype, int norb, int n_alpha, int n_beta, int spin,
                               double c, double s_re, double s_im, int i, int j, void* stream);

/* out = a+_{p spin} a_{q spin} vec (a single excitation within one spin
 * sector; out is zeroed first, vec and out must differ).  The building block of
 * the rank-2 reduced density matrices, which the reference computes with pyscf
 * (python/ffsim/states/rdm.py:181-274 via make_rdm12s / trans_rdm12s). */
int ffgb_apply_excitation(const void* vec, void* out, int dtype, int norb, int n_alpha, int n_beta, int spin,
                          int p, int q, void* stream);

/* Multiply every string with orbital orb occupied in one spin sector by
 * phase.  Replaces apply_phase_shift_in_place (src/gates/phase_shift.rs:17-30). */
int ffgb_apply_phase_shift(void* vec, int dtype, int norb, int n_alpha, int n_beta, int spin,
                           double phase_re, double phase_im, int orb, void* stream);

/* Orbital rotation W(mat_a) (x) W(mat_b); either matrix may be NULL (no
 * action on that sector).  Replaces the Python driver
 * python/ffsim/gates/orbital_rotation.py:117-199 and the per-Givens kernels.
 * Spinless systems: n_beta = -1 and mat_b ignored (vec has C(norb, n_alpha)
 * entries). */
int ffgb_apply_orbital_rotation(void* vec, int dtype, int norb, int n_alpha, int n_beta,
                                const double* mat_a, const double* mat_b, void* scratch,
                                size_t scratch_bytes, void* stream);

/* exp(-i t sum J^{st}_ij n_is n_jt / 2) (number representation) or the Z
 * representation, optionally conjugated by orbital rotations (rot_a, rot_b:
 * NULL = none).  mat_aa/mat_ab/mat_bb: real norb*norb row-major, NULL = no
 * interaction of that type.  Replaces
 * apply_diag_coulomb_evolution_in_place_{num,z}_rep
 * (src/gates/diag_coulomb.rs:19-190) and the Python wrapper
 * python/ffsim/gates/diag_coulomb.py:68-275.  Spinless: n_beta = -1. */
int ffgb_apply_diag_coulomb_evolution(void* vec, int dtype, int norb, int n_alpha, int n_beta,
                                      const double* mat_aa, const double* mat_ab,
                                      const double* mat_bb, double time, int z_representation,
                                      const double* rot_a, const double* rot_b, void* scratch,
                                      size_t scratch_bytes, void* stream);

/* exp(-i t sum_i lambda_i n_is), coeffs_a/coeffs_b real norb (NULL = none),
 * optionally conjugated by orbital rotations.  Replaces
 * apply_num_op_sum_evolution_in_place (src/gates/num_op_sum.rs:18-36) and
 * python/ffsim/gates/num_op_sum.py:62-236.  Spinless: n_beta = -1. */
int ffgb_apply_num_op_sum_evolution(void* vec, int dtype, int norb, int n_alpha, int n_beta,
                                    const double* coeffs_a, const double* coeffs_b, double time,
                                    const double* rot_a, const double* rot_b, void* scratch,
                                    size_t scratch_bytes, void* stream);

/* UCJ spin-balanced unitary: for each rep k, W(U_k^dag U_{k-1}) then the
 * diag-Coulomb evolution with (J_aa, J_ab, J_aa) at time -1, then the final
 * rotation W(U_final U_L) (U_final = I when final_rotation is NULL).
 * diag_coulomb_mats: [n_reps][2][norb][norb] real; orbital_rotations:
 * [n_reps][norb][norb] complex.  Replaces UCJOpSpinBalanced._apply_unitary_
 * (python/ffsim/variational/ucj_spin_balanced.py:657-696). */
int ffgb_ucj_spin_balanced_apply(void* vec, int dtype, int norb, int n_alpha, int n_beta,
                                 int n_reps, const double* diag_coulomb_mats,
                                 const double* orbital_rotations, const double* final_rotation,
                                 void* scratch, size_t scratch_bytes, void* stream);

/* ------------------------------------------------------------------ */
/* Contractions and linear operators                                    */
/* ------------------------------------------------------------------ */

/* out (+)= Z vec with Z the diagonal Coulomb operator
 * sum J^{st}_ij n_is n_jt / 2 (number rep.) or its Z representation.
 * Replaces contract_diag_coulomb_into_buffer_{num,z}_rep
 * (src/contract/diag_coulomb.rs:22-174) and
 * python/ffsim/contract/diag_coulomb.py:41-192. */
int ffgb_contract_diag_coulomb(const void* vec, void* out, int dtype, int norb, int n_alpha,
                               int n_beta, const double* mat_aa, const double* mat_ab,
                               const double* mat_bb, int z_representation, int accumulate,
                               void* stream);

/* Size of the fixed device scratch of ffgb_contract_diag_coulomb_static. */
#define FFGB_STATIC_SCRATCH_BYTES (1u << 20)

/* ffgb_contract_diag_coulomb without any device allocation.  No counterpart
 * in the reference: it exists for callers that cannot allocate device memory
 * (all of it is held by another allocator, or cudaMalloc/cudaFree would stall
 * a latency-bound loop).  Same arguments and results as
 * ffgb_contract_diag_coulomb.  Its scratch (occupation strings, 4*dim_a +
 * 4*dim_b bytes, and, when mat_bb is nonzero, a column table of element
 * size * dim_b bytes, each part rounded up to 256 bytes) lives in one
 * FFGB_STATIC_SCRATCH_BYTES array per device;
 * larger shapes return FFGB_ERR_ARG with the byte counts.  Nothing in that
 * array has to start at zero: the call writes every byte it reads.  Calls on
 * one device that overlap in time (different streams or host threads) share
 * the array and race: issue them on one stream or one at a time.  The first
 * call on each device looks up the array's address (cudaGetSymbolAddress),
 * so make it before any stream capture. */
int ffgb_contract_diag_coulomb_static(const void* vec, void* out, int dtype, int norb, int n_alpha,
                                      int n_beta, const double* mat_aa, const double* mat_ab,
                                      const double* mat_bb, int z_representation, int accumulate,
                                      void* stream);

/* out (+)= sum_i lambda_i (n_ia + n_ib) vec.  Replaces
 * contract_num_op_sum_spin_into_buffer (src/contract/num_op_sum.rs:20-39)
 * and python/ffsim/contract/num_op_sum.py:27-72. */
int ffgb_contract_num_op_sum(const void* vec, void* out, int dtype, int norb, int n_alpha,
                             int n_beta, const double* coeffs, int accumulate, void* stream);

/* out (+)= W(rot) Z W(rot)^dag vec, Z = diagonal operator given by
 * (one_body[norb] on n_ia + n_ib) + (mat, z_representation) two-body part
 * (mat may be NULL).  rot may be NULL.  This is one matvec of
 * diag_coulomb_linop / num_op_sum_linop
 * (python/ffsim/contract/diag_coulomb.py:195-272,
 * python/ffsim/contract/num_op_sum.py:75-131). */
int ffgb_rotated_diag_matvec(const void* vec, void* out, int dtype, int norb, int n_alpha,
                             int n_beta, const double* one_body, const double* mat,
                             int z_representation, const double* rot, int accumulate,
                             void* scratch, size_t scratch_bytes, void* stream);

/* Double-factorized Hamiltonian matvec out = H vec with
 * H = sum_pq kappa_pq a^dag a + 1/2 sum_t sum J^(t) n^(t) n^(t) + constant
 * (one_body_tensor complex norb*norb; diag_coulomb_mats [n_terms][norb][norb]
 * real; orbital_rotations [n_terms][norb][norb] complex).  Replaces
 * DoubleFactorizedHamiltonian._linear_operator_ matvec
 * (python/ffsim/hamiltonians/double_factorized_hamiltonian.py:244-275). */
int ffgb_df_matvec(const void* vec, void* out, int dtype, int norb, int n_alpha, int n_beta,
                   const double* one_body_tensor, int n_terms, const double* diag_coulomb_mats,
                   const double* orbital_rotations, double constant, int z_representation,
                   void* scratch, size_t scratch_bytes, void* stream);

/* Energy <vec|H|vec> of the same Hamiltonian, fused: each term rotates the
 * state into its basis and reduces sum_z z |phi|^2 in FP64 without forming
 * H vec.  pre_rotation (NULL = none) is applied to vec before every term
 * (used to merge a circuit's final orbital rotation).  *energy_out is a
 * host double; the call synchronizes the stream.  Matches
 * np.vdot(vec, H @ vec).real (tests/python/variational/ucj_spin_balanced_test.py:152-158). */
int ffgb_df_expectation(const void* vec, int dtype, int norb, int n_alpha, int n_beta,
                        const double* one_body_tensor, int n_terms,
                        const double* diag_coulomb_mats, const double* orbital_rotations,
                        double constant, int z_representation, const double* pre_rotation,
                        double* energy_out, void* scratch, size_t scratch_bytes, void* stream);

/* LUCJ energy from the Hartree-Fock state (or from vec_in when not NULL):
 * applies the UCJ circuit without its last rotation, merges that rotation
 * into every Hamiltonian term and returns <psi|H|psi>.  work_state must hold
 * one state (dim_a*dim_b complex of dtype).  Synchronizes the stream. */
int ffgb_lucj_energy(const void* vec_in, void* work_state, int dtype, int norb, int n_alpha,
                     int n_beta, int n_reps, const double* ucj_diag_coulomb_mats,
                     const double* ucj_orbital_rotations, const double* ucj_final_rotation,
                     const double* one_body_tensor, int n_terms, const double* diag_coulomb_mats,
                     const double* orbital_rotations, double constant, double* energy_out,
                     void* scratch, size_t scratch_bytes, void* stream);

/* ------------------------------------------------------------------ */
/* Batches: n_states states of one shape under one Hamiltonian          */
/* ------------------------------------------------------------------ */
/* Scratch bytes of the batch entry points (op 0: ffgb_batch_lucj_energy,
 * op 1: ffgb_batch_df_matvec) for n_states states; 0 for invalid shapes. */
size_t ffgb_batch_scratch_bytes(int op, int dtype, int norb, int n_alpha, int n_beta, long long n_states);

/* LUCJ energies of n_states parameter sets under one double-factorized
 * Hamiltonian: state b (the UCJ circuit of ucj_diag_coulomb_mats[b],
 * ucj_orbital_rotations[b] and, if not NULL, ucj_final_orbital_rotations[b],
 * applied to the Hartree-Fock state) is built in work_states[b] (n_states
 * contiguous states), then every Hamiltonian term runs once over all the
 * states.  energies_out: n_states host doubles.  Per state it equals
 * ffgb_lucj_energy to rounding.  The reference evaluates such energies one at a
 * time (np.vdot(psi, H @ psi).real, tests/python/variational/
 * ucj_spin_balanced_test.py:152-158; one parameter vector per call in the
 * line searches of python/ffsim/optimize/linear_method.py:181-243); complex64
 * with 9 <= norb <= 16
 * runs the terms on all states at once, other shapes state by state.
 * Arrays are per state, stacked: n_states * n_reps * 2 * norb^2 doubles and
 * n_states * n_reps * norb^2 complex.  Synchronizes the stream. */
int ffgb_batch_lucj_energy(void* work_states, long long n_states, int dtype, int norb, int n_alpha, int n_beta,
                           int n_reps, const double* ucj_diag_coulomb_mats, const double* ucj_orbital_rotations,
                           const double* ucj_final_orbital_rotations, const double* one_body_tensor, int n_terms,
                           const double* diag_coulomb_mats, const double* orbital_rotations, double constant,
                           double* energies_out, void* scratch, size_t scratch_bytes, const ffgb_control* control,
                           void* stream);

/* out[b] = H vec[b] for n_states contiguous states: the double-factorized
 * Hamiltonian's linear operator (python/ffsim/hamiltonians/
 * double_factorized_hamiltonian.py:244-275) applied to the columns of a
 * matrix, as in `hamiltonian @ jac` of python/ffsim/optimize/
 * linear_method.py:294 (SciPy applies the matvec column by column there).  complex64 with 9 <= norb <= 16 runs
 * every term once over all the states; other shapes state by state. */
int ffgb_batch_df_matvec(const void* vec, void* out, long long n_states, int dtype, int norb, int n_alpha,
                         int n_beta, const double* one_body_tensor, int n_terms, const double* diag_coulomb_mats,
                         const double* orbital_rotations, double constant, int z_representation, void* scratch,
                         size_t scratch_bytes, const ffgb_control* control, void* stream);

/* ------------------------------------------------------------------ */
/* Reductions and helpers                                               */
/* ------------------------------------------------------------------ */

/* Transition one-body density out[s][p][q] = <x| a+_{p s} a_{q s} |y> for
 * s = alpha, beta (complex, interleaved re/im; 2*norb*norb complex values; host
 * pointer; synchronizes).  The gradient of the LUCJ energy with respect to an
 * orbital-rotation generator.  Scratch: ffgb_scratch_bytes(3, ...).  The
 * reference computes this on the CPU (python/ffsim/states/rdm.py:73-274 via
 * pyscf's trans_rdm1s); no counterpart on its kernel path. */
int ffgb_transition_rdm1(const void* x, const void* y, int dtype, int norb, int n_alpha, int n_beta,
                         double* out, void* scratch, size_t scratch_bytes, void* stream);

/* Diagonal pair densities <x| n_{i s} n_{j t} |y> for (s, t) = (alpha, alpha),
 * (alpha, beta), (beta, beta): 3*norb*norb complex values (host pointer;
 * synchronizes).  The gradient of the LUCJ energy with respect to the
 * diagonal Coulomb matrices.  Scratch: ffgb_scratch_bytes(3, ...).  No
 * counterpart in the reference. */
int ffgb_pair_density(const void* x, const void* y, int dtype, int norb, int n_alpha, int n_beta, double* out,
                      void* scratch, size_t scratch_bytes, void* stream);

/* Both densities of one gate of the adjoint gradient, into DEVICE memory
 * out_dev, without synchronizing: the transition one-body densities of
 * ffgb_transition_rdm1 (alpha, beta) and, when pair != 0, the pair densities
 * of ffgb_pair_density (aa, ab, bb) after them -- 2 or 5 blocks of
 * norb*norb complex values (interleaved FP64).  One pair of transposes
 * serves both, and the caller reads every gate's densities after one
 * synchronization.  Scratch: ffgb_scratch_bytes(3, ...).  No counterpart in
 * the reference. */
int ffgb_gate_densities(const void* x, const void* y, int dtype, int norb, int n_alpha, int n_beta, int pair,
                        void* out_dev, void* scratch, size_t scratch_bytes, void* stream);

/* out[0..1] = sum conj(x) y in FP64 (host pointer; synchronizes). */
int ffgb_vdot(const void* x, const void* y, int dtype, long long n, double* out, void* stream);

/* vec <- one-hot at address 0 (Hartree-Fock state, states/slater.py:122-138). */
int ffgb_hartree_fock(void* vec, int dtype, long long n, void* stream);

/* ------------------------------------------------------------------ */
/* Resident evaluator: LUCJ energies of small shapes from a work queue.
 *
 * A persistent kernel (one CTA per request at a time, the state in shared
 * memory) evaluates <psi|H|psi> for psi = the spin-balanced UCJ operator
 * applied to Hartree-Fock (python/ffsim/variational/ucj_spin_balanced.py:657-696,
 * states/slater.py:122-138) and H a double-factorized Hamiltonian
 * (hamiltonians/double_factorized_hamiltonian.py:244-275), for norb <= 8, any
 * nelec and n_reps <= 4, in complex64 with FP64 energies.  Requests of
 * different shapes and Hamiltonians share one queue.  The queue lives in
 * host-mapped memory: submit writes a request and publishes it, the kernel's
 * CTAs claim requests in order, and poll reads the result.  A CTA that finds
 * no work for idle_seconds exits; when all have, the kernel's status is
 * FFGB_ERR_TIMEOUT and the next submit (or a poll of an unfinished request)
 * launches it again.  The reference evaluates these energies one call at a
 * time on the CPU; no counterpart in its interface. */
typedef struct ffgb_resident ffgb_resident;

/* Queue of n_slots requests served by n_ctas CTAs on a stream of its own
 * (the calling thread's current device).  Allocates host-mapped memory and a
 * small device block; launches nothing yet. */
int ffgb_resident_open(int n_slots, int n_ctas, double idle_seconds, ffgb_resident** out);
/* Register a double-factorized Hamiltonian (arguments as ffgb_df_expectation;
 * norb <= 8); *ham_id names it in submit.  Synchronous copy to the device. */
int ffgb_resident_hamiltonian(ffgb_resident* r, int norb, const double* one_body, int n_terms, const double* dcm,
                              const double* rots, double constant, int zrep, int* ham_id);
/* Queue the energy of one UCJ operator (arguments as ffgb_lucj_energy; from
 * Hartree-Fock) under Hamiltonian ham_id; *ticket identifies the request.
 * FFGB_ERR_OOM when the request's slot still holds an uncollected result. */
int ffgb_resident_submit(ffgb_resident* r, int ham_id, int norb, int n_alpha, int n_beta, int n_reps,
                         const double* ucj_dcm, const double* ucj_rots, const double* ucj_final, long long* ticket);
/* FFGB_OK with *energy once the request has finished (its slot is then free
 * again), FFGB_PENDING before, FFGB_ERR_CANCELLED if it was cancelled. */
int ffgb_resident_poll(ffgb_resident* r, long long ticket, double* energy);
/* Queue the device part of an adjoint gradient (norb <= 8, n_reps <= 4): the
 * circuit of the merged rotations rots (n_reps + 1 complex norb x norb
 * matrices V_1 .. V_{n_reps+1}: psi = W(V_{L+1}) D_L W(V_L) ... D_1 W(V_1)
 * |HF>) and phase gates D_k = exp(i sum J_k n n / 2) (ucj_dcm as in
 * ffgb_lucj_energy), then lambda = (H - c) psi, the energy, and the gates
 * undone on psi and lambda with the densities of every gate (as
 * ffgb_gate_densities).  The chain rule to the parameters is the caller's
 * (ffsim_gb300.gradient does it on the host).  No counterpart in the
 * reference, which differentiates by finite differences
 * (python/ffsim/optimize/_util.py:60-110). */
int ffgb_resident_submit_grad(ffgb_resident* r, int ham_id, int norb, int n_alpha, int n_beta, int n_reps,
                              const double* rots, const double* ucj_dcm, long long* ticket);
/* Collect a gradient request: *energy and dens[(n_reps + 1) x 5 x norb x
 * norb] complex (per gate j = 1 .. n_reps + 1: the transition one-body
 * densities of the alpha and beta sectors, then the pair densities aa, ab,
 * bb; zero for j = 1).  Return codes as ffgb_resident_poll. */
int ffgb_resident_poll_densities(ffgb_resident* r, long long ticket, double* energy, double* dens);
/* Ask the kernel to stop a request: it checks between gates and terms. */
int ffgb_resident_cancel(ffgb_resident* r, long long ticket);
/* Launch the kernel now if it is not running (it otherwise starts with the
 * first request). */
int ffgb_resident_start(ffgb_resident* r);
/* *running: whether the kernel is running; *kernel_status: FFGB_OK while it
 * runs or after it was stopped, FFGB_ERR_TIMEOUT after it exited because no
 * work came within idle_seconds. */
int ffgb_resident_status(ffgb_resident* r, int* running, int* kernel_status);
/* Stop the kernel (between requests), wait for it and free everything.
 * Results not yet collected are lost. */
int ffgb_resident_close(ffgb_resident* r);

#ifdef __cplusplus
}
#endif

#endif /* FFSIM_GB300_H */
