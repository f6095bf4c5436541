/*
 * tq_sv.h -- C ABI of the tyxonq_gb300 statevector library (libtyxonq_gb300.so).
 *
 * One GB300, one process.  Every entry point takes raw device pointers,
 * plain integers and a CUDA stream (passed as void*, NULL = legacy default
 * stream), enqueues its kernels on that stream and returns without
 * synchronising.  The caller owns every buffer: the library never allocates
 * or frees device memory on these paths.  Buffers that a call needs beyond its
 * inputs and outputs ("workspace") are passed in by the caller; the matching
 * *_workspace_bytes() query gives the size.
 *
 * Return convention: TQ_OK (0) on success, a negative TQ_ERR_* code on
 * failure; tq_last_error() copies a message for the last failure on the
 * calling thread.  Calls are thread-compatible: different threads may use
 * different streams concurrently.
 *
 * Basis ordering is the reference engine's big-endian convention: qubit 0 is
 * the most significant bit of the basis index
 * (tyxonq/libs/quantum_library/kernels/statevector.py:32,49;
 *  tyxonq/devices/simulators/statevector/engine.py:454,1050-1057).
 * Amplitudes are interleaved (re, im): TQ_C64 = float2, TQ_C128 = double2.
 * Matrices are passed as host arrays of doubles, row-major, (re, im)
 * interleaved; multi-qubit matrix indices take the FIRST listed qubit as the
 * most significant bit (statevector.py:53-56, gates.py:265-284).
 */
#ifndef TQ_SV_H
#define TQ_SV_H

#ifndef __CUDACC_RTC__
#include <stddef.h>
#include <stdint.h>
#endif

#if defined(__GNUC__)
#define TQ_API __attribute__((visibility("default")))
#else
#define TQ_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define TQ_C64 0
#define TQ_C128 1

#define TQ_MAX_QUBITS 34
#define TQ_MAX_KQ 5

#define TQ_OK 0
#define TQ_ERR_ARG (-1)
#define TQ_ERR_CUDA (-2)
#define TQ_ERR_RANGE (-3)
#define TQ_ERR_TIMEOUT (-4)
#define TQ_ERR_WORKSPACE (-5)
#define TQ_ERR_UNSUPPORTED (-6)

/* ------------------------------------------------------------ library */

/* Library ABI version (major*100 + minor). */
TQ_API int tq_version(void);

/* Copies the last error message of the calling thread into buf (always
 * NUL-terminated when len > 0).  Returns the last error code. */
TQ_API int tq_last_error(char* buf, size_t len);

/* Checked builds.  The library's checked variant (compiled with -DTQ_CHECKED)
 * guards the device-computed indices of its kernels: a failing check records
 * the first failing site and index and skips the access instead of trapping.
 * tq_check_status writes that site (0: none) and index and clears them; it
 * returns 1 in a checked build and 0 (site 0) in the normal build.  The
 * runtime-compiled kernels are not instrumented. */
#define TQ_SITE_GATE 1        /* single-gate kernels: amplitude index >= 2^n */
#define TQ_SITE_TILE 2        /* tile passes: tile amplitude index >= 2^n */
#define TQ_SITE_WAVE_TILE 3   /* wave items: tile amplitude index >= 2^n of the instance */
#define TQ_SITE_HPSI 4        /* H psi: partner tile or term index out of range */
#define TQ_SITE_SAMPLE 5      /* sampler: resolved index outside the state */
TQ_API int tq_check_status(unsigned* site, long long* index);

/* ------------------------------------------------------------ state preparation */

/* |basis_index> over n qubits.  Replaces init_statevector
 * (tyxonq/libs/quantum_library/kernels/statevector.py:19-25), which builds
 * |0...0>; basis_index generalises it to the Hartree-Fock bitstrings built by
 * get_init_circuit (chem_libs/quantum_chem_library/statevector_ops.py:172-199). */
TQ_API int tq_sv_init_basis(void* psi, int n, int dtype, int64_t basis_index, void* stream);

/* ------------------------------------------------------------ single gates (plain engine) */

/* Dense 2x2 on `qubit`.  Replaces apply_1q_statevector (statevector.py:28-42).
 * u: 8 doubles = [[u00,u01],[u10,u11]] as (re,im) pairs. */
TQ_API int tq_sv_apply_1q(void* psi, int n, int dtype, int qubit, const double* u, void* stream);

/* Diagonal 1q gate diag(d0, d1); d: 4 doubles.  Fast path of
 * apply_1q_statevector for rz/s/sdg/t/tdg/z/phase (gates.py:19-35,68-79,180-200).
 * When d0 == 1 only the |1> half of the state is read and written. */
TQ_API int tq_sv_apply_diag1(void* psi, int n, int dtype, int qubit, const double* d, void* stream);

/* Dense 4x4 on (q0, q1), q0 = high bit of the matrix index.  Replaces
 * apply_2q_statevector (statevector.py:45-59); q0 == q1 is a no-op as there
 * (statevector.py:46-47).  u: 32 doubles. */
TQ_API int tq_sv_apply_2q(void* psi, int n, int dtype, int q0, int q1, const double* u, void* stream);

/* CX / CZ / SWAP fast paths of apply_2q_statevector with gate_cx_4x4,
 * gate_cz_4x4, gate_swap_4x4 (gates.py:82-161). q0 == q1 is a no-op. */
TQ_API int tq_sv_apply_cx(void* psi, int n, int dtype, int control, int target, void* stream);
TQ_API int tq_sv_apply_cz(void* psi, int n, int dtype, int q0, int q1, void* stream);
TQ_API int tq_sv_apply_swap(void* psi, int n, int dtype, int q0, int q1, void* stream);

/* Dense 2^k x 2^k unitary on k <= TQ_MAX_KQ distinct qubits, qubits[0] = most
 * significant bit of the matrix index.  Replaces apply_kqubit_unitary
 * (statevector.py:71-129).  u: 2*4^k doubles (host). */
TQ_API int tq_sv_apply_kq(void* psi, int n, int dtype, const int* qubits, int k, const double* u, void* stream);

/* exp(-i theta/2 P) for a Pauli string P given as bit masks over basis-index
 * bits (x_mask = bits carrying X or Y, z_mask = bits carrying Y or Z).  One pass
 * over the state; equals the gate sequence of evolve_pauli_ops
 * (tyxonq/libs/circuits_library/utils.py:29-59) up to rounding. */
TQ_API int tq_sv_apply_pauli_rotation(void* psi, int n, int dtype, uint64_t x_mask, uint64_t z_mask,
                               double theta, void* stream);

/* psi <- (re + i im) * psi.  Used for the renormalisation after a Z projection
 * (engine.py:1075-1086, _project_z). */
TQ_API int tq_sv_scale(void* psi, int n, int dtype, double re, double im, void* stream);

/* ------------------------------------------------------------ measurement */

/* <Z_q> for every qubit q in [0, n): out_dev[q] (device, n doubles).
 * Replaces expect_z_statevector (statevector.py:62-68) and the per-qubit loop
 * of engine.py:467-473 with one pass.  FP64 accumulation. */
TQ_API size_t tq_sv_expect_z_workspace_bytes(int n);
TQ_API int tq_sv_expect_z_all(const void* psi, int n, int dtype, double* out_dev, void* ws,
                       size_t ws_bytes, void* stream);

/* probs[i] = |psi_i|^2 (float for TQ_C64, double for TQ_C128).  Replaces
 * engine.py:377-379 / probability() engine.py:1041-1047. */
TQ_API int tq_sv_probabilities(const void* psi, int n, int dtype, void* probs, void* stream);

/* Reduced density matrix of one qubit (unnormalised): out_dev[0..3] =
 * sum |a|^2, sum |b|^2, Re sum a conj(b), Im sum a conj(b) over the amplitude
 * pairs a = psi_i (qubit 0), b = psi_{i'} (qubit 1).  The Born weights of a
 * one-qubit Kraus channel, ||K_i psi||^2 = Tr(K_i rho K_i^dagger), follow on the
 * host; replaces the per-operator apply-and-sum loop of apply_kraus_statevector
 * (tyxonq/libs/quantum_library/kernels/statevector.py:132-218).  FP64 sums. */
TQ_API size_t tq_sv_qubit_rdm_workspace_bytes(int n);
TQ_API int tq_sv_qubit_rdm(const void* psi, int n, int dtype, int qubit, double* out_dev, void* ws,
                           size_t ws_bytes, void* stream);

/* Squared norm sum_i |psi_i|^2 into *out_dev (FP64). */
TQ_API size_t tq_sv_norm_workspace_bytes(int n);
TQ_API int tq_sv_norm2(const void* psi, int n, int dtype, double* out_dev, void* ws, size_t ws_bytes,
                void* stream);

/* Z-basis shot sampling from exact probabilities: out_indices[0..shots) gets
 * basis indices drawn i.i.d. from |psi_i|^2 / sum|psi|^2, returned in
 * ascending order (counts are their run lengths).  Replaces
 * nb.choice + bincount of engine.py:381-418.  Counter-based RNG (Philox4x32-10,
 * Salmon et al. SC'11) keyed by `seed`: the same seed gives the same shots. */
TQ_API size_t tq_sv_sample_workspace_bytes(int n, int64_t shots);
TQ_API int tq_sv_sample(const void* psi, int n, int dtype, int64_t shots, uint64_t seed,
                 int64_t* out_indices, void* ws, size_t ws_bytes, void* stream);

/* tq_sv_sample for callers that cannot allocate device memory.  No
 * counterpart in the reference.  Some callers cannot call cudaMalloc or hand
 * over a workspace: a host runtime that owns the device memory budget, or a
 * latency-critical loop in which an allocation (and the device
 * synchronisation it can imply) is not allowed.  This entry point takes only
 * the state and the output; its scratch is a fixed 8 MiB array in the
 * library's device memory (held on every GPU that loads the library, until
 * the process exits).  Requests whose tq_sv_sample_workspace_bytes(n, shots)
 * exceeds 8 MiB fail with TQ_ERR_RANGE (at 28 qubits that is about 980,000
 * shots).  The first call on a device looks the scratch address up
 * (cudaGetSymbolAddress), so make that first call before any stream capture.
 * The address is cached per device and CUDA context: after a device reset
 * (or a primary context released and created again) the next call looks it
 * up again, and that call too should come before any stream capture.
 * All calls share the one scratch array: calls that overlap on the GPU
 * (different streams, or different host threads) race and must be ordered by
 * the caller.  Results equal tq_sv_sample's for the same arguments. */
TQ_API int tq_sv_sample_noalloc(const void* psi, int n, int dtype, int64_t shots, uint64_t seed,
                                int64_t* out_indices, void* stream);

/* ------------------------------------------------------------ Pauli sums */

/* A Pauli-sum Hamiltonian H = sum_k c_k P_k in flip-mask groups.
 * Term k: P_k |i> = i^{ny_k} (-1)^{popc(i & zy_k)} |i ^ flip>, with
 * flip = bits carrying X or Y, zy = bits carrying Y or Z, ny = #Y.
 * weight = c_k * i^{ny_k} (complex: one of re/im is zero); f_re / f_im hold
 * the weight rounded to float, read by the complex64 kernels (this GPU runs
 * double -> float conversions at its FP64 rate, a small fraction of FP32).
 * Groups are contiguous term ranges sharing one flip mask.  Tables live in
 * device memory.  Semantics equal pauli_string_to_matrix / pauli_string_sum_dense
 * (tyxonq/libs/quantum_library/kernels/pauli.py:65-87) without forming 4^n. */
typedef struct {
  uint64_t flip;
  int32_t first_term;
  int32_t n_terms;
} tq_pauli_group;

typedef struct {
  uint64_t zy;
  double w_re;
  double w_im;
  float f_re;
  float f_im;
} tq_pauli_term;

/* E = <psi|H|psi> (real part) into *out_dev, FP64 accumulation, deterministic.
 * Replaces dynamics.expectation(psi, pauli_string_sum_dense(...))
 * (tyxonq/libs/quantum_library/dynamics.py:117-126). */
TQ_API size_t tq_sv_pauli_expectation_workspace_bytes(int n, int n_groups);
TQ_API int tq_sv_pauli_expectation(const void* psi, int n, int dtype, const tq_pauli_group* groups,
                            int n_groups, const tq_pauli_term* terms, int n_terms,
                            double* out_dev, void* ws, size_t ws_bytes, void* stream);

/* out = H psi (out must not alias psi).  Replaces apply_op
 * (chem_libs/hamiltonians_chem_library/hamiltonian_builders.py:283-318) without
 * densifying H. */
TQ_API int tq_sv_apply_pauli_sum(const void* psi, void* out, int n, int dtype, const tq_pauli_group* groups,
                          int n_groups, const tq_pauli_term* terms, int n_terms, void* stream);

/* ------------------------------------------------------------ fused tile passes */

/* A gate program executed as shared-memory tile passes.  Pass p names t local
 * bit positions pos[0..t) (ascending; pos[j] == j for j < nlow so global reads
 * come in runs of 2^nlow contiguous amplitudes).  The state is cut into
 * 2^(n-t) tiles of 2^t amplitudes (one tile = one value of the non-local
 * bits); each tile is read once, ops[op_begin..op_end) are applied to it in
 * shared memory, and it is written back once.  Op bit positions and masks are
 * LOCAL (0..t-1).  This replaces the reference's per-op interpreter loop
 * (engine.py:52-374 / :914-1039), which touches the whole state for every gate.
 *
 * Gradient fields (adjoint only): slot >= 0 marks a parametrised op whose
 * derivative dU/dtheta = -i/2 G U contributes Im <lam|G|psi> to slot_out[slot],
 * with G|i> = [i & gcm == gcm] i^gny (-1)^{popc(i & gzm)} |i ^ gxm>. */
#define TQ_TILE_MAX_BITS 16

typedef struct {
  int32_t kind; /* 1 dense2x2, 2 diag2x2, 3 dense4x4, 4 CX, 5 CZ, 6 SWAP, 7 Pauli rotation */
  int32_t a;    /* local bit of the first qubit (matrix high bit / control) */
  int32_t b;    /* local bit of the second qubit (matrix low bit / target) */
  int32_t slot; /* gradient slot, -1 = none */
  uint32_t xm, zm, cm;      /* kind 7: exp(-i a/2 P) on indices with (i & cm) == cm;
                               m[0] = cos(a/2), m[1] = -i sin(a/2) i^ny */
  uint32_t gxm, gzm, gcm;   /* generator masks (slot >= 0) */
  int32_t gny;              /* number of Y factors in the generator */
  int32_t pidx;             /* >= 0: angle a = pscale * theta[pidx], matrix built on the device
                               (kind 7: Pauli rotation; kind 2: phase diag(1, e^{ia})) */
  double pscale;
  double gcoef;             /* dE/d(angle) = gcoef * Im <lam|G|psi> (batched kernel) */
  uint32_t zo;              /* kind 7 in register stages: Z factors on local bits outside the stage */
  int32_t fuse_next;        /* forward register stages: the next fuse_next ops act on the same single
                               register bit a with no zo / zg sign (kinds 1, 2, 7) and are multiplied
                               into this op on the device; 0 = none */
  uint64_t zg;              /* kind 7: Z factors on non-local (global) bits; with zo they contribute
                               one sign per tile / thread, so only X/Y qubits need to be local */
  float mf[32];             /* matrix, complex64 kernels: row-major (re, im) */
  double md[32];            /* matrix, complex128 kernels */
} tq_tile_op;

typedef struct {
  int32_t t;
  int32_t nlow;
  int32_t op_begin;
  int32_t op_end;
  int32_t pos[TQ_TILE_MAX_BITS];
} tq_tile_pass;

/* Register stage of a staged tile pass: 4 local bit positions (ascending) whose
 * 16 amplitudes each thread holds in registers while ops[op_begin..op_end)
 * (bit indices / masks in register space 0..3) are applied. */
typedef struct {
  int32_t bits[4];
  int32_t op_begin;
  int32_t op_end;
} tq_tile_stage;

/* Forward staged passes: like tq_sv_run_tiles, but each pass's
 * [op_begin, op_end) indexes `stages` (device), and each stage applies its ops
 * in registers (one shared-memory sweep per stage instead of per op).  Needs
 * 9 <= t <= 14 (complex64) / 13 (complex128); CTAs of 2^(t-4) threads. */
TQ_API int tq_sv_run_staged(void* psi, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                            const tq_tile_stage* stages, const tq_tile_op* ops, const double* theta, void* stream);

/* ------------------------------------------------------------ Kraus trajectory batches */

/* One Kraus channel on `qubit` of n_traj trajectories of an n-qubit circuit,
 * stored as n_traj consecutive states of 2^n amplitudes: per trajectory the
 * qubit's reduced density matrix, the Born weights p_i = Tr(K_i rho K_i^dagger)
 * of the n_ops (<= 16) operators in kraus_dev (device, 8 doubles each,
 * row-major (re, im)), the first operator whose cumulative normalised weight
 * reaches status_dev[t] (and whose weight is positive), and psi_t <-
 * K_i psi_t / sqrt(p_i); chosen_dev[t] = i.  Fixed-order sums, no host round
 * trip.  Replaces the per-run unravelling of apply_kraus_statevector
 * (tyxonq/libs/quantum_library/kernels/statevector.py:132-218, engine.py:145-155),
 * one trajectory per call there, for a whole batch of trajectories here. */
TQ_API size_t tq_traj_kraus_workspace_bytes(int n, int n_traj);
TQ_API int tq_traj_kraus(void* psi, int n, int n_traj, int dtype, int qubit, const double* kraus_dev, int n_ops,
                         const double* status_dev, int32_t* chosen_dev, void* ws, size_t ws_bytes, void* stream);

/* ------------------------------------------------------------ circuit-specialised passes */

/* Runtime compilation (NVRTC, sm_103a) of staged forward pass kernels whose op
 * lists are straight-line code.  `source` is CUDA C++ written by
 * tyxonq_gb300/jit.py: it includes the library's device headers (found
 * through `include_dirs`) and defines one extern "C" kernel with the
 * parameters (T* psi, int n, PassArgs P, const tq_tile_stage* stages,
 * const tq_tile_op* ops, const ROp<R>* op_records, int dbuf).  On success
 * *cubin (host memory, release with tq_jit_free_host) holds the compiled
 * code; `log` (optional) receives the compiler log on failure.  These replace
 * the same interpreter loop as tq_sv_run_staged (engine.py:52-374 /
 * :914-1039), specialised per circuit structure; angles and matrices stay data
 * (op table and theta). */
TQ_API int tq_jit_build(const char* source, const char* const* include_dirs, int n_include_dirs, void** cubin,
                        size_t* cubin_size, char* log, size_t log_cap);
TQ_API void tq_jit_free_host(void* p);

/* Load a cubin of tq_jit_build on the current device; *kernel_out is the
 * handle of its kernel `kernel_name` (release with tq_jit_unload). */
TQ_API int tq_jit_load(const void* cubin, size_t cubin_size, const char* kernel_name, void** kernel_out);
TQ_API int tq_jit_unload(void* kernel);

/* Workspace of tq_jit_run_staged: the compiled op records of an n_ops table. */
TQ_API size_t tq_jit_rops_bytes(int dtype, int n_ops);

/* Staged forward passes with specialised kernels: pass p runs kernels[p]
 * (a tq_jit_load handle; CTAs of 2^(t - stage_bits) threads, stage_bits 4 or
 * 5), or the library's interpreting kernel where kernels[p] is NULL (4-bit
 * stages only).  Tables as tq_sv_run_staged (ops holds n_ops records;
 * stages_host is a host copy of `stages`, for launch sizes); at most 256 ops
 * per specialised pass; ws: tq_jit_rops_bytes(dtype, n_ops) bytes, 16-byte
 * aligned. */
TQ_API int tq_jit_run_staged(void* const* kernels, int stage_bits, void* psi, int n, int dtype,
                             const tq_tile_pass* passes, int n_passes, const tq_tile_stage* stages_host, const tq_tile_stage* stages,
                             const tq_tile_op* ops, int n_ops, const double* theta, void* ws, size_t ws_bytes,
                             void* stream);

/* Largest t supported for a dtype (shared-memory capacity). */
TQ_API int tq_sv_tile_max_bits(int dtype);

/* Forward: apply passes[0..n_passes) in order.  passes: host array; ops and
 * theta (angles of ops with pidx >= 0; may be NULL if there are none): device. */
TQ_API int tq_sv_run_tiles(void* psi, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                           const tq_tile_op* ops, const double* theta, void* stream);

/* Adjoint reverse sweep over passes (already in reverse order, ops in each pass
 * in reverse application order): for each op, first the gradient term (slot >= 0)
 * on (psi, lam), then psi <- U^dag psi, lam <- U^dag lam.  slot_out: device,
 * n_slots doubles (FP64, overwritten).  Follows the reverse loop of the
 * reference's CI-space adjoint energy_and_grad_civector
 * (chem_libs/quantum_chem_library/civector_ops.py:141-200). */
TQ_API size_t tq_sv_adjoint_tiles_workspace_bytes(int n, int n_slots);
TQ_API int tq_sv_adjoint_tiles(void* psi, void* lam, int n, int dtype, const tq_tile_pass* passes, int n_passes,
                               const tq_tile_op* ops, const double* theta, int n_slots, double* slot_out, void* ws,
                               size_t ws_bytes, void* stream);

/* Im <lam|G|psi> into *out_dev (FP64) for one generator G|i> = [i & cm == cm]
 * i^ny (-1)^{popc(i & zm)} |i ^ xm> (masks over basis-index bits, ny = popc(xm & zm)):
 * the per-gate gradient term of the unfused (plain engine) reverse sweep. */
TQ_API int tq_sv_generator_im(const void* psi, const void* lam, int n, int dtype, uint64_t xm, uint64_t zm,
                              uint64_t cm, double* out_dev, void* ws, size_t ws_bytes, void* stream);

/* ------------------------------------------------------------ batched VQE */

/* One VQE instance of a batch: energy E = <psi|H|psi> and dE/dtheta by the
 * adjoint sweep, psi = U(theta)|basis>.  Resident instances (streamed == 0)
 * keep psi and lam = H psi in shared memory: fwd/adj index op ranges whose bit
 * positions are global.  Streamed instances keep psi, lam in the caller's
 * pool at pool + scratch_offset (psi) and + scratch_offset + 2^n (lam),
 * amplitudes; fwd/adj index pass-table ranges.  Adjoint ops carry
 * slot = parameter index within the instance and gcoef. */
typedef struct {
  int32_t n;
  int32_t streamed;
  int32_t fwd_begin, fwd_count;
  int32_t adj_begin, adj_count;
  int32_t group_begin, group_count; /* Pauli groups of this instance's H (terms indexed globally) */
  int32_t theta_offset;
  int32_t grad_offset;
  int64_t scratch_offset;
  int64_t basis;
} tq_batch_inst;

/* Persistent launch over work[0..n_work) (instance indices, cost-sorted).
 * CTAs pull instances from *counter (device int, zeroed by the caller before
 * the launch) with atomicAdd; each CTA runs groups_per_cta independent thread
 * groups (threads_per_cta / groups_per_cta threads each, named barriers) for
 * resident instances, or one group for streamed ones.  grads must be zeroed
 * by the caller; energies[i] and grads[grad_offset..] are written per instance.
 * This is new: the reference evaluates VQE instances one at a time in Python
 * loops (devices/base.py:378-381, examples/vqe_batched_architecture_search.py:181-201). */
TQ_API size_t tq_batch_smem_bytes(int dtype, int max_resident_n, int groups_per_cta, int streamed_t);
TQ_API int tq_batch_run(int dtype, const tq_batch_inst* insts, const int32_t* work, int n_work, int streamed,
                        int groups_per_cta, int threads_per_cta, int grid, size_t smem_bytes,
                        const tq_tile_pass* passes, const tq_tile_op* ops, const tq_pauli_group* groups,
                        const tq_pauli_term* terms, const double* theta, void* pool, double* energies,
                        double* grads, int32_t* counter, void* stream);

/* ------------------------------------------------------------ batched VQE, L2-resident waves */

/* Large instances of a batch are evaluated in waves whose states fit in L2.
 * A wave phase is one launch over work items; each item is one tile of one
 * instance.  Offsets are in amplitudes into the state pool (psi and lam of an
 * instance live at psi_off and lam_off); theta/grad offsets index the batch's
 * parameter vector; part_off indexes the FP64 partial-sum buffer. */
typedef struct {
  int64_t psi_off;
  int64_t lam_off;
  int32_t pass;        /* forward / adjoint: pass-table index (stages in [op_begin, op_end)) */
  int32_t tile;        /* tile index within the pass (or H psi output tile) */
  int32_t theta_off;
  int32_t part_off;    /* adjoint: first partial slot of this item; H psi: energy partial slot */
  int32_t n;           /* qubits of the instance */
  int32_t group_begin; /* H psi: Pauli groups of the instance */
  int32_t group_count;
  int32_t basis_lo;    /* forward pass 0 of an instance: initial basis index (low 32 bits), else -1 */
} tq_wave_item;

/* kind 0: staged forward passes (psi), kind 1: H psi (lam = H psi over 2^hbits
 * output tiles, energy partial per item), kind 2: staged adjoint passes (psi,
 * lam, gradient partials per item and parameter op).  Every pass keeps at
 * least 4 contiguous low bits (nlow >= 4); a forward (kind 0) or adjoint
 * (kind 2) pass holds at most max_pass_ops ops, which sizes the shared memory
 * of the launch.  Items whose pass breaks either rule are skipped.
 * stage_bits: register bits per stage of the passes (forward 4; adjoint 3 or
 * 4 -- a CTA has 2^(t - stage_bits) threads holding 2^stage_bits amplitudes
 * of psi and of lam each; bits[stage_bits..3] of a tq_tile_stage are unused). */
TQ_API int tq_wave_run(int kind, int dtype, const tq_wave_item* items, int n_items, int t, int hbits,
                       int stage_bits, const tq_tile_pass* passes, const tq_tile_stage* stages,
                       const tq_tile_op* ops, const tq_pauli_group* groups, const tq_pauli_term* terms,
                       const double* theta, void* pool, double* partials, double* norm_partials,
                       int max_pass_ops, void* stream);

/* Divide energies and gradients by <psi|psi> (summed in order from the H psi
 * items' norm_partials of tq_wave_run kind 1): row r scales energies[inst[r]]
 * by 1 / sum(norm_partials[first[r] .. first[r] + count[r])) and
 * grads[goff[r] .. goff[r] + gcount[r]) likewise.  For exact unitary circuits
 * <psi|psi> = 1 and nothing changes; for complex64 states it removes the norm
 * drift of rounded rotation coefficients (E = <psi|H|psi> / <psi|psi>), the
 * largest part of the complex64 energy error against the reference's
 * complex128 dynamics.expectation (dynamics.py:117-126). */
TQ_API int tq_wave_normalize(const double* norm_partials, const int32_t* first, const int32_t* count,
                             const int32_t* inst, const int32_t* goff, const int32_t* gcount, int n_rows,
                             double* energies, double* grads, void* stream);

/* One launch of a wave phase (kind 0 forward, 2 adjoint with 4-bit stages)
 * with a circuit-specialised kernel (tq_jit_load of a wave source written by
 * tyxonq_gb300/jit.py): every item of items[0..n_items) must use a pass whose
 * body the kernel was generated for.  Arguments and shared memory as
 * tq_wave_run, whose interpreting kernels it replaces pass body by pass body;
 * both stand in for the reference's per-instance loop (devices/base.py:378-381). */
TQ_API int tq_jit_wave_run(void* kernel, int kind, int dtype, const tq_wave_item* items, int n_items, int t,
                           const tq_tile_pass* passes, const tq_tile_stage* stages, const tq_tile_op* ops,
                           const double* theta, const void* rops, void* pool, double* partials, int max_ops,
                           void* stream);

/* Op records of wave passes, built once per evaluation instead of once per
 * tile: job j writes n_ops records (tq_jit_rops_bytes each) for ops
 * [op_begin, op_begin + n_ops) with the angles at theta + theta_off, adjoint
 * records (with gradient terms) when flags & 1, to out + out_record.  Passing
 * out to tq_jit_wave_run as rops makes each item copy its records from
 * rops + item.group_begin records and reads its op count from
 * item.group_count (forward and adjoint items do not use their group fields
 * otherwise); NULL rops: the kernel builds them per item. */
typedef struct {
  int32_t op_begin;
  int32_t n_ops;
  int32_t theta_off;
  int32_t flags;
  int64_t out_record;
} tq_rop_job;
TQ_API int tq_wave_rops(int dtype, const tq_rop_job* jobs, int n_jobs, const tq_tile_op* ops, const double* theta,
                        void* out, void* stream);

/* H psi and / or <psi|H|psi> of one state (n >= 12) through the wave H psi
 * kernel: output tiles of 4096 amplitudes, 16 per thread, each group's terms
 * summed per class of the bits that tell a thread's amplitudes apart, then a
 * 16-point Walsh-Hadamard transform; partner tiles staged in shared memory
 * once per distinct flip >> 12.  The group list is cut into slices (more CTAs
 * for small states) whose partial outputs are added in slice order.  Same
 * semantics as tq_sv_apply_pauli_sum / tq_sv_pauli_expectation; groups must
 * be sorted by flip, and terms sorted by bits 8..11 of zy within each group
 * run fastest.  out or energy_out (device FP64) may be NULL, not both (with
 * out NULL no output is written at all); ws holds
 * tq_sv_pauli_sum_tiled_workspace_bytes(n, dtype, n_groups, out != NULL)
 * bytes (partial outputs only when there are several slices and an output).
 * Fixed-order sums: bit-identical replays. */
TQ_API size_t tq_sv_pauli_sum_tiled_workspace_bytes(int n, int dtype, int n_groups, int with_out);
TQ_API int tq_sv_pauli_sum_tiled(const void* psi, void* out, int n, int dtype, const tq_pauli_group* groups,
                                 int n_groups, const tq_pauli_term* terms, int n_terms, double* energy_out, void* ws,
                                 size_t ws_bytes, void* stream);

/* Fixed-order reductions of wave partials: out[k] (+)= scale[k] * sum of
 * partials[first[k] + j * stride[k]] for j < count[k]; accumulate != 0 adds. */
TQ_API int tq_wave_reduce(const double* partials, const int32_t* first, const int32_t* count, const int32_t* stride,
                          const double* scale, const int32_t* out_index, int n_out, double* out, int accumulate,
                          void* stream);

/* Re <a|b> into *out_dev (FP64), used by energy = <psi|H psi>. */
TQ_API size_t tq_sv_inner_workspace_bytes(int n);
TQ_API int tq_sv_inner_re(const void* a, const void* b, int n, int dtype, double* out_dev, void* ws,
                   size_t ws_bytes, void* stream);

/* ------------------------------------------------------------ CI-space UCC */

/* CI vector c (D real amplitudes, device) of the determinants with fixed
 * alpha / beta electron counts.  Excitation j maps determinant i to
 * fperm[j*D + i] with sign fphase[j*D + i] (0 where it annihilates i), and
 * f2phase[j*D + i] is the sign of its square; evolution
 *   c <- c + omc_t[j] * f2phase_j * c + sin_t[j] * fphase_j * c[fperm_j]
 * replaces evolve_civector_by_tensor
 * (chem_libs/quantum_chem_library/civector_ops.py:334-350).  Applies
 * excitations 0..n_ex-1 in order, or n_ex-1..0 with -sin_t (their inverses)
 * when reverse != 0.  sin_t / omc_t are HOST arrays; tmp is a D-double device
 * buffer; fperm entries must lie in [0, D). */
TQ_API int tq_ci_apply_excitations(double* civ, double* tmp, int64_t D, const int32_t* fperm, const int8_t* fphase,
                                   const int8_t* f2phase, const double* sin_t, const double* omc_t, int n_ex,
                                   int reverse, void* stream);

/* Reverse sweep of energy_and_grad_civector (civector_ops.py:141-200): from
 * the evolved ket and bra = H ket, un-apply excitations n_ex-1..0 to both and
 * write grads[j] = sum_i bra_i fphase_j[i] ket[fperm_j[i]] (device, FP64,
 * fixed-order sums); dE/dtheta_j = 2 grads[j].  sin_t / omc_t are HOST arrays. */
TQ_API size_t tq_ci_adjoint_workspace_bytes(int64_t D, int n_ex);
TQ_API int tq_ci_adjoint(const double* ket, const double* bra, int64_t D, const int32_t* fperm, const int8_t* fphase,
                         const int8_t* f2phase, const double* sin_t, const double* omc_t, int n_ex, double* grads,
                         void* ws, size_t ws_bytes, void* stream);

/* sum_i a_i b_i into *out_dev (FP64, fixed order). */
TQ_API size_t tq_ci_dot_workspace_bytes(int64_t D);
TQ_API int tq_ci_dot(const double* a, const double* b, int64_t D, double* out_dev, void* ws, size_t ws_bytes,
                     void* stream);

/* Scatter a CI vector into an n-qubit state (psi zeroed first; determinant
 * bitstring = basis index, fermion mode m = basis bit m) and read the CI
 * components of a state back (real parts).  H conserves the particle
 * numbers, so H applied in the full state and gathered equals H in CI space
 * (the reference forms the CI-space operator, hamiltonian_builders.py:283-318). */
TQ_API int tq_ci_embed(const double* civ, const uint64_t* strings, int64_t D, void* psi, int n, int dtype,
                       void* stream);
TQ_API int tq_ci_gather(const void* psi, const uint64_t* strings, int64_t D, int dtype, double* out, void* stream);

/* y = H x with H restricted to the CI space as CSR (row_ptr[D + 1] int64,
 * col int32, val FP64; device), one warp per row, fixed-order sums: the
 * apply_op(hamiltonian, ket) of energy_and_grad_civector (civector_ops.py:178,
 * hamiltonian_builders.py:283-318) with the CI-space operator that
 * hamiltonian_builders.py:165-178 contracts through pyscf. */
TQ_API int tq_ci_spmv(const int64_t* row_ptr, const int32_t* col, const double* val, int64_t D, const double* x,
                      double* y, void* stream);

/* Whole energy_and_grad_civector (civector_ops.py:141-200) for
 * D <= tq_ci_pairs_max_dim(n_ex): ket = unit vector init_index evolved by
 * excitations 0..n_ex-1 (one CTA, vector in shared memory), bra = H ket (CSR
 * as in tq_ci_spmv, many CTAs), out[0] = <bra, ket> and, when grad != 0, the
 * reverse sweep of tq_ci_adjoint with out[1 + j] = grads[j]
 * (dE/dtheta_j = 2 grads[j]), fixed-order sums.  Each excitation is given by
 * its PAIRS, the determinants it changes: int32 pairs [total][2] =
 * {i, (p << 1) | (fphase_j[i] < 0)} with p = fperm_j[i] > i, fphase_j[p] =
 * -fphase_j[i] and f2phase_j = -1 on both (every other determinant has
 * fphase_j = f2phase_j = 0); excitation j owns pairs pair_start[j] ..
 * pair_start[j + 1] (int64 [n_ex + 1], device), at most max_pairs <= 2 *
 * threads of them (TQ_ERR_RANGE above).  threads (256 or 1024) is the CTA
 * size of the sweeps: 256 keeps the per-excitation barrier short when every
 * excitation has at most 512 pairs.  part_start (int64 [n_ex + 2], device)
 * places the partial sums: part_start[0] = 0, part_start[1] = min(D,
 * threads), part_start[2 + j] = part_start[1 + j] + min(pairs of j,
 * threads); n_partials = part_start[n_ex + 1].
 * sin_omc: DEVICE FP64 [n_ex][2] = {sin t_j, 1 - cos t_j}.  ket_out (D
 * doubles, device) receives the evolved ket unless NULL; ws holds
 * tq_ci_energy_grad_workspace_bytes(D, n_partials) bytes.  Pairs outside
 * [0, D) are skipped.  TQ_ERR_RANGE when D is above the limit. */
TQ_API int64_t tq_ci_pairs_max_dim(int n_ex);
TQ_API size_t tq_ci_energy_grad_workspace_bytes(int64_t D, int64_t n_partials);
TQ_API int tq_ci_energy_grad(int64_t D, int64_t init_index, int n_ex, const int32_t* pairs,
                             const int64_t* pair_start, int64_t max_pairs, const int64_t* part_start,
                             int64_t n_partials, const double* sin_omc, const int64_t* row_ptr, const int32_t* col,
                             const double* val, int grad, int threads, double* ket_out, double* out, void* ws,
                             size_t ws_bytes, void* stream);

/* One fermionic excitation on the n-qubit statevector (fermion mode m =
 * basis bit m, i.e. qubit n-1-m).  F = T - T^dagger changes only the basis
 * states whose excitation bits (m_neg | m_pos, k = 2 or 4 of them, ascending
 * in bits[0..k)) equal m_neg or m_pos; they pair up as s_neg = base | m_neg,
 * s_pos = base | m_pos with F s_pos = phi s_neg, F s_neg = -phi s_pos,
 * phi = sign * (popcount(s_neg & zmask) odd ? 1 : -1) (the Jordan-Wigner
 * Z string; zmask holds no excitation bit), and F^2 = -1 on them.  So
 * exp(theta F) = psi + (1 - cos) F^2 psi + sin F psi
 * (statevector_ops.py:140-168 evolve_excitation) is a 2x2 rotation on each
 * pair and leaves every other amplitude as it is. */
typedef struct {
  uint64_t m_neg;
  uint64_t m_pos;
  uint64_t zmask;
  int32_t sign; /* +1 or -1 */
  int32_t k;    /* 2 (single) or 4 (double) */
  int32_t bits[4];
} tq_excitation;

/* Apply excitations 0..n_ex-1 in order (reverse = 0) or their inverses
 * n_ex-1..0 (reverse != 0) to psi: get_statevector's loop over
 * evolve_excitation (statevector_ops.py:66-114).  exc: DEVICE array of n_ex
 * records; sincos: DEVICE FP64 [n_ex][2] = {sin t_j, cos t_j}.  Records with
 * k not 2 / 4, bits out of range or masks that do not split the excitation
 * bits are skipped. */
TQ_API int tq_sv_apply_excitations(void* psi, int n, int dtype, const tq_excitation* exc, int n_ex,
                                   const double* sincos, int reverse, void* stream);

/* Reverse sweep for the energy gradient (the reference differentiates
 * get_statevector with torch autograd, pytorch_backend.py:446-564): from the
 * evolved psi and lam = H psi, un-apply excitations n_ex-1..0 to both and
 * write grads[j] = Re sum_s conj(lam_s) (F_j psi)_s (device FP64,
 * fixed-order sums); dE/dtheta_j = 2 grads[j].  psi and lam are overwritten. */
TQ_API size_t tq_sv_excitation_adjoint_workspace_bytes(int n, int n_ex);
TQ_API int tq_sv_excitation_adjoint(void* psi, void* lam, int n, int dtype, const tq_excitation* exc, int n_ex,
                                    const double* sincos, double* grads, void* ws, size_t ws_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TQ_SV_H */
