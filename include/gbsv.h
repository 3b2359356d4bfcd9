/*
 * gbsv.h -- C ABI of the GB300 state-vector engine (libgbsv.so).
 *
 * Every entry point takes raw device pointers, plain sizes and a
 * cudaStream_t passed as void*, returns an int status (GBSV_OK == 0) and
 * never allocates or frees caller memory.  Nothing here names a torch type;
 * a ctypes / cffi binding is all a Python caller needs.
 *
 * Layout contract (identical to unitair's "vector layout"):
 *   - a state is 2^n complex amplitudes, contiguous, interleaved (re, im);
 *     complex64 = 2 x float, complex128 = 2 x double;
 *   - qubit 0 is the MOST significant bit of the amplitude index, i.e.
 *     qubit q has stride 2^(n-1-q) amplitudes
 *     (unitair: src/unitair/states/conversions.py:5-45, tensor layout is a
 *     C-order view of the last dim as (2,...,2));
 *   - a k-qubit operator is a row-major 2^k x 2^k complex matrix whose row
 *     and column index is sum_j b_{q_j} 2^(k-1-j) for qubits = (q_0..q_{k-1}),
 *     so the first listed qubit is the matrix MSB
 *     (unitair: src/unitair/simulation/operations.py:151-186 and :322);
 *   - out[a] = sum_b op[a, b] * in[b]  (no conjugation).
 *
 * Batches: num_states states are processed; state s is read at
 * in + s * in_stride (in_stride == 0 broadcasts one state to every output,
 * unitair's "operator batched, state unbatched" case,
 * operations.py:304-309) and written densely at out + s * 2^n.  Operator s
 * is read at ops + s * op_stride complex elements (0 = one shared operator).
 * Any other broadcast that unitair accepts is reduced to these two strides
 * by the host layer before the call.
 *
 * In-place use (in == out) is allowed for every apply entry point whose
 * in_stride is 2^n: each amplitude group is read and written by the same
 * thread.
 */
#ifndef GBSV_H
#define GBSV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define GBSV_OK 0
#define GBSV_ERR_INVALID_ARG 1   /* bad size, qubit index, dtype or stride */
#define GBSV_ERR_UNSUPPORTED 2   /* valid request outside this build's limits */
#define GBSV_ERR_CUDA 3          /* a CUDA runtime call failed */
#define GBSV_ERR_SCRATCH 4       /* scratch buffer missing or too small */
#define GBSV_ERR_TIMEOUT 5       /* a bounded device-side wait gave up */

/* ---- element types ---------------------------------------------------- */
#define GBSV_C64 0    /* complex64: float re, float im */
#define GBSV_C128 1   /* complex128: double re, double im */
#define GBSV_F32 2    /* real float32 (angles, diagonals, probabilities) */
#define GBSV_F64 3    /* real float64 */

#define GBSV_MAX_DIMS 8
#define GBSV_MAX_DENSE_QUBITS 12

/* Broadcast descriptor for batched reductions and elementwise ops: the
 * output has shape[0..ndim-1]; operand a (b) element at multi-index i is
 * at sum_d i[d] * stride_a[d] (stride_b[d]); a zero stride broadcasts. */
typedef struct gbsv_bcast {
  int32_t ndim;
  int32_t pad_;
  int64_t shape[GBSV_MAX_DIMS];
  int64_t stride_a[GBSV_MAX_DIMS];
  int64_t stride_b[GBSV_MAX_DIMS];
} gbsv_bcast_t;

/* ---- library information --------------------------------------------- */
int gbsv_abi_version(void);
const char* gbsv_status_string(int status);
/* Text of the last CUDA or argument error seen by this thread. */
const char* gbsv_last_error(void);
/* Number of kernels this library has launched in this process. */
uint64_t gbsv_launch_count(void);

/* ---- complex128 arithmetic --------------------------------------------- */
#define GBSV_C128_PAIRS 0  /* double-float pairs on the FP32 pipe (default) */
#define GBSV_C128_FP64 1   /* native FP64 */

/* Process-wide choice of the complex128 gate arithmetic.  GB300 issues FP64
 * at about 1/64 of its FP32 rate, so by default the complex128 gate kernels
 * (gbsv_apply_operator with one operator shared by every state) compute in
 * pairs of floats: about 47 significant bits, a relative error of a few
 * 2^-47 per gate with no bias; amplitudes and entries outside [2^-40, 2^60]
 * still take FP64.  GBSV_C128_FP64 restores FP64 throughout.  No
 * counterpart in unitair (its complex128 path is torch's CPU FP64).
 * Returns GBSV_ERR_INVALID_ARG for an unknown mode. */
int gbsv_set_c128_arith(int mode);
int gbsv_get_c128_arith(void);

/* ---- gate application ------------------------------------------------- */

/* Apply a dense k-qubit operator (0 <= k <= GBSV_MAX_DENSE_QUBITS) to the
 * listed qubits of every state.  Replaces unitair.simulation.apply_operator
 * (src/unitair/simulation/operations.py:45-148) together with
 * apply_operator_tensor (:151-186) and act_first_qubits_tensor (:258-329):
 * the permute -> einsum -> permute sequence becomes one pass that addresses
 * amplitude pairs / quads by bit insertion.  qubits is a HOST array.
 * state_in == state_out (in place) is supported for k <= 5 (complex64) /
 * k <= 4 (complex128), and for complex64 operators on 6-12 qubits over
 * contiguous states (in_stride == 2^num_qubits when num_states > 1) except
 * per-state operators (op_stride != 0) on states of fewer than 2^(13-k)
 * groups of 2^k amplitudes (2^7 for k = 6).  Other in-place requests
 * return GBSV_ERR_UNSUPPORTED. */
int gbsv_apply_operator(const void* state_in, void* state_out, int dtype,
                        int num_qubits, int64_t num_states, int64_t in_stride,
                        const void* ops, int64_t op_stride,
                        const int32_t* qubits, int num_targets, void* stream);

/* Apply a 2x2 operator to every qubit.  Replaces
 * unitair.simulation.apply_all_qubits (operations.py:332-413).  With
 * op_qubit_stride == 0 the same operator (per state) acts on all qubits,
 * as in unitair; a non-zero op_qubit_stride (complex elements) reads a
 * separate operator for qubit q at ops + s*op_stride + q*op_qubit_stride
 * (an extension: unitair rejects per-qubit operator batches). */
int gbsv_apply_all_qubits(const void* state_in, void* state_out, int dtype,
                          int num_qubits, int64_t num_states,
                          int64_t in_stride, const void* ops,
                          int64_t op_stride, int64_t op_qubit_stride,
                          void* stream);

/* out = exp(-i * angles) * state with broadcasting.  Replaces
 * unitair.simulation.apply_phase (operations.py:15-42).  bc describes the
 * output shape; operand a is the real angle tensor (angle_dtype GBSV_F32 or
 * GBSV_F64), operand b the state (state_dtype GBSV_C64 / GBSV_C128); out is
 * dense in out_dtype (GBSV_C64 / GBSV_C128, torch's promotion result). */
int gbsv_apply_phase(const void* angles, int angle_dtype, const void* state,
                     int state_dtype, void* out, int out_dtype,
                     const gbsv_bcast_t* bc, void* stream);

/* ---- fused gate stages ------------------------------------------------ */

/* One fused-stage gate record (48 bytes, device memory).  kind:
 *   0 dense 2x2 on tile bit b0;
 *   1 dense 4x4 on tile bits b0 (matrix MSB) and b1;
 *   2 diagonal on nq (1 or 2) qubits, each a tile bit (>= 0) or a bit
 *     outside the tile encoded as -1 - position.
 * The gate acts only on tiles whose base satisfies (base & cmask) == cval
 * (controls outside the tile).  Its values sit at pool + mat
 * (+ state * mat_bstride for per-state gates): 4, 16 or 2^nq complex. */
typedef struct gbsv_fused_gate {
  int32_t kind;
  int32_t nq;
  int32_t b0, b1;
  uint64_t cmask, cval;
  int64_t mat;
  int64_t mat_bstride;
} gbsv_fused_gate_t;

/* Largest tile (qubits) a stage may use for this dtype (shared memory). */
int gbsv_fused_max_tile_qubits(int dtype);

/* Run one fused stage: every tile of 2^tile_qubits amplitudes (tile bits =
 * tile_positions[0..tile_qubits-1], a HOST array whose first
 * contiguous_qubits entries are 0..contiguous_qubits-1) is read once from
 * state_in, the gates are applied in shared memory in order, and the tile
 * is written once to state_out (in place allowed).  Replaces a run of
 * unitair apply_operator calls (src/unitair/simulation/operations.py:45-148)
 * -- each of which makes three passes over the state -- with one pass; the
 * same idea generalises unitair's host-side single-qubit fusion in
 * apply_to_qubits (operations.py:416-503, gates/matrix_algebra.py:6-51). */
int gbsv_run_stage(const void* state_in, void* state_out, int dtype,
                   int num_qubits, int64_t num_states, int64_t in_stride,
                   int tile_qubits, int contiguous_qubits,
                   const int32_t* tile_positions, const void* gates,
                   int num_gates, const void* pool, void* stream);

/* Register bits per thread of gbsv_run_stage_layouts for this dtype. */
int gbsv_fused_register_bits(int dtype);

/* One register layout of a stage (32 bytes, device memory): the tile bits
 * rb[0..R-1] index a thread's R = gbsv_fused_register_bits registers, and
 * gates[first_gate .. first_gate+num_gates) run in that layout.  In gate
 * records of a layout stage, dense targets (kind 0, 1) are REGISTER bits;
 * kind 3 is a 2x2 on register bit b0 applied where tile bit b1 is 1. */
typedef struct gbsv_layout {
  int32_t rb[5];
  int32_t first_gate;
  int32_t num_gates;
  int32_t pad_;
} gbsv_layout_t;

/* gbsv_run_stage with register blocking: the tile is staged in shared
 * memory, but each layout moves it into registers once and applies all of
 * its gates there (2^(tile_qubits - R) threads per tile, at most 512). */
int gbsv_run_stage_layouts(const void* state_in, void* state_out, int dtype,
                           int num_qubits, int64_t num_states,
                           int64_t in_stride, int tile_qubits,
                           int contiguous_qubits,
                           const int32_t* tile_positions, const void* gates,
                           const void* layouts, int num_layouts,
                           const void* pool, void* stream);

/* One register stage of a program, for gbsv_run_stages_multi (host
 * array).  gates is the program's record array and layouts this stage's
 * first layout record (device); tile_positions as for gbsv_run_stage. */
typedef struct gbsv_multi_stage {
  const void* state_in;
  void* state_out;
  const void* gates;
  const void* layouts;
  const void* pool;
  int64_t num_states;
  int64_t in_stride;
  int32_t num_layouts;
  int32_t contiguous_qubits;
  int32_t tile_positions[16];
} gbsv_multi_stage_t;

/* gbsv_run_stage_layouts for many programs at once: stage i of the host
 * array runs on its own states, all num_stages in one launch (batches of
 * 48), the CTAs shared in proportion to each stage's tiles.  Every stage
 * has num_qubits qubits and tile_qubits tile bits.  The serving loop
 * launches the r-th stage of every admitted circuit of one size together,
 * so small states fill the GPU.  No counterpart in unitair, which applies
 * one operator to one batch at a time. */
int gbsv_run_stages_multi(int dtype, int num_qubits, int tile_qubits,
                          const gbsv_multi_stage_t* stages, int num_stages,
                          void* stream);

/* Many circuits in one launch: CTA i runs gates[gate_first[i] ..
 * gate_first[i] + gate_count[i]) (records as for gbsv_run_stage with the
 * whole state as the tile, i.e. tile bit b = amplitude-index bit b) on the
 * state of 2^num_qubits amplitudes at state_ptrs[i], in place (each state
 * 16-byte aligned; a CTA whose state is not leaves it untouched).  state_ptrs
 * (uint64), gate_first and gate_count (int32) are device arrays of num_ctas
 * entries.  num_qubits <= gbsv_fused_max_tile_qubits(dtype).  This is the
 * batched launch of the serving loop: requests with different circuits and
 * the same qubit count run together.  No counterpart in unitair, which
 * applies one operator to one batch at a time. */
int gbsv_run_programs(int dtype, int num_qubits, int num_ctas,
                      const void* state_ptrs, const void* gate_first,
                      const void* gate_count, const void* gates,
                      const void* pool, void* stream);

/* ---- tensor-core stages (complex64) ------------------------------------ */

/* One block of a tensor-core stage (64 bytes, device memory): a 32x32
 * matrix on the 5 tile bits that index a thread's registers.  Offsets are
 * in amplitudes within the swizzled tile (amplitude index bits 1-3 XOR
 * bits 4-6, 7-9 and 10-12): rspo[k] for register-index bit k, tspo[j] for
 * thread-index bit j (128 threads).  mat indexes the image array (16 KiB
 * per block: B the 64x64 real form of U^T, Bh = rint(1024 * B) and
 * Bl = 1024 * B - Bh, stored as the fp16 K = 128 x N = 64 operand
 * [Bl; Bh] in the tensor cores' K-major no-swizzle layout with 8-row
 * groups 2048 bytes apart).  After the block, amplitudes are scaled by
 * a per-thread factor factors[fac + p * 128 + thread] (fac >= 0; p = the
 * state's bits at positions opos[0 .. nout-1], bit k of p from opos[k]) --
 * the diagonal gates that commute with the block, folded on the host -- and
 * by the post-diagonals diags[first_diag .. first_diag + num_diag).  flags
 * bit 0: register bit 0 is tile bit 0. */
typedef struct gbsv_tc_block {
  int16_t rspo[5];
  int16_t tspo[7];
  int32_t mat;
  int32_t first_diag;
  int32_t num_diag;
  int32_t flags;
  int32_t fac;
  int8_t nout;
  int8_t opos[7];
  int32_t pad_[3];
} gbsv_tc_block_t;

/* A 1- or 2-qubit diagonal applied after a block (48 bytes): each qubit is
 * a register bit (0..4), a thread-index bit (5 + j) or -1 - its position
 * outside the tile; qubit 0 is the MSB of the value index; reg != 0 when a
 * qubit is a register bit. */
typedef struct gbsv_tc_diag {
  int32_t nq;
  int32_t enc[2];
  int32_t reg;
  float d[8];
} gbsv_tc_diag_t;

/* One fused stage on the tensor cores: 12 tile bits (tile_positions, the
 * first contiguous_qubits of them the positions 0, 1, ...; the rest any
 * order), applied block by block with tcgen05.mma (A = the tile's columns
 * in tensor memory, B = the block image in shared memory), one HBM pass.
 * complex64 only, num_qubits >= 12, 1..64 blocks, states and images 16-byte
 * aligned; in place when state_in == state_out.  Generalises the
 * contraction unitair runs per gate (operations.py:322, torch.einsum over
 * the gate's qubit axes) to a product of gates applied as one matrix. */
int gbsv_run_stage_tc(const void* state_in, void* state_out, int dtype,
                      int num_qubits, int64_t num_states, int64_t in_stride,
                      int tile_qubits, int contiguous_qubits,
                      const int32_t* tile_positions, const void* blocks,
                      int num_blocks, const void* diags, const void* images,
                      const void* factors, void* stream);

/* Nonzero bits record a bounded wait inside a tensor-core stage that ran out
 * (1: block image, 2: MMA completion, 4 / 8: draining); clear != 0 resets
 * it.  Synchronizes the device.  No counterpart in the reference. */
int gbsv_tc_status(int* status, int clear);

/* ---- permutations, multi-controlled gates, sampling -------------------- */

/* out qubit j <- in qubit perm[j] (perm a HOST array of num_qubits entries;
 * out != in).  Replaces unitair's permute_qubits / swap / roll_qubits
 * (src/unitair/simulation/operations.py:506-654). */
int gbsv_permute_qubits(const void* in, void* out, int dtype, int num_qubits,
                        int64_t num_states, const int32_t* perm,
                        void* stream);

/* out = (-1)^k * in where k counts the masks (device array of uint64
 * amplitude-index bit masks, at most 256) whose bits are all set in the
 * amplitude index; in place allowed.  One mask per (control, target) pair
 * is unitair's multi_cz (operations.py:657-748); one mask over all listed
 * qubits is multi_controlled_z (:751-783). */
int gbsv_phase_flip(const void* in, void* out, int dtype, int num_qubits,
                    int64_t num_states, const void* masks, int num_masks,
                    void* stream);

/* X on `target` where every control qubit (HOST array) is 1; in place
 * allowed.  unitair's multi_controlled_x (operations.py:786-805) builds it
 * as H, multi_controlled_z, H. */
int gbsv_multi_controlled_x(const void* in, void* out, int dtype,
                            int num_qubits, int64_t num_states,
                            const int32_t* controls, int num_controls,
                            int target, void* stream);

/* Scratch bytes gbsv_sample needs for a state of `dim` amplitudes. */
size_t gbsv_sample_scratch_bytes(int64_t dim);

/* Draw num_samples basis indices from |state|^2 / sum |state|^2 (one state
 * of dim = 2^n amplitudes) into out_indices (device int64).  Samples are a
 * pure function of (seed, sample number).  state and scratch 16-byte
 * aligned.  Replaces the sampling in
 * unitair's measure (src/unitair/simulation/measurement.py:9-70). */
int gbsv_sample(const void* state, int dtype, int64_t dim,
                int64_t num_samples, uint64_t seed, int64_t* out_indices,
                void* scratch, size_t scratch_bytes, void* stream);

/* ---- host-side circuit planner ------------------------------------------ */

/* One gate of a circuit to plan (host memory).  kind: 0 dense, 1 diagonal,
 * 2 controlled-U (4x4 of the form diag(I, U), the first qubit controls).
 * Its row-major 2^nq x 2^nq complex128 matrix is at matrices + mat
 * (+ b * mat_bstride for per-state copy b of num_batch). */
typedef struct gbsv_gate_desc {
  int32_t kind;
  int32_t nq;
  int32_t q0, q1;
  int64_t mat;
  int64_t mat_bstride;
  int64_t num_batch;
} gbsv_gate_desc_t;

/* One pass of a planned circuit.  type 0: a single unfused gate (first =
 * gate index); 1: a shared-memory stage (records [first, first+count));
 * 2: a register-blocked stage (layouts [first, first+count)).  positions
 * are the stage's tile bits (the first `contiguous` are 0..contiguous-1). */
typedef struct gbsv_plan_op {
  int32_t type;
  int32_t contiguous;
  int32_t first, count;
  int32_t positions[16];
} gbsv_plan_op_t;

/* Caller-owned output buffers of gbsv_plan (host memory) and their counts. */
typedef struct gbsv_plan {
  int32_t dtype;          /* pool element type, GBSV_C64 or GBSV_C128 */
  int32_t used_layouts;   /* 1 if stages are register-blocked */
  gbsv_plan_op_t* ops;
  int32_t max_ops, num_ops;
  gbsv_fused_gate_t* records;
  int32_t max_records, num_records;
  gbsv_layout_t* layouts;
  int32_t max_layouts, num_layouts;
  void* pool;
  int64_t max_pool, pool_len;
} gbsv_plan_t;

/* Plan a circuit into fused stages on the host: greedy stages of
 * tile_qubits tile bits (the lowest min_contiguous always included),
 * register layouts of register_bits bits when the tile allows (0 = plain
 * shared-memory stages), gate
 * records specialised by structure, and the matrix pool converted to
 * plan->dtype.  fuse == 0 plans one pass per gate.  Returns
 * GBSV_ERR_SCRATCH if an output buffer is too small.  This is the native
 * counterpart of the planner in fusion.py (same output), fast enough to run
 * per request in the serving loop.  No counterpart in unitair. */
int gbsv_plan(const gbsv_gate_desc_t* gates, int num_gates,
              const void* matrices, int num_qubits, int tile_qubits,
              int min_contiguous, int register_bits, int fuse,
              gbsv_plan_t* plan);

/* ---- gradients --------------------------------------------------------- */

/* Scratch bytes gbsv_operator_grad needs (0 = none). */
size_t gbsv_operator_grad_scratch_bytes(int64_t num_states, int num_qubits,
                                        int num_targets, int shared);

/* dL/dU for out = U psi applied on `qubits` (torch's convention
 * grad_U = grad_out psi^H, summed over the non-target qubits):
 *   grad_ops[s][a, c] = sum_rest grad_out_s[rest|a] * conj(psi_s[rest|c]).
 * shared != 0 sums over all states into one matrix (the operator was shared
 * by the batch).  num_targets <= 6.  This is the operator half of the
 * autograd backward that unitair gets from torch through its einsum
 * (src/unitair/simulation/operations.py:322); the state half is
 * gbsv_apply_operator with the conjugate-transposed operator. */
int gbsv_operator_grad(const void* grad_out, const void* state_in, int dtype,
                       int num_qubits, int64_t num_states, int64_t in_stride,
                       const int32_t* qubits, int num_targets,
                       void* grad_ops, int shared, void* scratch,
                       size_t scratch_bytes, void* stream);

/* ---- adjoint differentiation ------------------------------------------ */

/* One term c * P of a Pauli-sum observable (32 bytes, device memory).
 * P = i^(#Y) X^xmask Z^zmask over amplitude-index bit positions (qubit q is
 * bit n-1-q; a Y sets the bit in both masks), and (re, im) = c * i^(#Y). */
typedef struct gbsv_pauli_term {
  uint64_t xmask, zmask;
  double re, im;
} gbsv_pauli_term_t;

/* out = H psi for H = sum_k terms[k] (at most 256 terms; out != psi).
 * No counterpart in unitair, whose observables are diagonals
 * (diag_expectation_value, src/unitair/states/innerprod.py:49-59); X/Y
 * terms such as X_i X_{i+1} need this. */
int gbsv_pauli_sum_apply(const void* psi, void* out, int dtype,
                         int num_qubits, int64_t num_states,
                         const void* terms, int num_terms, void* stream);

/* Scratch bytes gbsv_adjoint_rotation_step needs. */
size_t gbsv_adjoint_scratch_bytes(int64_t num_states, int num_qubits);

/* One backward step of the adjoint method for a rotation
 * U = exp(-i theta/2 P) on `qubit` (generator 0 = X, 1 = Y, 2 = Z), with
 * theta_s = angle_scale * angles[s * angle_stride] (float32 or float64):
 *   grad[s * grad_stride] += grad_factor * Im <lam_s| P |psi_s>
 * (FP64 accumulation), then psi_s <- U^dag psi_s and lam_s <- U^dag lam_s
 * in place.  One read and one write of both states.  Replaces torch
 * autograd through unitair's gate application
 * (src/unitair/simulation/operations.py:45-148), which stores every
 * intermediate state. */
int gbsv_adjoint_rotation_step(void* psi, void* lam, int dtype,
                               int num_qubits, int64_t num_states, int qubit,
                               int generator, const void* angles,
                               int angle_dtype, int64_t angle_stride,
                               double angle_scale, double* grad,
                               int64_t grad_stride, double grad_factor,
                               void* scratch, size_t scratch_bytes,
                               void* stream);

/* One op of a fused backward stage (80 bytes, device memory): kind 0 is a
 * rotation exp(-i theta/2 P) (gen 0 X, 1 Y, 2 Z) on tile bit `bit` (or
 * -1 - position outside the tile, Z only) with theta = scale *
 * params[s * num_params + pidx] whose gradient goes to `slot`; kind 1 is a
 * fixed gate whose ADJOINT is the record g (kinds 0-2 of
 * gbsv_fused_gate_t, values in pool). */
typedef struct gbsv_adjoint_op {
  int32_t kind, gen, bit, slot, pidx, pad_;
  double scale;
  gbsv_fused_gate_t g;
} gbsv_adjoint_op_t;

/* One fused backward stage of the adjoint method over the tiles of psi and
 * lam (same tile rules as gbsv_run_stage; tile_positions on the host):
 * applies the ops in order to both states in shared memory, one read and
 * one write of each state, and for every rotation adds
 *   slot_scale[k] * Im <lam_s|P|psi_s>   (FP64, summed over the state's
 * tiles in index order) to grad[s * num_params + slot_param[k]].
 * slot_param / slot_scale are device arrays of num_slots entries; scratch
 * holds num_slots * num_states * (2^(n - tile_qubits) + 2) doubles (tile
 * partials, then the cos / sin of every rotation per state).  psi and lam
 * 16-byte aligned. */
int gbsv_adjoint_stage(void* psi, void* lam, int dtype, int num_qubits,
                       int64_t num_states, int tile_qubits,
                       int contiguous_qubits, const int32_t* tile_positions,
                       const void* ops, int num_ops, const void* pool,
                       const void* params, int params_dtype,
                       int64_t num_params, int num_slots,
                       const int32_t* slot_param, const double* slot_scale,
                       double* grad, void* scratch, size_t scratch_bytes,
                       void* stream);

/* ---- reductions (FP64 accumulation) ----------------------------------- */

/* Scratch bytes a reduction over num_rows rows of length dim needs; 0 means
 * the reduction runs in one kernel without scratch. */
size_t gbsv_reduce_scratch_bytes(int64_t num_rows, int64_t dim);

/* sum_i |state[r, i]|^2 for every row r.  Replaces
 * unitair.states.norm_squared (src/unitair/states/innerprod.py:29-46).
 * out_dtype GBSV_F32 / GBSV_F64 (the engine always accumulates in FP64). */
int gbsv_norm_squared(const void* state, int dtype, int64_t num_rows,
                      int64_t dim, void* out, int out_dtype, void* scratch,
                      size_t scratch_bytes, void* stream);

/* Renormalisation checkpoint for deep circuits: measures every row's
 * squared norm (FP64 accumulation, written to norms_out, device float64
 * [num_rows]) and scales the row in place so its squared norm becomes
 * target_norms[row] (device float64 [num_rows]; typically the norms the
 * circuit started from, which a unitary circuit preserves).  Rounding in
 * long gate sequences drifts the norm; the caller reads the drift from
 * norms_out.  scratch as for gbsv_norm_squared.  Keeps the quantity
 * unitair's norm_squared reports (src/unitair/states/innerprod.py:29-46)
 * fixed; unitair itself has no such step. */
int gbsv_renormalize(void* state, int dtype, int64_t num_rows, int64_t dim,
                     const void* target_norms, void* norms_out, void* scratch,
                     size_t scratch_bytes, void* stream);

/* gbsv_norm_squared for callers that cannot allocate device memory: a host
 * program that reaches the library through a thin FFI and holds only
 * buffers another runtime gave it has no allocator to call, and a
 * latency-critical loop must avoid cudaMalloc, which can synchronize the
 * device.  Same inputs and outputs as gbsv_norm_squared; the FP64 partial
 * sums live in a fixed 64 KiB device array inside the library (held on every
 * GPU that loads it until exit) instead of caller scratch, and a request
 * whose partials do not fit is rejected with GBSV_ERR_UNSUPPORTED.  Each
 * call looks up that array's device address in the current context (no
 * allocation, no synchronization); under lazy module loading the first call
 * on a device also loads the library's device code, which can synchronize,
 * so make one warm-up call outside a latency-critical loop and before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * race.  Calls no cudaMalloc/cudaFree.  No counterpart in the reference
 * (unitair allocates through torch). */
int gbsv_norm_squared_noalloc(const void* state, int dtype, int64_t num_rows,
                              int64_t dim, void* out, int out_dtype,
                              void* stream);

/* |state[i]|^2 elementwise; out is real of the state's precision.
 * Replaces unitair.states.abs_squared (innerprod.py:4-26). */
int gbsv_abs_squared(const void* state, int dtype, int64_t count, void* out,
                     void* stream);

/* sum_i conj(a[r, i]) * b[r, i] over broadcast rows (bc: row shape and row
 * strides in units of rows of length dim; inner strides are 0 or 1).
 * Replaces unitair.states.inner_product (innerprod.py:62-65).  out_dtype
 * GBSV_C64 / GBSV_C128. */
int gbsv_inner_product(const void* a, const void* b, int dtype,
                       const gbsv_bcast_t* bc, int64_t dim,
                       int64_t inner_stride_a, int64_t inner_stride_b,
                       void* out, int out_dtype, void* scratch,
                       size_t scratch_bytes, void* stream);

/* sum_i diag[r, i] * |state[r, i]|^2 over broadcast rows (operand a = diag,
 * b = state).  Replaces unitair.states.diag_expectation_value
 * (innerprod.py:49-59).  out_dtype GBSV_F32 / GBSV_F64. */
int gbsv_diag_expectation(const void* diag, int diag_dtype,
                          const void* state, int state_dtype,
                          const gbsv_bcast_t* bc, int64_t dim,
                          int64_t inner_stride_diag,
                          int64_t inner_stride_state, void* out,
                          int out_dtype, void* scratch, size_t scratch_bytes,
                          void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBSV_H */
