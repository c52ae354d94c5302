/*
 * qgb.h -- C ABI of the GB300 (sm_103a) gate-application engine.
 *
 * Plain C: pointers, sizes and a CUDA stream passed as `void*` (a
 * cudaStream_t; NULL = legacy default stream). No allocation of state happens
 * behind these calls: every state, matrix and scratch buffer is owned by the
 * caller (in the Python host layer: torch's caching allocator). Every entry
 * point is asynchronous on `stream`, returns 0 on success or a negative
 * QGB_E* code, and leaves a message for qgb_last_error() (thread-local).
 * Argument errors are detected on the host before any launch.
 *
 * State layout (the reference's convention): a state of n qubits is 2^n
 * interleaved complex numbers (float2 for QGB_C64, double2 for QGB_C128);
 * site q is bit (n-1-q) of the flat index (site 0 is the most significant
 * axis of the reference's reshape([2]*n), tensorQ/statevector_sim.py:36,47).
 * A gate on sites `indices[0..k)` carries a row-major 2^k x 2^k matrix whose
 * row/column bit (k-1-j) belongs to indices[j] (tensorQ/statevector_sim.py:124-140).
 * A density matrix of n qubits is vec(rho) of 4^n entries, row (ket) index
 * in the high n bits, column (bra) index in the low n bits
 * (tensorQ/density_matrix_sim.py:12-42).
 */
#ifndef QGB_H
#define QGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QGB_ABI_VERSION 1

enum { QGB_C64 = 0, QGB_C128 = 1 };

enum {
    QGB_OK = 0,
    QGB_EINVAL = -1,   /* bad argument, detected on the host before launch */
    QGB_ECUDA = -2,    /* CUDA runtime error (launch or attribute call)      */
    QGB_ETIMEOUT = -3, /* a bounded device-side wait ran out                 */
    QGB_ESCRATCH = -4  /* scratch buffer too small (size query: qgb_*_scratch_bytes) */
};

#define QGB_MAX_QUBITS 34       /* 2^34 c64 amplitudes = 128 GiB */
#define QGB_MAX_K 6             /* largest dense gate (64 x 64)  */
#define QGB_SWEEP_MAX_OPS 64
#define QGB_SWEEP_MAX_HIGH 10
#define QGB_SWEEP_MAX_TILE_BITS 14

/* One fused pass over the state: a tile of 2^(low_bits + n_high) amplitudes
 * (flat bits [0, low_bits) plus the listed high bits) is staged in shared
 * memory, every op is applied to it in order, and it is written back.
 * op_pos[i][j] is the tile-local bit (0 .. low_bits+n_high-1) of matrix bit
 * (k-1-j); tile bit low_bits+h is flat bit high_bits[h]. op_mat[i] is the
 * element offset of op i's 2^k x 2^k matrix in the `mats` buffer. */
typedef struct {
    int32_t low_bits;
    int32_t n_high;
    int32_t high_bits[QGB_SWEEP_MAX_HIGH];
    int32_t n_ops;
    int32_t op_k[QGB_SWEEP_MAX_OPS];
    int32_t op_pos[QGB_SWEEP_MAX_OPS][QGB_MAX_K];
    int64_t op_mat[QGB_SWEEP_MAX_OPS];
} qgb_sweep;

/* One tensor-core tile sweep: the tile is 8192 amplitudes, the flat bits
 * [0, low_bits) (low_bits >= 4: contiguous runs of at least 128 bytes) and the
 * 13 - low_bits listed high bits; up to QGB_TCS_MAX_BLOCKS fused 5-qubit
 * blocks are applied to it in order, each on five tile bits. block_pos[b][j]
 * is the tile bit (0 .. 12; tile bit low_bits+h is flat bit high_bits[h]) of
 * matrix bit (4 - j); block_mat[b] the element offset of its 32 x 32
 * complex64 matrix in `mats`. */
#define QGB_TCS_MAX_BLOCKS 4
typedef struct {
    int32_t low_bits;
    int32_t high_bits[9];
    int32_t n_blocks;
    int32_t block_pos[QGB_TCS_MAX_BLOCKS][5];
    int64_t block_mat[QGB_TCS_MAX_BLOCKS];
} qgb_tc_sweep;

/* One pass of the adjoint reverse sweep over a batch of (state, co-state)
 * pairs, with the tile geometry of qgb_sweep. The ops are gates on 1 or 2
 * sites listed in the order the reverse sweep meets them (the circuit's last
 * gate first; gates on disjoint sites may be swapped). For op i and pair b:
 * if op_out[i] >= 0, grad_out[op_out[i] * batch + b] = Im <lam_b| P_i |phi_b>
 * at the gate's output, P_i the rotation generator given by one nonzero per
 * row (column op_gen_col[i][r], value op_gen_val[i][r] = (re, im)): a Pauli
 * product, so every value is +-1 or +-i and the columns are a permutation
 * (other rows are rejected with QGB_EINVAL); then
 * phi_b and lam_b <- U^dagger, U the 2^k x 2^k matrix at
 * mats + b * mat_stride + op_mat[i] elements (matrix order as qgb_sweep). */
typedef struct {
    int32_t low_bits;
    int32_t n_high;
    int32_t high_bits[QGB_SWEEP_MAX_HIGH];
    int32_t n_ops;
    int32_t op_k[QGB_SWEEP_MAX_OPS];
    int32_t op_pos[QGB_SWEEP_MAX_OPS][2];
    int64_t op_mat[QGB_SWEEP_MAX_OPS];
    int32_t op_out[QGB_SWEEP_MAX_OPS];
    int32_t op_gen_col[QGB_SWEEP_MAX_OPS][4];
    double op_gen_val[QGB_SWEEP_MAX_OPS][4][2];
} qgb_adjoint_sweep;

/* One tile sweep of the persistent trajectory kernel: the tile is the low L
 * flat bits times the H listed high bits (ascending, >= L); ops
 * [op_begin, op_end) of the op table run on it, in order (at most 128). */
typedef struct {
    int32_t L, H;
    int32_t high_bits[QGB_SWEEP_MAX_HIGH];
    int32_t op_begin, op_end;
} qgb_traj_sweep;

/* One gate of a trajectory sweep: width k (1 or 2), its sites as tile
 * positions in matrix order (pos[0] is the matrix's most significant bit),
 * the gate's index in the circuit (the Philox event of its channels, and what
 * the jump log records) and the element offset of its 2^k x 2^k matrix;
 * flags bit 0: the matrix is diagonal. Consecutive ops form runs over R tile
 * bits (R = min(4, tile bits) for complex64, min(3, tile bits) for
 * complex128) applied to groups of 2^R amplitudes in registers: the first op
 * of a run holds the run's length in `run` and the tile positions of its R
 * local bits in run_pos (local bit i <-> run_pos[i]); the others hold run = 0.
 * lpos: each site's local bit in its run (run_pos[lpos[j]] == pos[j]). */
typedef struct {
    int32_t k;
    int32_t pos[2];
    int32_t gate;
    int64_t mat;
    int32_t flags;
    int32_t run;
    int32_t run_pos[4];
    int32_t lpos[2];
} qgb_traj_op;

int qgb_abi_version(void);
const char* qgb_last_error(void);
/* Reads and clears the device status word set by bounded waits; returns
 * QGB_OK or QGB_ETIMEOUT. Synchronises `stream`. */
int qgb_check_status(void* stream);
/* Health check of the failure path (no counterpart in the reference, which
 * has no device code): one warp runs the library's bounded wait -- the helper
 * every kernel uses for its mbarrier and flag waits -- on a wait that cannot
 * finish, with limit_ns (at most 10 s): mode 0 an mbarrier that nobody
 * arrives on, mode 1 the device int at `flag` reaching 1 (nothing sets it),
 * mode 2 an mbarrier whose arrival comes first (completes). A wait that gives
 * up records its code in the status word, so the next qgb_check_status
 * returns QGB_ETIMEOUT, and the kernel returns; the context stays usable. */
int qgb_wait_probe(int mode, unsigned long long limit_ns, const int* flag, void* stream);
/* Peak rate of the fused multiply-add pipe (no counterpart in the reference):
 * sm_count * blocks_per_sm CTAs of 256 threads each run 8 independent chains
 * of `iters` FMAs in float32 (precision 0), float64 (precision 1) or packed
 * float32 pairs (precision 2, fma.rn.f32x2: twice the flops per instruction);
 * 2 * 8 * iters * 256 * CTAs flops (twice that for precision 2), no memory traffic. Time it with events on
 * `stream`; `out` is a device buffer of at least one value per CTA that is
 * never written in practice. The complex128 kernels' roofline is this rate. */
int qgb_fma_probe(int precision, int iters, int blocks_per_sm, void* out, void* stream);

/* ---- statevector ------------------------------------------------------ */

/* Replaces op_action (tensorQ/statevector_sim.py:124-140) as called by
 * StatevectorSim.apply_gate (:50-52): sv <- op on sites indices[0..k).
 * `op` is a device pointer to the 2^k x 2^k matrix in the state's dtype.
 * batch > 1 applies to `batch` states spaced sv_stride elements apart, each
 * with its own matrix spaced op_stride elements apart (0 = shared matrix). */
int qgb_op_action(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                  int64_t op_stride, int64_t batch, int64_t sv_stride, void* stream);

/* qgb_op_action for an op the caller knows to be unitary (fused gate blocks):
 * the tensor-core path then rescales each group of 2^k amplitudes to its input
 * norm, which a unitary preserves exactly, removing the systematic shrinkage of
 * the tensor cores' round-toward-zero fp32 accumulation (about 1e-7 of the
 * norm per pass). Other paths ignore the hint. No counterpart in the
 * reference, which applies gates through op_action (:124-140). */
int qgb_op_action_unitary(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                          int64_t op_stride, int64_t batch, int64_t sv_stride, void* stream);

/* qgb_op_action_unitary for one state (batch 1) as link `link` of a chain of
 * consecutive unitary passes over the same state: instead of restoring every
 * group's norm, the tensor-core path works in epochs of 4 passes. The pass that
 * starts the chain records its input's squared norm (the reference) in `chain`
 * (6 doubles of device memory, 3 rotating slots), the last pass of each epoch
 * its output's squared norm, and the first pass of the next epoch scales its
 * matrix by sqrt(reference / that norm); the norm stays within about one
 * epoch's drift (~4e-7 relative) of the reference. The caller numbers the
 * passes 0, 1, 2, ... and restarts at 0 after anything else touched the state;
 * link 0 clears the buffer. A pass that does not run on the tensor cores
 * (complex128, k < 4, batch > 1) clears the chain, so that a new one starts.
 * Replaces, like qgb_op_action, the reference's per-gate op_action
 * (tensorQ/statevector_sim.py:124-140), which has no norm control. */
int qgb_op_action_unitary_chain(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                                int64_t op_stride, int64_t batch, int64_t sv_stride, double* chain, int link,
                                void* stream);

/* qgb_op_action for one vector (batch 1) with the operator multiplied by the
 * float64 factor *factor, read on the device when the pass runs (so that a
 * factor computed by an earlier kernel on the stream can scale it without a
 * host round trip). On the tensor-core path the factor is folded into the
 * matrix; elsewhere a second pass multiplies the result. With
 * qgb_dm_trace_factor it forms the trace chain of complex64 density matrices
 * (a CPTP map keeps Tr rho; the tensor cores' round-toward-zero accumulation
 * shrinks it by ~1e-7 per pass). Replaces, like qgb_op_action, the
 * reference's per-op superoperator application DensityMatrixSim.apply_gate
 * (tensorQ/density_matrix_sim.py:38-42), which needs no such control. */
int qgb_op_action_scaled(void* sv, int dtype, int n, const int* indices, int k, const void* op,
                         const double* factor, void* stream);

/* Trace of one density matrix of n sites (vec(rho), 4^n entries), summed in
 * float64 in a fixed order by one CTA, into `chain` (3 doubles of device
 * memory): start != 0 sets chain[0] = Tr rho (the chain's reference) and
 * chain[1] = 1; otherwise chain[1] = chain[0] / Tr rho, the factor that the
 * next qgb_op_action_scaled applies. chain[2] = the trace measured. Callers
 * measure only where the ops applied so far form whole channels (both halves
 * of every unitary), where the trace equals the reference in exact
 * arithmetic. Counterpart of DensityMatrixSim.normalize_state's trace
 * (tensorQ/density_matrix_sim.py:85-89), without the division. */
int qgb_dm_trace_factor(const void* rho, int dtype, int n, double* chain, int start, void* stream);

/* A fused pass (several gates per read+write of the state), planned by the
 * host compiler from a Circuit's gate list (core/base_sim.py:30-53 loop). */
int qgb_apply_sweep(void* sv, int dtype, int n, const qgb_sweep* sweep, const void* mats,
                    int64_t mat_stride, int64_t batch, int64_t sv_stride, void* stream);

/* Selects the sweep kernel: 0 (default) = cp.async double-buffered tiles,
 * 1 = TMA-staged tiles with a producer warp when the geometry allows it
 * (runs of at least 128 bytes). Process-wide; both give identical results. */
int qgb_set_sweep_impl(int impl);

/* Several fused 5-qubit blocks per read and write of a complex64 state, on
 * the tensor cores (tcgen05, split-fp16 operands, fp32 accumulation): the
 * multi-block counterpart of qgb_op_action for fused circuits (the reference
 * applies each gate as its own op_action contraction,
 * tensorQ/statevector_sim.py:124-140, in BaseSim.run's loop,
 * core/base_sim.py:30-53). One state of n >= 14 qubits. With `chain` (6
 * doubles of device scratch, zeroed by the call at link 0) the sweep is a link
 * of the norm chain of unitary passes, as qgb_op_action_unitary_chain: link
 * numbers consecutive unitary passes from 0; the first pass of every epoch of
 * 4 corrects the norm drift measured at the end of the previous epoch. With
 * chain = NULL the blocks need not be unitary. */
int qgb_apply_tc_sweep(void* sv, int dtype, int n, const qgb_tc_sweep* sweep, const void* mats, double* chain,
                       int link, void* stream);
size_t qgb_tc_sweep_bytes(void);

/* An uneven batch of complex64 density matrices in one persistent launch on
 * the tensor cores (qgb_dm_batch_run): the batched counterpart of running
 * DensityMatrixSim (tensorQ/density_matrix_sim.py:38-42, driven by
 * core/base_sim.py:30-53) circuit by circuit, with each circuit's results
 * Tr rho, Tr rho^2 and Re Tr(rho Z_q) (tensorQ/density_matrix_sim.py:49-89)
 * from its last pass. A circuit (7..14 qubits) is a vec(rho) of 4^n entries
 * at `state` (16-byte aligned, overwritten: the run starts from
 * |0...0><0...0|) and its passes first_pass .. first_pass + n_passes - 1
 * of the pass table, in order; results go to row out_row. A pass applies a
 * 64 x 64 complex64 matrix (device address `mat`, matrix order) to the six
 * vec(rho) bits `bits` (bit bits[j] <-> matrix bit 5 - j). flags: 1 the pass
 * multiplies its matrix by 1 / the output trace of pass tslot (an earlier
 * pass of the same circuit flagged 2: the trace chain), 2 the pass measures
 * its output's trace, 4 the circuit's last pass (required on it, and only on
 * it), 8 the circuit's first pass (likewise). Every sum runs in a fixed order:
 * results are bitwise reproducible. */
typedef struct {
    uint64_t state;
    int32_t n;
    int32_t first_pass;
    int32_t n_passes;
    int32_t out_row;
} qgb_dm_circuit;

typedef struct {
    uint64_t mat;
    int32_t circ;
    int32_t bits[6];
    int32_t flags;
    int32_t tslot;
    int32_t pad;
} qgb_dm_pass;

size_t qgb_dm_batch_circuit_bytes(void);
size_t qgb_dm_batch_pass_bytes(void);
/* Work items of the batch: per pass, its tiles of 8192 entries dealt
 * round-robin to min(items_per_pass, tiles / 16) items (at least one;
 * concurrent items of a pass stream neighbouring memory; items_per_pass = the
 * SM count makes a large circuit's pass one wave), plus one finishing item per
 * circuit (-1 on bad arguments). */
int64_t qgb_dm_batch_items(const qgb_dm_circuit* circs, int ncirc, int items_per_pass);
/* Bytes of the device table (pass geometry, circuits, items). */
size_t qgb_dm_batch_table_bytes(int ncirc, int npasses, int64_t nitems);
/* Fills `table` (host memory of table_bytes) after checking the circuits and
 * passes; the caller copies it to device memory for qgb_dm_batch_run. */
int qgb_dm_batch_build(void* table, size_t table_bytes, const qgb_dm_circuit* circs, int ncirc,
                       const qgb_dm_pass* passes, int npasses, int items_per_pass);
/* Bytes of the device work buffer (counters and one slot per item). */
size_t qgb_dm_batch_work_bytes(int ncirc, int64_t nitems);
/* Runs every pass of every circuit in one persistent launch; out (device,
 * out_rows x out_cols float64, out_cols >= 16) and the work buffer are
 * cleared by the call. Asynchronous on `stream`. */
int qgb_dm_batch_run(const void* table, size_t table_bytes, int ncirc, int npasses, int64_t nitems, double* out,
                     int out_rows, int out_cols, void* work, size_t work_bytes, void* stream);

/* Arithmetic of complex128 tile sweeps (qgb_apply_sweep): 1 (default) =
 * double-float -- each float64 component carried as a pair of floats (48
 * significant bits) inside the tile, FP32 instructions only, the state in HBM
 * still complex128 -- 0 = float64 kernels. Process-wide; QGB_C128_ARITH=fp64
 * selects 0 at start-up. No reference counterpart: the reference's numpy
 * complex128 op_action (tensorQ/statevector_sim.py:124-140) has one arithmetic. */
int qgb_set_c128_arith(int mode);
int qgb_get_c128_arith(void);

/* Selects the kernel for complex64 dense blocks of k >= 4 qubits on at least
 * 2^(k+7) amplitudes: 0 = CUDA-core kernels only, 1 = tensor cores (tcgen05,
 * split-tf32 operands with fp32 accumulation) for k = 5, 6, 2 (default) =
 * tensor cores for k = 4, 5, 6. Process-wide; the environment variable
 * QGB_DENSE_IMPL sets the initial value. Results agree to fp32 rounding.
 * qgb_get_dense_impl returns the current selection. */
int qgb_set_dense_impl(int impl);
int qgb_get_dense_impl(void);

/* Writes |bits> (StatevectorSim.initialize_state, :31-48) to `batch` states. */
int qgb_init_basis(void* sv, int dtype, int n, uint64_t index, int64_t batch, int64_t sv_stride,
                   void* stream);

/* sv *= scale[b] for every state b (scale: device, float64, one per state). */
int qgb_scale(void* sv, int dtype, int n, const double* scale, int64_t batch, int64_t sv_stride,
              void* stream);

/* Scratch bytes needed by the reductions below for a given problem. */
size_t qgb_reduce_scratch_bytes(int n, int nterms, int64_t batch);

/* out[b] = ||sv_b||^2 in float64 (normalize_state, :107-109). */
int qgb_norm2(const void* sv, int dtype, int n, int64_t batch, int64_t sv_stride, double* out,
              void* scratch, size_t scratch_bytes, void* stream);

/* Replaces pauli_expectation_sv (tensorQ/statevector_sim.py:217-234):
 * out[b * nterms + t] = coeff[t] * <sv_b| P_t |sv_b> accumulated in float64.
 * `paulis` holds nterms strings of n characters 'i','x','y','z' and `coeff`
 * nterms weights (both host memory; coeff may be NULL for weights of 1). */
int qgb_pauli_expectation(const void* sv, int dtype, int n, const char* paulis, const double* coeff,
                          int nterms, int64_t batch, int64_t sv_stride, double* out, void* scratch,
                          size_t scratch_bytes, void* stream);

/* Allocation-free form of qgb_pauli_expectation for one state (no counterpart
 * in the reference): for callers that must not allocate device memory --
 * real-time loops that may not stall on the allocator, plugins whose host
 * application owns all device memory through its own pool and forbids
 * cudaMalloc/cudaFree beside it, GPUs whose memory is already fully reserved
 * so that even a small allocation would fail. Instead of a caller buffer it
 * uses one fixed 1 MiB device array inside the library, so it accepts at most
 * 64 terms and returns QGB_EINVAL beyond that. CUDA loads the library's device
 * code lazily: the array is reserved on a device when the first call there
 * (or the first call of any other reduction entry point) loads that code, and
 * held until the process exits -- make one warm-up call before reserving the
 * rest of the device's memory and before any stream capture, or set
 * CUDA_MODULE_LOADING=EAGER. Every call looks the array's address up again
 * (cudaGetSymbolAddress, the caller's device current), so it stays right
 * after a cudaDeviceReset. Calls share the array: calls that overlap on the
 * GPU race. Results equal qgb_pauli_expectation's (out: nterms float64,
 * device). */
int qgb_pauli_expectation_noalloc(const void* sv, int dtype, int n, const char* paulis, const double* coeff,
                                  int nterms, double* out, void* stream);

/* Applies one Pauli string per state in place (the sampled noise layers of
 * MonteCarloSim, tensorQ/monte_carlo_sim.py:14-28, which the reference turns
 * into X/Y/Z gates): state b gets i^ny[b] X^xmask[b] Z^zmask[b], flat-bit
 * masks (site q = bit n-1-q, a Y site in both masks). Masks and counts are
 * device arrays of `batch` entries. */
int qgb_pauli_layer(void* sv, int dtype, int n, const uint64_t* xmask, const uint64_t* zmask, const int* ny,
                    int64_t batch, int64_t sv_stride, void* stream);

/* Outcome probabilities of measuring `m` sites (measure_sv,
 * tensorQ/statevector_sim.py:185-193, whose probabilities are the diagonal of
 * rdm_from_sv, :182-183): probs[b] = sum over the other sites of |psi|^2, with
 * sites[0] the most significant bit of b (the reference orders the sites
 * ascending: pass them sorted for its outcome strings). float64, device,
 * 2^m entries, m <= 30, bitwise reproducible. Scratch:
 * qgb_probs_scratch_bytes(n, m) bytes (0 when m is within 5 of n). */
size_t qgb_probs_scratch_bytes(int n, int m);
int qgb_outcome_probs(const void* sv, int dtype, int n, const int* sites, int m, double* probs, void* scratch,
                      size_t scratch_bytes, void* stream);

/* Draws `shots` outcomes (int64 indices into probs, device) from the 2^m
 * probabilities (m <= 28, need not be normalised): float64 prefix sums and a
 * binary search per shot on a Philox4x32-10 uniform, counter (shot, 0, 1) under
 * key `seed` -- the same seed gives the same shots. Replaces the
 * numpy.random.choice call of measure_sv (:189-193). Scratch:
 * qgb_sample_scratch_bytes(m). */
size_t qgb_sample_scratch_bytes(int m);
int qgb_sample_outcomes(const double* probs, int m, int64_t shots, uint64_t seed, int64_t* out, void* scratch,
                        size_t scratch_bytes, void* stream);

/* Post-measurement state (measure_and_collapse_sv, :195-215): out (2^(n-m)
 * entries, the unmeasured sites in their order) = psi restricted to the
 * measured bits `outcome` (sites[0] its most significant bit), divided by
 * sqrt(probs[outcome]) read on the device. */
int qgb_collapse(const void* sv, int dtype, int n, const int* sites, int m, uint64_t outcome, const double* probs,
                 void* out, void* stream);

/* <a_b|b_b> = sum conj(a) b for every state b: out[2b], out[2b+1] = real,
 * imaginary part (float64). With b = (x)_q O_q a it gives
 * StatevectorSim.local_expectation / one_local_expectation (:63-73, :81-94). */
int qgb_inner_product(const void* a, const void* b, int dtype, int n, int64_t batch, int64_t stride, double* out,
                      void* scratch, size_t scratch_bytes, void* stream);

/* out = sum_t coeff[t] P_t sv  (H|psi> for the adjoint start); out and sv
 * distinct buffers of the same shape; paulis and coeff in host memory, at most
 * 128 terms. */
int qgb_pauli_apply(const void* sv, void* out, int dtype, int n, const char* paulis,
                    const double* coeff, int nterms, int64_t batch, int64_t sv_stride, void* stream);

/* Replaces partial_overlap (tensorQ/statevector_sim.py:155-180) on sites
 * indices[0..k), 1 <= k <= 10: out[b, r, c] = sum_rest a_b[r, rest]
 * conj(b_b[c, rest]), rows/cols ordered by `indices` as a gate matrix;
 * float64 complex out (device, batch * 4^k double2). Scratch:
 * qgb_partial_overlap_scratch_bytes (for k <= 2 also qgb_reduce_scratch_bytes(n, 32, batch)). */
int qgb_partial_overlap(const void* a, const void* b, int dtype, int n, const int* indices, int k,
                        int64_t batch, int64_t sv_stride, double* out, void* scratch,
                        size_t scratch_bytes, void* stream);
size_t qgb_partial_overlap_scratch_bytes(int n, int k, int64_t batch);

/* One step of the adjoint (reverse-mode) gradient sweep for a gate U on
 * sites indices[0..k), k <= 2, in a single pass over two distinct vectors:
 * phi <- U^dagger phi (uncompute), then, if grad_out is not NULL,
 * grad_out[2*(r*2^k+c)] (+1) = re (im) of sum_rest lam[r,rest] conj(phi[c,rest])
 * with the updated phi (float64, device, 2*4^k doubles; torch's gradient of a
 * real loss is twice this when lam is the loss's dL/d conj(psi)), and
 * lam <- U^dagger lam. Together with qgb_pauli_apply it replaces the
 * autograd tape of the reference's torch path (core/param_gates.py:21-49,
 * applications/compilation.py:73-133) with O(1) state memory; the reduction is
 * partial_overlap (tensorQ/statevector_sim.py:155-180). */
int qgb_adjoint_step(void* phi, void* lam, int dtype, int n, const int* indices, int k, const void* op,
                     double* grad_out, void* scratch, size_t scratch_bytes, void* stream);

/* qgb_adjoint_step for `batch` states (at sv_stride elements; phi and lam
 * batches disjoint), state b with its own gate matrix at op + b * op_stride
 * elements; grad_out (if not NULL) gets each state's 2 * 4^k doubles back to
 * back. One launch for every parameter set of a batched gradient. */
int qgb_adjoint_step_batched(void* phi, void* lam, int dtype, int n, const int* indices, int k, const void* op,
                             int64_t op_stride, int64_t batch, int64_t sv_stride, double* grad_out, void* scratch,
                             size_t scratch_bytes, void* stream);

/* The reverse step for a rotation U = expm(-i theta P) (P a Pauli product on
 * the k sites, P^2 = I; `generator` = P as 4^k complex128 pairs, row-major in
 * the order of `indices`, exactly one nonzero per row, else QGB_EINVAL):
 * uncomputes phi and lam like qgb_adjoint_step_batched and writes
 * grad_out[b] = Im <lam_b| P |phi_b>, both taken at the gate's
 * output. For a real loss with co-state lam, dL/dtheta = 2 * grad_out[b]: the
 * angle derivative of core/param_gates.py:51-103 without the 2 * 4^k
 * matrix-gradient slots. */
int qgb_adjoint_step_rotation(void* phi, void* lam, int dtype, int n, const int* indices, int k, const void* op,
                              int64_t op_stride, const double* generator, int64_t batch, int64_t sv_stride,
                              double* grad_out, void* scratch, size_t scratch_bytes, void* stream);

/* Register runs of the adjoint reverse sweep (qgb_adjoint_sweep_step): -1
 * (default) or 3 groups consecutive gates whose sites fit 3 tile bits and
 * applies each group to registers holding 8 amplitudes of the state and the
 * co-state (one shared-memory pass and one barrier per group; real matrices,
 * diagonals, CNOT/SWAP/X permutations and the generator's row pattern --
 * diagonal, flipped or other -- specialised at compile time); 0 runs one
 * shared-memory pass per
 * gate. Process-wide; results agree to rounding. No reference counterpart. */
int qgb_set_adjoint_runs(int bits);

/* Scratch bytes for qgb_adjoint_sweep_step (a function of the problem only). */
size_t qgb_adjoint_sweep_scratch_bytes(int n, int tile_bits, int n_ops, int64_t batch);

/* The adjoint reverse sweep for many gates per pass (qgb_adjoint_sweep): phi
 * and lam (batch pairs at sv_stride elements, disjoint, 16-byte aligned) are
 * read and written once per call instead of once per gate, and the rotation
 * derivatives of qgb_adjoint_step_rotation come out for every op with
 * op_out >= 0 (each slot written once, fixed summation order). */
int qgb_adjoint_sweep_step(void* phi, void* lam, int dtype, int n, const qgb_adjoint_sweep* sweep, const void* mats,
                           int64_t mat_stride, int64_t batch, int64_t sv_stride, double* grad_out, void* scratch,
                           size_t scratch_bytes, void* stream);

/* Parametrised gate matrices M(theta) = expm(-i theta P) = cos(theta) I -
 * i sin(theta) P (core/param_gates.py:21-80, no factor 1/2) for `nsets`
 * parameter sets in one launch: gate g of set s (kinds[g]: 1 RX, 2 RY, 3 RZ,
 * 4 RXX, 5 RYY, 6 RZZ; other kinds are left to the caller) with angle
 * params[s * nparams + pidx[g]] (float64), written row-major in `dtype` at
 * out + s * set_stride + g * gate_stride elements. All arrays in device memory.
 * Replaces the per-gate host construction and host-to-device copy of the
 * reference (tensorQ/statevector_sim.py:19-29). */
int qgb_param_matrices(const int* kinds, const int* pidx, int ngates, const double* params, int nparams,
                       int64_t nsets, void* out, int dtype, int64_t gate_stride, int64_t set_stride, void* stream);

/* Angle gradients from per-gate derivatives: grad_out[s * nparams + j] =
 * scale * sum over the gates g of parameter j (CSR csr_ptr / csr_gate, in that
 * order) of gate_values[g * nsets + s], e.g. the outputs of
 * qgb_adjoint_step_rotation (scale 2 * dL/dE). Device arrays. Replaces the
 * autograd walk from each gate matrix back to its angle (torch.linalg.matrix_exp
 * backward, core/param_gates.py:51-103). */
int qgb_param_grads(const int* csr_ptr, const int* csr_gate, int nparams, int64_t nsets, const double* gate_values,
                    double scale, double* grad_out, void* stream);

/* ---- noisy trajectories -------------------------------------------------- */

/* Blocks per trajectory used by qgb_traj_step (sizes its `partials`: at least
 * ntraj * qgb_traj_blocks(n) * 4 doubles). */
int qgb_traj_blocks(int n);

/* One gate of a batch of `ntraj` noisy trajectories (states of n qubits,
 * `stride` elements apart), replacing the per-sample statevector runs of
 * MonteCarloSim (tensorQ/monte_carlo_sim.py:14-35) and extending them to
 * amplitude damping. Applies, per trajectory: the pending normalised Kraus
 * operators of the previous gate's sites (`prev_sites`, `kprev`; read from
 * `kraus`), then the gate (`sites`, `k` <= 2, device matrix `gate`), then an
 * independent depolarising Pauli (I w.p. 1-p_dep, X/Y/Z w.p. p_dep/3) on each
 * gate site; then draws each site's amplitude-damping branch (gamma) from the
 * exact populations and overwrites `kraus` (device, ntraj x 2 x 4 complex of
 * the state dtype) with the chosen K0/sqrt(1-p) or K1/sqrt(p) for the next
 * call. k = 0 only applies the pending operators. Random numbers are
 * Philox4x32-10 of (event, trajectory, 2*site + {0: Pauli, 1: damping}) keyed
 * by `seed`; `event` must be unique per gate of a run. pauli_log / jump_log
 * (device, ntraj x 2 bytes, or NULL) record the branches. */
int qgb_traj_step(void* sv, int dtype, int n, int64_t ntraj, int64_t stride, const int* sites, int k,
                  const void* gate, const int* prev_sites, int kprev, void* kraus, double p_dep, double gamma,
                  uint64_t seed, uint32_t event, double* partials, uint8_t* pauli_log, uint8_t* jump_log,
                  void* stream);

/* Every trajectory of a noisy circuit in one persistent launch (replaces the
 * reference's per-sample loop MonteCarloSim.circuit_sample /
 * expectation_sample, tensorQ/monte_carlo_sim.py:14-35, extended to amplitude
 * damping as in qgb_traj_step). Each CTA takes the next trajectory from a
 * work counter and runs it through every sweep (tables `sweeps_dev` /
 * `ops_dev` in device memory, `sweeps_host` / `ops_host` the same tables in
 * host memory, checked before the launch; `mat_elems` matrices' elements at
 * `mats` in the state's dtype): after each gate,
 * on each of its sites, depolarising p_dep (the Paulis qgb_traj_step draws
 * for the same seed) then amplitude damping gamma, unravelled exactly by the
 * no-jump norm (a sweep that contains a jump runs again from its input with
 * the jump). Output: the normalised final states at sv + t * stride,
 * jump_count[t] (device, may be NULL) and, when max_log > 0, the first max_log
 * jumps of trajectory t as (gate, site) pairs at jump_log[(t * max_log + i) *
 * 2]. scratch: qgb_traj_run_scratch_bytes(dtype, n, largest tile bits, ntraj)
 * bytes of device memory (a work counter and one state per resident CTA). */
int qgb_traj_run(void* sv, int dtype, int n, int64_t ntraj, int64_t stride, const qgb_traj_sweep* sweeps_host,
                 const qgb_traj_sweep* sweeps_dev, int nsweeps, const qgb_traj_op* ops_host,
                 const qgb_traj_op* ops_dev, int nops, const void* mats, int64_t mat_elems, double p_dep,
                 double gamma, uint64_t seed, int* jump_count, int* jump_log, int max_log, void* scratch,
                 size_t scratch_bytes, void* stream);
size_t qgb_traj_run_scratch_bytes(int dtype, int n, int tile_bits, int64_t ntraj);
size_t qgb_traj_sweep_bytes(void);
size_t qgb_traj_op_bytes(void);

/* The Philox uniform the trajectory kernels draw (host-side, for replays). */
void qgb_philox_uniform(uint32_t event, uint32_t traj, uint32_t stream, uint64_t seed, double* out);

/* ---- batches of small uneven circuits ------------------------------------ */

/* Layout sizes of the two device tables qgb_fuse_blocks reads:
 *   block (qgb_fuse_block_bytes() bytes): int64 out (element offset of the
 *     block's 2^k x 2^k row-major matrix in `out`), int32 k (<= 6), int32
 *     op_begin, int32 op_end (its entries in the entry table, first applied
 *     first), int32 pad;
 *   entry (qgb_fuse_entry_bytes() bytes): int32 k (<= the block's k), int32
 *     pos[6] (block-matrix bit of each op bit, 0 = most significant, in the
 *     op's matrix order), int32 pad, int64 mat (complex128 element offset of
 *     the op's 2^k x 2^k row-major matrix in `op_mats`). */
size_t qgb_fuse_block_bytes(void);
size_t qgb_fuse_entry_bytes(void);

/* The matrix products of gate fusion, on the device (no counterpart in the
 * reference, which applies each gate as its own contraction through
 * BaseSim.run, core/base_sim.py:30-53): block b = E_m ... E_1, E_i the
 * embedding of entry i's op matrix into the block's bits, composed in float64
 * and written to `out` in `dtype`. Tables and op matrices are device memory;
 * `out_elems` and `op_elems` bound every offset: an entry outside them is
 * skipped and reported by qgb_check_status (QGB_EINVAL). */
int qgb_fuse_blocks(void* out, int dtype, int64_t out_elems, const void* blocks, int nblocks,
                    const void* entries, int nentries, const void* op_mats, int64_t op_elems, void* stream);

/* Layout sizes of the two device tables qgb_batch_small reads:
 *   circuit (qgb_batch_circuit_bytes() bytes): int64 offset (elements into
 *     `states`), int64 out_offset (doubles into `out`), int32 nbits, int32
 *     op_begin, int32 op_end, int32 flags (bit 0: start from basis state 0),
 *     int32 dm_sites (> 0: the vector is vec(rho) of that many qubits, <= 7),
 *     int32 pad;
 *   op (qgb_batch_op_bytes() bytes): int32 k, int32 pos[6] (flat bits of the
 *     circuit's vector, matrix order), int64 mat (element offset in `mats`). */
size_t qgb_batch_circuit_bytes(void);
size_t qgb_batch_op_bytes(void);

/* Runs `ncirc` independent circuits in one launch, one CTA per circuit: each
 * vector (at most 2^max_bits entries, max_bits <= 14 for complex64 and 13 for
 * complex128) is staged in shared memory once, the circuit's ops
 * [op_begin, op_end) are applied in order, and it is written back -- the
 * DensityMatrixSim / StatevectorSim run loop (core/base_sim.py:30-53) for
 * many small circuits at once. If `out` is not NULL, every density-matrix
 * circuit also writes Re Tr(rho), Tr(rho^2) and Re Tr(rho Z_i) (i < dm_sites)
 * to out[out_offset ..] in float64 (DensityMatrixSim.one_local_expectation,
 * tensorQ/density_matrix_sim.py:60-70). Tables live in device memory. */
int qgb_batch_small(void* states, int dtype, const void* circuits, int ncirc, const void* ops, const void* mats,
                    int max_bits, int max_k, double* out, void* stream);

/* ---- density matrix ---------------------------------------------------- */

/* Replaces DensityMatrixSim.apply_gate (tensorQ/density_matrix_sim.py:38-42)
 * for a superoperator given in the reference's to_superop() layout
 * (core/gates.py:43-44, core/noise.py:10-13): a row-major 4^k x 4^k matrix
 * whose row/col bits are (bra sites.., ket sites..) in `indices` order.
 * Applied to vec(rho) of n qubits (4^n entries). Input legs follow
 * `indices`; output legs follow ascending site order, exactly as the
 * reference's generate_gate_indices (:91-99) assigns them. */
int qgb_dm_apply_superop(void* rho, int dtype, int n, const int* indices, int k,
                         const void* superop, int64_t batch, int64_t rho_stride, void* stream);

/* out[b * nterms + t] = coeff[t] * Tr(rho_b P_t) for Pauli strings (float64;
 * paulis and coeff in host memory). */
int qgb_dm_pauli_expectation(const void* rho, int dtype, int n, const char* paulis,
                             const double* coeff, int nterms, int64_t batch, int64_t rho_stride,
                             double* out, void* scratch, size_t scratch_bytes, void* stream);

/* out[b] = Re Tr((x)_q O_q rho_b) for single-site operators (host, n 2x2
 * complex128 row-major) -- DensityMatrixSim.local_expectation /
 * one_local_expectation (:49-70). */
int qgb_dm_product_expectation(const void* rho, int dtype, int n, const double* ops, int64_t batch,
                               int64_t rho_stride, double* out, void* scratch, size_t scratch_bytes,
                               void* stream);

/* out[b] = Re Tr(rho_b) (float64) -- normalize_state (:85-89). */
int qgb_dm_trace(const void* rho, int dtype, int n, int64_t batch, int64_t rho_stride, double* out,
                 void* scratch, size_t scratch_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QGB_H */
