/*
 * tqk.h -- C ABI of the GB300 statevector engine (libtqk.so).
 *
 * Plain pointers and sizes only.  Every entry point:
 *   - takes device pointers for statevectors / matrices / outputs,
 *   - takes the CUDA stream to launch on as an opaque handle (cudaStream_t / CUstream),
 *   - validates its arguments on the host and returns a TQK_* status (0 = OK),
 *   - never synchronises the stream and never allocates device memory; callers pass
 *     scratch buffers sized by the matching *_scratch_bytes query.
 * tqk_last_error() returns the message of the last failing call on this host thread.
 *
 * Layout: a statevector is complex64 (interleaved float re, im) of shape [bsz, 2^n];
 * wire 0 is the MOST significant bit of the in-row index.  A k-wire matrix is
 * complex64 row-major [mat_batch, 2^k, 2^k] indexed with wires[0] most significant;
 * mat_batch is 1 (broadcast over the state batch) or bsz (one matrix per row).
 *
 * Each declaration cites the upstream torchquantum interface it replaces
 * (path:line inside the upstream project).
 */
#ifndef TQK_H_
#define TQK_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TQK_OK = 0,
  TQK_BAD_WIRES = 1,        /* wire out of range, duplicated, or too many */
  TQK_BAD_SHAPE = 2,        /* bsz / n / batch / size inconsistent */
  TQK_BAD_POINTER = 3,      /* null or misaligned pointer */
  TQK_TOO_MANY_QUBITS = 4,  /* n or k beyond the supported maximum */
  TQK_CUDA_ERROR = 5,       /* a CUDA launch or API call failed */
  TQK_TIMEOUT = 6,          /* a bounded device-side wait gave up */
  TQK_SCRATCH_TOO_SMALL = 7,
  TQK_UNSUPPORTED = 8
};

#define TQK_MAX_QUBITS 34      /* per batch row */
#define TQK_MAX_DENSE_WIRES 12 /* generic dense gate width */
#define TQK_MAX_OP_WIRES 16    /* wires one op may touch (controls + targets) */

const char* tqk_last_error(void);
int tqk_version(void);

/* ---------------------------------------------------------------- gate application
 * Replaces functional/gate_wrapper.py:96-140 (apply_unitary_bmm) and :18-93
 * (apply_unitary_einsum), as dispatched from gate_wrapper (gate_wrapper.py:441-446).
 * All are in place on `state`. */

/* Dense U (2^k x 2^k) on `wires` (k = 1..TQK_MAX_DENSE_WIRES). */
int tqk_apply_matrix(void* state, int64_t bsz, int n, const int32_t* wires, int k,
                     const void* mat, int64_t mat_batch, void* stream);

/* Controlled dense block: the 2^kt x 2^kt block `mat` acts on `targets` (kt = 1 or 2)
 * where every control wire is 1.  Same operator as the upstream 2^(nc+kt) matrix whose
 * upper-left block is identity (e.g. crx_matrix, functional/rx.py:87-115). */
int tqk_apply_controlled(void* state, int64_t bsz, int n, const int32_t* controls, int nc,
                         const int32_t* targets, int kt, const void* mat, int64_t mat_batch,
                         void* stream);

/* Multi-controlled X on `target` where every control equals ctrl_val (1: cnot/toffoli/
 * multicnot, functional/paulix.py; 0: multixcnot).  nc may be 0 (Pauli X). */
int tqk_apply_mcx(void* state, int64_t bsz, int n, const int32_t* controls, int nc, int ctrl_val,
                  int target, void* stream);

/* Multiply amplitudes whose `wires` are all 1 by phase[b] (complex64, phase_batch 1|bsz).
 * k = 0 multiplies every amplitude (globalphase).  cz/ccz/s/t/u1/cu1/... */
int tqk_apply_phase(void* state, int64_t bsz, int n, const int32_t* wires, int k,
                    const void* phase, int64_t phase_batch, void* stream);

/* Diagonal gate: amplitude *= diag[b][bits of `wires`] (diag complex64 [batch, 2^k]).
 * rz/rzz/crz/multirz (functional/rz.py). */
int tqk_apply_diagonal(void* state, int64_t bsz, int n, const int32_t* wires, int k,
                       const void* diag, int64_t diag_batch, void* stream);

/* Exchange |..0 1> and |..1 0> on (w0, w1) where every control is 1 (swap, cswap). */
int tqk_apply_swap(void* state, int64_t bsz, int n, const int32_t* controls, int nc, int w0,
                   int w1, void* stream);

/* Reset `wires` to |0> and renormalise each row (functional/reset.py). */
int64_t tqk_reset_scratch_bytes(int64_t bsz, int n);
int tqk_reset(void* state, int64_t bsz, int n, const int32_t* wires, int k, void* scratch,
              int64_t scratch_bytes, void* stream);

/* ---------------------------------------------------------------- measurement
 * |psi|^2 as float32 [bsz, 2^n] (the probabilities read by measurements.py:297-299). */
int tqk_probs(const void* state, int64_t bsz, int n, float* out, void* stream);

/* Computational-basis sampling (upstream tq.measure, measurement/measurements.py:37-74,
 * draws on the host with random.choices).  For every row b and shot s, out[b*shots + s]
 * is the first index i with sum_{j<=i} |psi_j|^2 > uniforms[b*shots + s] * sum_j |psi_j|^2
 * (inverse CDF in float64; uniforms in [0, 1) from the caller).  scratch: at least
 * tqk_sample_scratch_bytes(bsz, n) bytes of device memory. */
int64_t tqk_sample_scratch_bytes(int64_t bsz, int n);
int tqk_sample(const void* state, int64_t bsz, int n, const double* uniforms, int64_t shots, int64_t* out,
               void* scratch, int64_t scratch_bytes, void* stream);

/* Expectation values of m Pauli strings, out[b*m + j] = Re <psi_b| P_j |psi_b> (float64).
 * P_j is given by bit masks over the in-row index (bit n-1-w <-> wire w):
 * xmask = X|Y positions, zmask = Z|Y positions; the i^(#Y) factor is applied.
 * Replaces expval_joint_analytical (measurement/measurements.py:232-279), which
 * builds a dense 2^n x 2^n kron Hamiltonian.  Deterministic (fixed-order reduction).
 * Strings sharing one X-mask: one pass per 8 strings.  Several X-masks: strings are
 * grouped (in order, up to 8 per group, while the group's X-masks span at most
 * 13 - c dimensions above c contiguous low bits, c >= 4) and each group is one pass over
 * cosets of that span staged in shared memory.  status: device int; TQK_TIMEOUT is
 * written there (and the affected expvals are NaN) if a staged load did not complete. */
int64_t tqk_pauli_expval_scratch_bytes(int64_t bsz, int n, int m);
int tqk_pauli_expval(const void* state, int64_t bsz, int n, const uint64_t* xmask,
                     const uint64_t* zmask, int m, double* out, void* scratch,
                     int64_t scratch_bytes, int* status, void* stream);

/* Same result as tqk_pauli_expval, without caller scratch: the block partials live in
 * a 1 MiB array inside libtqk.so (one per device, shared by every call), so the call
 * allocates nothing.  For callers that cannot allocate: a host binding this C ABI over
 * FFI that holds only raw pointers to its own buffers and has no device allocator, or
 * a service held to a fixed device-memory budget.  No counterpart in the upstream
 * project.  Limits: its partials, bsz * min(ceil(1216 / bsz), ceil(2^n / 1024)) * 64
 * bytes (one pass per distinct X-mask), must fit tqk_pauli_expval_noalloc_capacity()
 * bytes (1 MiB: up to bsz = 16384 at n <= 10, bsz = 1216 at any n) and m <= 4096, else
 * TQK_SCRATCH_TOO_SMALL / TQK_BAD_SHAPE.  Calls that overlap on the GPU race on the
 * shared array.  The first call on a device looks up the array's address
 * (cudaGetSymbolAddress, device current) and caches it per CUDA context; make that
 * first call before any stream capture (and again after a device reset). */
int64_t tqk_pauli_expval_noalloc_capacity(void);
int tqk_pauli_expval_noalloc(const void* state, int64_t bsz, int n, const uint64_t* xmask,
                             const uint64_t* zmask, int m, double* out, void* stream);

/* out = sum_j coef[b*m + j] * P_j psi  (complex64 [bsz, 2^n], not aliasing state; coef
 * float32 device).  The backward of the expvals above (cotangent of psi); the strings
 * are grouped as for tqk_pauli_expval, one coset pass per group (the first writes out,
 * later ones add to it).  status: device int, TQK_TIMEOUT if a staged load did not
 * complete (out is then incomplete). */
int tqk_pauli_apply_sum(const void* state, int64_t bsz, int n, const uint64_t* xmask,
                        const uint64_t* zmask, int m, const float* coef, void* out,
                        int* status, void* stream);

/* ---------------------------------------------------------------- adjoint backward
 * One reverse step of the adjoint method for a gate applied with the matching forward
 * entry point above: psi <- U^H psi (or psi <- uncompute psi when `uncompute` is not
 * NULL: the exact inverse, for gates that are not unitary such as upstream's cu2),
 * lam <- U^H lam, and (if grad != NULL)
 * grad[g] += sum over the gate's amplitude groups of lam_after * conj(psi_before)^T,
 * accumulated in float64 (complex128 interleaved), g = batch row if the operand is
 * per-row else 0.  Replaces the autograd graph of torch.bmm/permute recorded by
 * apply_unitary_bmm (gate_wrapper.py:127-138).  grad must be zeroed by the caller. */
int tqk_adjoint_matrix(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires, int k,
                       const void* mat, int64_t mat_batch, const void* uncompute, double* grad,
                       void* stream);
int tqk_adjoint_controlled(void* psi, void* lam, int64_t bsz, int n, const int32_t* controls,
                           int nc, const int32_t* targets, int kt, const void* mat,
                           int64_t mat_batch, const void* uncompute, double* grad, void* stream);
int tqk_adjoint_phase(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires, int k,
                      const void* phase, int64_t phase_batch, double* grad, void* stream);
int tqk_adjoint_diagonal(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires, int k,
                         const void* diag, int64_t diag_batch, double* grad, void* stream);

/* ---------------------------------------------------------------- fused blocks (tensor cores)
 * A fused 6-wire block (64x64 complex U) applied to every column of the state as one
 * tcgen05 GEMM with split-BF16 operands (hi.hi + hi.lo + lo.hi, fp32 accumulate).
 * Replaces the per-block dense bmm of upstream static mode: QuantumGraph.apply_unitary
 * (graph/graphs.py:836-860) -> qubitunitaryfast (functional/qubit_unitary.py:143).
 *
 * tqk_fused_prepare converts U (complex128 [u_batch, 64, 64], row-major, rows = output
 * pattern, wires[0] the most significant bit) into the operand image the kernel reads
 * (tqk_fused_image_bytes(u_batch) bytes, 16-byte aligned).  The image is laid out for
 * the block's target bits: pass the same 6 wires (in the same order) that the image
 * will be applied on; only their relative order matters.  tqk_fused_apply needs
 * n >= 13; u_batch is 1 or bsz.  `status` is a device int: the kernel writes
 * TQK_TIMEOUT there if one of its bounded waits gives up (it then stops early). */
int64_t tqk_fused_image_bytes(int64_t u_batch);
int tqk_fused_prepare(const void* u, int64_t u_batch, const int32_t* wires, void* image, void* stream);
/* The image of U^H, built directly from U (what tqk_fused_prepare of U^H would give). */
int tqk_fused_prepare_adjoint(const void* u, int64_t u_batch, const int32_t* wires, void* image, void* stream);
/* One operand image for tqk_fused_prepare_many: the image of U (adjoint == 0) or of U^H
 * (adjoint != 0), U complex128 [u_batch][64][64], laid out for `wires` as in
 * tqk_fused_prepare; `image` holds tqk_fused_image_bytes(u_batch) bytes, 16-byte aligned. */
typedef struct {
  const void* u;
  void* image;
  int64_t u_batch;
  int32_t wires[6];
  int32_t adjoint;
  int32_t pad;
} tqk_image_job; /* 56 bytes */
/* Builds njobs images in one launch.  `jobs` is a DEVICE array (read by the kernel);
 * max_u_batch >= every job's u_batch. */
int tqk_fused_prepare_many(const tqk_image_job* jobs, int njobs, int64_t max_u_batch, void* stream);
/* One stored-input cotangent for tqk_fused_cross_add_many: gu += M from the cross term mr. */
typedef struct {
  const double* mr; /* [batch][128][128] float64, from tqk_fused_adjoint_stored */
  void* gu;         /* complex128 [batch][64][64] */
  int64_t batch;
} tqk_cross_job;    /* 24 bytes */
/* tqk_fused_cross_grad(mr, NULL, batch, gu) for njobs blocks in one launch; `jobs` is a
 * DEVICE array, max_batch >= every job's batch. */
int tqk_fused_cross_add_many(const tqk_cross_job* jobs, int njobs, int64_t max_batch, void* stream);
/* Block cotangent from an adjoint step: gu[b] += M_b U_b (complex128 [batch, 64, 64]),
 * where M_b is the complex 64 x 64 matrix held by the real cross term mr[b]
 * ([batch, 128, 128] float64 from tqk_fused_adjoint) and U_b the block unitary
 * (complex128 [batch, 64, 64]); the product runs in float32, the sum in float64.
 * u == NULL: gu[b] += M_b (the cross term of tqk_fused_adjoint_stored, taken against the
 * block's input state, is the cotangent itself). */
int tqk_fused_cross_grad(const double* mr, const void* u, int64_t batch, void* gu, void* stream);
int tqk_fused_apply(void* state, int64_t bsz, int n, const int32_t* wires, const void* image,
                    int64_t u_batch, int* status, void* stream);
/* Out-of-place tqk_fused_apply: state_out = U state_in, state_in unchanged.  The two
 * buffers are the same (in place) or do not overlap.  A forward that writes every
 * block's output to a new buffer keeps each block's input state for
 * tqk_fused_adjoint_stored. */
int tqk_fused_apply_to(const void* state_in, void* state_out, int64_t bsz, int n, const int32_t* wires,
                       const void* image, int64_t u_batch, int* status, void* stream);

/* A fused block applied to |0...0>: `state` holds exactly |0...0> in every row; row b's
 * amplitude at the block's pattern j (wires[0] the pattern's most significant bit, every
 * other bit clear) becomes U_b[j][0] rounded to complex64 (u: complex128 [u_batch][64][64]),
 * which is U |0...0> without a pass over the state.  The block's reverse step is then
 * skipped: its cotangent is lam conj(e_0)^T, lam read at the same 64 offsets. */
int tqk_fused_zero_input(void* state, int64_t bsz, int n, const int32_t* wires, const void* u, int64_t u_batch,
                         void* stream);
/* Adjoint step of a fused block on the tensor cores: psi <- U^H psi, lam <- U^H lam
 * (image_h = tqk_fused_prepare of U^H on the same wires), and, if mr_out != NULL, the real cross term
 * mr_out[g][2j+p][2j'+q] += sum over columns of Re/Im parts lam_{j,p} * psi_{j',q}
 * (float64, g = batch row if u_batch == bsz > 1 else 0; zeroed by the caller), from
 * which M[j][j'] = sum lam[j] conj(psi[j']) and the cotangent of U, M U, follow.
 * Replaces the autograd graph upstream records for the block's bmm. */
int tqk_fused_adjoint(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires,
                      const void* image_h, int64_t u_batch, double* mr_out, int* status,
                      void* stream);
/* Adjoint step of a fused block whose input state is still stored: psi_in = the state
 * the block was applied to (read only), lam <- U^H lam in place, and, if mr_out != NULL,
 * the real cross term of lam (before the step) against psi_in in the layout of
 * tqk_fused_adjoint, from which the cotangent of U is M itself (tqk_fused_cross_grad
 * with u = NULL).  Reads two states and writes one, where tqk_fused_adjoint writes two. */
int tqk_fused_adjoint_stored(const void* psi_in, void* lam, int64_t bsz, int n, const int32_t* wires,
                             const void* image_h, int64_t u_batch, double* mr_out, int* status, void* stream);

/* ---------------------------------------------------------------- gate programs
 * Parameterised gates whose operand the GPU builds from the parameters in place.
 * Replaces the per-gate torch matrix builders (functional/u3.py:52-77, rx.py:19-46,
 * ry.py:50-67, rz.py:150-172, ...) and their autograd graphs: operands and the analytic
 * derivatives of every operand entry are evaluated in float64. */
enum {
  TQK_G_U3 = 0, TQK_G_RX = 1, TQK_G_RY = 2, TQK_G_RZ = 3, TQK_G_PHASE = 4, TQK_G_ROT = 5,
  TQK_G_U2 = 6, TQK_G_R = 7, TQK_G_CRX = 8, TQK_G_CRY = 9, TQK_G_CRZ = 10, TQK_G_CU3 = 11,
  TQK_G_CU1 = 12, TQK_G_CROT = 13, TQK_G_CU = 14, TQK_G_RZZ = 15, TQK_G_RXX = 16,
  TQK_G_RYY = 17, TQK_G_RZX = 18, TQK_G_SINGLEEXC = 19
};
/* op kinds (operand shapes) inside fused blocks */
enum { TQK_K_DENSE = 0, TQK_K_CTRL = 1, TQK_K_X = 2, TQK_K_PHASE = 3, TQK_K_DIAG = 4, TQK_K_SWAP = 5 };

typedef struct {
  int32_t type;          /* TQK_G_* */
  int32_t inverse;       /* operand is the conjugate transpose (conjugate for diagonals) */
  int32_t batch;         /* operand rows: 1 (broadcast) or bsz */
  int32_t nparam;
  const void* p;         /* parameter (row 0, column 0), float32 or float64, read in place */
  int64_t p_row_stride;  /* elements between rows (0 when batch == 1) */
  int64_t p_col_stride;  /* elements between parameters of a row */
  int32_t p_is_double;
  int32_t pad0;
  void* op128;           /* out: complex128 operand [batch][size], or NULL */
  void* op64;            /* out: complex64 operand [batch][size], or NULL */
  const void* op_grad;   /* in (tqk_param_grads): complex128 operand cotangent [batch][size] */
  double* grad;          /* float64 buffer laid out like the parameters (same strides), or NULL */
} tqk_gate_desc;

typedef struct {
  int32_t kind;          /* TQK_K_* */
  int32_t nw;            /* wires of the op (controls first, then targets) */
  int32_t pos[6];        /* row-index bit of each op wire inside the block */
  int32_t nctrl;
  int32_t ctrl_val;
  int32_t batch;         /* operand rows: 1 or bsz */
  int32_t op_size;       /* complex entries per operand row */
  const void* operand;   /* complex128 [batch][op_size] */
  void* grad;            /* complex128 operand cotangent (atomically accumulated), or NULL */
} tqk_block_op;

typedef struct {
  int32_t first_op, num_ops;
  int32_t k;             /* block width (<= 6): U is 2^k x 2^k, block wire i <-> row bit k-1-i */
  int32_t batch;         /* 1 or bsz */
  void* u;               /* complex128 [batch][2^k][2^k] */
  const void* gu;        /* complex128 dL/dU, same layout, or NULL */
} tqk_block_desc;

int tqk_gate_operand_size(int type);
/* gates[ngates] (device array): write every gate's operand (op128 and/or op64). */
int tqk_gate_operands(const tqk_gate_desc* gates, int ngates, void* stream);
/* grad[...] += d loss / d param for every gate with grad != NULL, from op_grad. */
int tqk_param_grads(const tqk_gate_desc* gates, int ngates, void* stream);
/* U = G_m ... G_1 per (block, batch row) in float64; replaces upstream static mode's
 * block unitary construction (graph/graphs.py:712-792).  The tables are device memory and
 * are not read on the host: a block with k outside 1..6, or an op outside its limits
 * (1..6 wires, positions below k, dense / controlled parts of 1 or 2 targets, operand rows
 * of at least the entries its kind reads), is skipped by the kernel (U not written / the
 * op not applied), never indexed out of bounds. */
int tqk_block_build(const tqk_block_desc* blocks, int nblocks, int max_batch, const tqk_block_op* ops,
                    void* stream);
/* From dL/dU (desc.gu) and U (desc.u): every op's operand cotangent, atomically added
 * into op.grad (ops with grad == NULL are skipped). */
int tqk_block_unbuild(const tqk_block_desc* blocks, int nblocks, int max_batch,
                      const tqk_block_op* ops, void* stream);

/* ---------------------------------------------------------------------------------
 * Staged low-qubit runs (plain method).  Upstream applies every gate as its own
 * permute + bmm pass (functional/gate_wrapper.py:96-140); tqk_staged_apply applies a run
 * of up to TQK_STAGED_MAX_OPS consecutive ops whose targets lie in the lowest tile_bits
 * bits of the amplitude index (wires n - tile_bits .. n - 1) in ONE pass: each CTA loads
 * contiguous tiles of 2^tile_bits amplitudes of a batch row into shared memory (128-bit
 * loads), applies the ops in order there, and writes the tiles back.  Controls, phase
 * wires and diagonal wires may be anywhere.  tqk_staged_adjoint is the matching reverse
 * step of the adjoint method on (psi, lam): ops in reverse order, psi <- U^H psi,
 * lam <- U^H lam, and for every op with a grad slot the operand cotangent
 * sum lam_in conj(psi_out) added in float64 (as tqk_adjoint_matrix / _phase / _diagonal
 * do for one op).  Ops whose uncompute is not U^H (non-unitary) must not be staged. */
enum { TQK_S_DENSE1 = 0, TQK_S_X = 1, TQK_S_PHASE = 2, TQK_S_DIAG = 3 };
enum { TQK_STAGED_MAX_OPS = 64, TQK_STAGED_MAX_TILE_BITS = 12, TQK_STAGED_MAX_WIRES = 8 };

typedef struct {
  int32_t kind;        /* TQK_S_DENSE1: 2x2 on wires[nwires-1] where every control wires[0..nwires-1)
                          is 1;  TQK_S_X: flip wires[nwires-1] where every control equals ctrl_val;
                          TQK_S_PHASE: multiply by a phase where every wire is 1;
                          TQK_S_DIAG: diagonal (2^nwires entries, nwires <= 2, wires[0] = MSB) */
  int32_t nwires;      /* 1..TQK_STAGED_MAX_WIRES */
  int32_t wires[TQK_STAGED_MAX_WIRES];
  int32_t ctrl_val;    /* X only: 1 or 0 */
  int32_t pad;
  const void* operand; /* complex64: DENSE1 [batch][2][2], PHASE [batch], DIAG [batch][2^nwires]; X: NULL */
  int64_t batch;       /* 1 (shared by every row) or bsz */
  double* grad;        /* adjoint only: complex128 cotangent of the operand (interleaved, same shape
                          as the operand), or NULL */
} tqk_staged_op; /* 72 bytes */

/* status: device int; TQK_TIMEOUT is written there if a tile's bulk load (TMA) did not
 * complete within ~2 s (the pass then stops early). */
int tqk_staged_apply(void* state, int64_t bsz, int n, const tqk_staged_op* ops, int nops, int tile_bits,
                     int* status, void* stream);
int tqk_staged_adjoint(void* psi, void* lam, int64_t bsz, int n, const tqk_staged_op* ops, int nops,
                       int tile_bits, int* status, void* stream);

/* ---------------------------------------------------------------- persistent circuit batches
 * Many independent circuits of different sizes (n <= 24) in one launch.  tqk_batch_plan
 * splits each circuit into passes whose target bits fit a tile of 2^tile_bits amplitudes
 * (tile_bits 10..14) held in shared memory (circuits with n <= tile_bits: one pass, one
 * tile, never touching HBM; larger ones stream their state, states + state_off, once per
 * pass).  tqk_batch_items lists the
 * work: one item per (circuit, pass, tile), in waves of pass index, so a pass's tiles run
 * on many SMs at once.  One persistent CTA per SM takes items in order; an item of pass
 * p > 0 first waits (bounded) until every tile of pass p - 1 of its circuit is done.
 * Outputs <Z_{z_wire}> per circuit (float64) and, if t_done != NULL, each circuit's
 * completion time (globaltimer ns; t_done[ncirc] = the launch's start).  Upstream runs
 * such batches as a Python loop over circuits, each gate a torch bmm
 * (functional/gate_wrapper.py:96-140). */
enum { TQK_B_DENSE1 = 0, TQK_B_CTRL1 = 1, TQK_B_CZ = 2, TQK_B_CZ_LADDER = 3 };
enum { TQK_BATCH_TILE_BITS = 14, TQK_BATCH_MAX_QUBITS = 24 };

typedef struct {
  int32_t kind;  /* TQK_B_* */
  int32_t w0;    /* DENSE1: target; CTRL1: control; CZ: first wire; CZ_LADDER: first wire */
  int32_t w1;    /* CTRL1: target; CZ: second wire; CZ_LADDER: last wire (CZ on (w, w+1), w0 <= w < w1) */
  int32_t mat;   /* DENSE1 / CTRL1: index of a row-major 2x2 complex64 matrix in `mats` */
} tqk_batch_op; /* 16 bytes */

typedef struct {
  int32_t n;          /* qubits, 1..TQK_BATCH_MAX_QUBITS */
  int32_t z_wire;     /* output <Z> on this wire */
  int32_t first_op;   /* ops[first_op .. first_op + num_ops) */
  int32_t num_ops;
  int64_t state_off;  /* amplitude offset of the circuit's state in `states`; -1 for none
                         (allowed only for single-pass circuits without written states) */
  int32_t first_pass; /* written by tqk_batch_plan */
  int32_t num_passes; /* written by tqk_batch_plan */
} tqk_batch_circuit; /* 32 bytes */

typedef struct {
  int32_t first_op;   /* into the planned op array */
  int32_t num_ops;
  uint32_t tile_mask; /* amplitude-index bits inside the tile (min(n, tile_bits) of them) */
  int32_t flags;      /* 1: first pass (starts from |0..0>), 2: last pass (reduces <Z>) */
} tqk_batch_pass; /* 16 bytes */

typedef struct {
  int32_t circuit;    /* index into circuits */
  int32_t pass;       /* index into passes (a pass of that circuit) */
  int32_t tile;       /* 0 .. 2^(n - popcount(tile_mask)) - 1 */
  int32_t pad;
} tqk_batch_item; /* 16 bytes */

typedef struct {
  int32_t tile_bits;   /* 10..14: tile of 2^tile_bits amplitudes; must equal the plan's */
  int32_t threads;     /* threads per CTA: 128, 256 or 512 */
  int32_t ctas_per_sm; /* persistent CTAs per SM, 1..8 (clamped to what fits) */
  int32_t pad;
} tqk_batch_config; /* 16 bytes; NULL = {14, 512, 1} */

/* Host only (no GPU work): validate `circuits` and their ops (matrix indices < n_mats),
 * write each circuit's passes into passes[0 .. return value) and its ops, regrouped by
 * pass (ops that commute may move across passes), into ops_out at the same positions;
 * fills first_pass/num_passes.  Returns the number of passes, or -TQK_* on error
 * (-TQK_SCRATCH_TOO_SMALL if more than max_passes are needed). */
int tqk_batch_plan(tqk_batch_circuit* circuits, int ncirc, const tqk_batch_op* ops_in, int n_mats,
                   tqk_batch_op* ops_out, tqk_batch_pass* passes, int max_passes, int tile_bits);
/* Host only: the work items of planned circuits in dispatch order (wave w = every
 * circuit's w-th pass, circuits in array order, tiles ascending); returns their number,
 * or -TQK_SCRATCH_TOO_SMALL if more than max_items. */
int64_t tqk_batch_items(const tqk_batch_circuit* circuits, int ncirc, const tqk_batch_pass* passes,
                        tqk_batch_item* items, int64_t max_items);
/* Device arrays: circuits (planned), ops (= ops_out of the plan), passes, items, mats
 * (complex64 [*, 2, 2]), states (complex64; may be NULL if no circuit needs one),
 * z_out[ncirc], pass_done[npasses] and counter (one int) all zeroed by the caller before
 * each launch, t_done[ncirc + 1] or NULL, status (device int; TQK_TIMEOUT if a wait gave
 * up, TQK_BAD_SHAPE if a pass is wider than config->tile_bits).  write_states != 0 stores
 * every final state.  config: tile size (the one the plan used), CTA shape and CTAs per
 * SM (host-side autotuning picks them); NULL for the defaults.  The launch is a single
 * kernel on `stream` with no host synchronisation, so it can be captured in a CUDA
 * graph once a first launch of the same variant has run on the device uncaptured. */
int tqk_batch_run(const tqk_batch_circuit* circuits, int ncirc, const tqk_batch_op* ops,
                  const tqk_batch_pass* passes, const tqk_batch_item* items, int64_t n_items,
                  const void* mats, void* states, int write_states, double* z_out, int* pass_done,
                  uint64_t* t_done, int* counter, int* status, const tqk_batch_config* config,
                  void* stream);

/* ---------------------------------------------------------------- compiled segments
 * The tape-level entry points: a compiled gate run (a segment of the tape: plain ops,
 * staged low-qubit runs and fused blocks, in forward order) applied and reversed with
 * one call each.  Together they replace the per-gate dispatch of upstream's
 * gate_wrapper (functional/gate_wrapper.py:324-446, each gate an apply_unitary_bmm,
 * :96-140), static mode's block application (graph/graphs.py:836-860) and the autograd
 * graph both record.  The table lives in HOST memory; every operand, image, state and
 * cotangent it points to is device memory the caller owns (the entry points allocate
 * nothing: block outputs and the reverse sweep's working state are caller buffers).
 * The other steps of a training step are single calls too: operands (tqk_gate_operands),
 * block unitaries (tqk_block_build), operand images (tqk_fused_prepare_many), expvals
 * and the backward seed (tqk_pauli_expval, tqk_pauli_apply_sum), then after the reverse
 * sweep the stored-input block cotangents (tqk_fused_cross_add_many), the member
 * operand cotangents (tqk_block_unbuild) and the parameter gradients (tqk_param_grads). */
enum {
  TQK_X_DENSE = 0,       /* dense U on wires[0..nw) (tqk_apply_matrix); operand [batch][2^nw][2^nw] */
  TQK_X_CTRL = 1,        /* controlled block: controls wires[0..nctrl), targets the rest */
  TQK_X_MCX = 2,         /* multi-controlled X: controls wires[0..nctrl) == ctrl_val, target wires[nctrl] */
  TQK_X_PHASE = 3,       /* phase on amplitudes whose wires are all 1; operand [batch] */
  TQK_X_DIAG = 4,        /* diagonal; operand [batch][2^nw] */
  TQK_X_SWAP = 5,        /* controlled swap of wires[nctrl], wires[nctrl + 1] */
  TQK_X_STAGED = 6,      /* staged run: `staged[0..nstaged)` in one shared-memory pass */
  TQK_X_BLOCK_TC = 7,    /* fused 6-wire block on the tensor cores: image / image_h */
  TQK_X_BLOCK_DENSE = 8, /* fused block on the CUDA cores: operand = U (complex64) */
  TQK_X_BLOCK_ZERO = 9   /* fused 6-wire block applied to |0...0> (tqk_fused_zero_input, u = U):
                            forward only; in the reverse table it must carry skip_reverse */
};
typedef struct {
  int32_t kind;            /* TQK_X_* */
  int32_t nw;              /* wires used (controls first) */
  int32_t nctrl;
  int32_t ctrl_val;
  int32_t wires[TQK_MAX_OP_WIRES];
  int64_t batch;           /* operand / block batch: 1 or bsz */
  const void* operand;     /* complex64 operand (DENSE, CTRL, PHASE, DIAG, BLOCK_DENSE) */
  const void* uncompute;   /* DENSE / CTRL: exact inverse for psi (non-unitary gates), or NULL */
  const void* image;       /* BLOCK_TC forward image (tqk_fused_prepare of U) */
  const void* image_h;     /* BLOCK_TC reverse image (of U^H) */
  const void* u;           /* BLOCK_TC: U, complex128 [batch][64][64] (in-place reverse step's M U);
                              BLOCK_ZERO: the same U, whose column 0 the op writes */
  void* out;               /* BLOCK_TC forward: the block's output buffer (its input is then kept
                              as the stored input), or NULL to apply in place */
  const void* stored;      /* BLOCK_TC reverse: the block's stored input, or NULL (uncompute) */
  double* grad;            /* reverse: operand / block cotangent (complex128 interleaved), or NULL */
  double* mr;              /* BLOCK_TC reverse with grad: cross-term buffer [batch][128][128] float64,
                              zeroed; a stored-input step leaves M there (add it with
                              tqk_fused_cross_add_many), an in-place step adds M U to grad */
  const tqk_staged_op* staged; /* STAGED: the run's ops (their grad slots are used in reverse) */
  int32_t nstaged;
  int32_t tile_bits;       /* STAGED */
  int32_t skip_reverse;    /* the reverse sweep stops before this op (it must be op 0: a first block
                              on |0...0>, whose cotangent the caller takes from lam) */
  int32_t pad;
} tqk_exec_op;             /* 184 bytes */

/* Optional per-op callback of the runners: called on the calling thread just before
 * (after == 0) and just after (after == 1) the launches of op `index` are enqueued, e.g.
 * to record CUDA events around one kind of kernel on the stream. */
typedef void (*tqk_exec_hook)(int index, int kind, int after, void* user);

/* Forward: apply ops[0..nops) to `state` ([bsz, 2^n] complex64).  A BLOCK_TC op with `out`
 * writes its result there and the sweep continues on `out`; *final receives the buffer
 * holding the result (state, or the last such out).  *launches (optional) receives the
 * number of kernels launched; hook may be NULL. */
int tqk_segment_forward(void* state, int64_t bsz, int n, const tqk_exec_op* ops, int nops, int* status,
                        void** final, int64_t* launches, tqk_exec_hook hook, void* user, void* stream);
/* Reverse sweep of the adjoint method: psi_end is the segment's result (read only), lam
 * the cotangent there (updated in place to the cotangent at the segment's start).  Ops
 * are reversed last to first: a BLOCK_TC op with `stored` reads its stored input and
 * moves the sweep's state to it; any other op uncomputes the state in place, on
 * `work` (a caller buffer of one state) after a copy when the sweep's state is read only
 * (psi_end or a stored input); work == psi_end lets the sweep uncompute the result in
 * place.  Operand cotangents accumulate into each op's grad.  *start (optional) receives
 * where the sweep's state ended: the state at the segment's start (work, psi_end or a
 * stored input); *launches (optional): kernels and copies launched; hook may be NULL. */
int tqk_segment_backward(const void* psi_end, void* lam, void* work, int64_t bsz, int n, const tqk_exec_op* ops,
                         int nops, int* status, const void** start, int64_t* launches, tqk_exec_hook hook,
                         void* user, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* TQK_H_ */
