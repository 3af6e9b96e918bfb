// segment.cu -- the tape-level entry points: a compiled segment (plain ops, staged runs,
// fused blocks) applied forward and reversed by the adjoint method with one call each.
//
// Host code only: the runner walks a host table of tqk_exec_op records and launches
// each op's kernel through the per-op entry points, on one stream, with no
// synchronisation and no allocation.  The reverse sweep's state is a cursor: it starts at
// the segment's result (read only), moves to a block's stored input after that block's
// reverse step (read only), and is copied into the caller's work buffer the first time an
// op has to uncompute it in place after such a move -- so neither the result nor a stored
// input is ever written, and a second sweep over the same segment gives the same values.
#include <cuda_runtime.h>

#include "common.cuh"

namespace tqk {
namespace {

struct Cursor {
  const void* state;  // where the sweep's state is
  void* work;         // caller buffer of one state
  size_t bytes;
  bool owned;         // the state is the work buffer (writable)
  cudaStream_t st;
  int64_t* launches;
  // the state, made writable: copied into the work buffer if it is read only
  int writable(void** out, const char* what) {
    if (!owned) {
      if (work == nullptr) return fail(TQK_BAD_POINTER, "%s: a reverse step needs the work buffer", what);
      if (state != work) {
        const cudaError_t e = cudaMemcpyAsync(work, state, bytes, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return fail(TQK_CUDA_ERROR, "%s: state copy failed: %s", what, cudaGetErrorString(e));
        ++*launches;
      }
      state = work;
      owned = true;
    }
    *out = work;
    return TQK_OK;
  }
};

int check_op(const tqk_exec_op& op, int i, const char* what) {
  if (op.nw < 0 || op.nw > TQK_MAX_OP_WIRES || op.nctrl < 0 || op.nctrl > op.nw)
    return fail(TQK_BAD_SHAPE, "%s: op %d has nw=%d, nctrl=%d", what, i, op.nw, op.nctrl);
  switch (op.kind) {
    case TQK_X_STAGED:
      if (op.staged == nullptr || op.nstaged <= 0) return fail(TQK_BAD_POINTER, "%s: op %d: empty staged run", what, i);
      return TQK_OK;
    case TQK_X_BLOCK_TC:
      if (op.nw != 6) return fail(TQK_BAD_SHAPE, "%s: op %d: a tensor-core block has 6 wires", what, i);
      if (op.grad != nullptr && (op.mr == nullptr || (op.stored == nullptr && op.u == nullptr)))
        return fail(TQK_BAD_POINTER, "%s: op %d: a block cotangent needs mr (and u without a stored input)", what,
                    i);
      return TQK_OK;
    case TQK_X_BLOCK_ZERO:
      if (op.nw != 6 || op.u == nullptr)
        return fail(TQK_BAD_SHAPE, "%s: op %d: a zero-input block has 6 wires and its U", what, i);
      return TQK_OK;
    case TQK_X_MCX:
      if (op.nw != op.nctrl + 1) return fail(TQK_BAD_SHAPE, "%s: op %d: MCX has one target", what, i);
      return TQK_OK;
    case TQK_X_SWAP:
      if (op.nw != op.nctrl + 2) return fail(TQK_BAD_SHAPE, "%s: op %d: SWAP has two targets", what, i);
      return TQK_OK;
    case TQK_X_DENSE:
    case TQK_X_CTRL:
    case TQK_X_PHASE:
    case TQK_X_DIAG:
    case TQK_X_BLOCK_DENSE:
      return TQK_OK;
    default:
      return fail(TQK_BAD_SHAPE, "%s: op %d has unknown kind %d", what, i, op.kind);
  }
}

}  // namespace
}  // namespace tqk

using namespace tqk;

extern "C" int tqk_segment_forward(void* state, int64_t bsz, int n, const tqk_exec_op* ops, int nops, int* status,
                                   void** final, int64_t* launches, tqk_exec_hook hook, void* user, void* stream) {
  const char* what = "tqk_segment_forward";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (nops < 0 || (nops > 0 && ops == nullptr)) return fail(TQK_BAD_POINTER, "%s: null op table", what);
  if (status == nullptr) return fail(TQK_BAD_POINTER, "%s: null status word", what);
  int64_t count = 0;
  void* cur = state;
  for (int i = 0; i < nops; ++i) {
    const tqk_exec_op& op = ops[i];
    if ((rc = check_op(op, i, what))) return rc;
    const int32_t* w = op.wires;
    if (hook) hook(i, op.kind, 0, user);
    switch (op.kind) {
      case TQK_X_DENSE:
      case TQK_X_BLOCK_DENSE:
        rc = tqk_apply_matrix(cur, bsz, n, w, op.nw, op.operand, op.batch, stream);
        break;
      case TQK_X_CTRL:
        rc = tqk_apply_controlled(cur, bsz, n, w, op.nctrl, w + op.nctrl, op.nw - op.nctrl, op.operand, op.batch,
                                  stream);
        break;
      case TQK_X_MCX:
        rc = tqk_apply_mcx(cur, bsz, n, w, op.nctrl, op.ctrl_val, w[op.nctrl], stream);
        break;
      case TQK_X_PHASE:
        rc = tqk_apply_phase(cur, bsz, n, w, op.nw, op.operand, op.batch, stream);
        break;
      case TQK_X_DIAG:
        rc = tqk_apply_diagonal(cur, bsz, n, w, op.nw, op.operand, op.batch, stream);
        break;
      case TQK_X_SWAP:
        rc = tqk_apply_swap(cur, bsz, n, w, op.nctrl, w[op.nctrl], w[op.nctrl + 1], stream);
        break;
      case TQK_X_STAGED:
        rc = tqk_staged_apply(cur, bsz, n, op.staged, op.nstaged, op.tile_bits, status, stream);
        break;
      case TQK_X_BLOCK_TC:
        if (op.out != nullptr) {
          rc = tqk_fused_apply_to(cur, op.out, bsz, n, w, op.image, op.batch, status, stream);
          cur = op.out;
        } else {
          rc = tqk_fused_apply(cur, bsz, n, w, op.image, op.batch, status, stream);
        }
        break;
      case TQK_X_BLOCK_ZERO:
        rc = tqk_fused_zero_input(cur, bsz, n, w, op.u, op.batch, stream);
        break;
    }
    if (rc) return rc;
    if (hook) hook(i, op.kind, 1, user);
    ++count;
  }
  if (final) *final = cur;
  if (launches) *launches = count;
  return TQK_OK;
}

extern "C" int tqk_segment_backward(const void* psi_end, void* lam, void* work, int64_t bsz, int n,
                                    const tqk_exec_op* ops, int nops, int* status, const void** start,
                                    int64_t* launches, tqk_exec_hook hook, void* user, void* stream) {
  const char* what = "tqk_segment_backward";
  int rc = check_state(psi_end, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(lam, bsz, n, what))) return rc;
  if (work != nullptr && (rc = check_state(work, bsz, n, what))) return rc;
  if (nops < 0 || (nops > 0 && ops == nullptr)) return fail(TQK_BAD_POINTER, "%s: null op table", what);
  if (status == nullptr) return fail(TQK_BAD_POINTER, "%s: null status word", what);
  for (int i = 0; i < nops; ++i)
    if ((rc = check_op(ops[i], i, what))) return rc;
  for (int i = 1; i < nops; ++i)
    if (ops[i].skip_reverse) return fail(TQK_BAD_SHAPE, "%s: only op 0 may skip the reverse sweep", what);
  for (int i = 0; i < nops; ++i)
    if (ops[i].kind == TQK_X_BLOCK_ZERO && !ops[i].skip_reverse)
      return fail(TQK_BAD_SHAPE, "%s: op %d: a zero-input block has no reverse step (set skip_reverse)", what, i);
  int64_t count = 0;
  cudaStream_t st = as_stream(stream);
  Cursor psi{psi_end, work, static_cast<size_t>(bsz) * (static_cast<size_t>(8) << n), false, st, &count};
  if (work == psi_end) psi.owned = true;  // the caller lets the sweep write the result in place
  for (int i = nops - 1; i >= 0; --i) {
    const tqk_exec_op& op = ops[i];
    if (op.skip_reverse) break;
    const int32_t* w = op.wires;
    void* p = nullptr;
    if (op.kind == TQK_X_BLOCK_TC && op.stored != nullptr) {
      if (hook) hook(i, op.kind, 0, user);
      rc = tqk_fused_adjoint_stored(op.stored, lam, bsz, n, w, op.image_h, op.batch, op.grad ? op.mr : nullptr,
                                    status, stream);
      if (rc) return rc;
      if (hook) hook(i, op.kind, 1, user);
      ++count;
      psi.state = op.stored;
      psi.owned = false;
      continue;
    }
    if ((rc = psi.writable(&p, what))) return rc;
    if (hook) hook(i, op.kind, 0, user);
    switch (op.kind) {
      case TQK_X_DENSE:
        rc = tqk_adjoint_matrix(p, lam, bsz, n, w, op.nw, op.operand, op.batch, op.uncompute, op.grad, stream);
        break;
      case TQK_X_BLOCK_DENSE:
        rc = tqk_adjoint_matrix(p, lam, bsz, n, w, op.nw, op.operand, op.batch, nullptr, op.grad, stream);
        break;
      case TQK_X_CTRL:
        rc = tqk_adjoint_controlled(p, lam, bsz, n, w, op.nctrl, w + op.nctrl, op.nw - op.nctrl, op.operand,
                                    op.batch, op.uncompute, op.grad, stream);
        break;
      case TQK_X_MCX:
        rc = tqk_apply_mcx(p, bsz, n, w, op.nctrl, op.ctrl_val, w[op.nctrl], stream);
        if (!rc) {
          ++count;
          rc = tqk_apply_mcx(lam, bsz, n, w, op.nctrl, op.ctrl_val, w[op.nctrl], stream);
        }
        break;
      case TQK_X_PHASE:
        rc = tqk_adjoint_phase(p, lam, bsz, n, w, op.nw, op.operand, op.batch, op.grad, stream);
        break;
      case TQK_X_DIAG:
        rc = tqk_adjoint_diagonal(p, lam, bsz, n, w, op.nw, op.operand, op.batch, op.grad, stream);
        break;
      case TQK_X_SWAP:
        rc = tqk_apply_swap(p, bsz, n, w, op.nctrl, w[op.nctrl], w[op.nctrl + 1], stream);
        if (!rc) {
          ++count;
          rc = tqk_apply_swap(lam, bsz, n, w, op.nctrl, w[op.nctrl], w[op.nctrl + 1], stream);
        }
        break;
      case TQK_X_STAGED:
        rc = tqk_staged_adjoint(p, lam, bsz, n, op.staged, op.nstaged, op.tile_bits, status, stream);
        break;
      case TQK_X_BLOCK_TC: {
        double* mr = op.grad ? op.mr : nullptr;
        rc = tqk_fused_adjoint(p, lam, bsz, n, w, op.image_h, op.batch, mr, status, stream);
        if (!rc && mr != nullptr) {  // the in-place step's cotangent is M U
          ++count;
          rc = tqk_fused_cross_grad(mr, op.u, op.batch, op.grad, stream);
        }
        break;
      }
    }
    if (rc) return rc;
    if (hook) hook(i, op.kind, 1, user);
    ++count;
  }
  if (start) *start = psi.state;
  if (launches) *launches = count;
  return TQK_OK;
}
