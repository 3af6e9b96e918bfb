// program.cu -- gate operands from parameters, fused-block unitaries, and their
// backward, all on the GPU in float64.
//
// A recorded circuit is described by plain arrays (include/tqk.h):
//   tqk_gate_desc  one parameterised gate: its type, where its parameters live (any
//                  strided float32/float64 tensor, read in place), where its operand goes;
//   tqk_block_op   one op inside a fused block (kind, bit positions in the block);
//   tqk_block_desc one fused block (its ops, width, batch, where U goes).
// Kernels:
//   k_gate_operands  params -> operands (complex128 and complex64), one gate per block;
//   k_param_grads    operand cotangents -> d loss / d params (analytic derivatives,
//                    atomically added into a float64 buffer laid out like the params);
//   k_block_build    U = G_m ... G_1 for every (block, batch row), 2^k x 2^k in shared memory;
//   k_block_unbuild  the reverse: from dL/dU, every op's operand cotangent
//                    (W <- G_j^H W, X <- G_j^H X, grad_j = sum over the other bits of X W^H).
#include <math.h>

#include "common.cuh"

namespace tqk {
namespace prog {

// Complex scalars: float64 (C2) for operands and block unitaries; float32 (F2) for the
// block unbuild sweeps, whose input cotangent carries complex64 accuracy (partial sums
// go to float64 before any atomic).
template <typename R>
struct CT {
  R x, y;
  using real = R;
};
using C2 = CT<double>;
using F2 = CT<float>;
__device__ __forceinline__ C2 mk(double a, double b) { return C2{a, b}; }
template <typename C>
__device__ __forceinline__ C mkc(double a, double b) {
  return C{static_cast<typename C::real>(a), static_cast<typename C::real>(b)};
}
template <typename C>
__device__ __forceinline__ C cmul2(C a, C b) {
  return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C>
__device__ __forceinline__ C conj2(C a) {
  return C{a.x, -a.y};
}
template <typename C>
__device__ __forceinline__ C cadd2(C a, C b) {
  return C{a.x + b.x, a.y + b.y};
}
__device__ __forceinline__ C2 expi(double t) {
  double s, c;
  sincos(t, &s, &c);
  return C2{c, s};
}
__device__ __forceinline__ C2 scale(C2 a, double s) { return C2{a.x * s, a.y * s}; }
__device__ __forceinline__ C2 mul_i(C2 a) { return C2{-a.y, a.x}; }  // i * a

// Operand size (complex entries) per operand shape.
__host__ __device__ inline int operand_size(int type) {
  switch (type) {
    case TQK_G_RZ: return 2;
    case TQK_G_PHASE: case TQK_G_CU1: return 1;
    case TQK_G_CRZ: case TQK_G_RZZ: return 4;
    case TQK_G_RXX: case TQK_G_RYY: case TQK_G_RZX: case TQK_G_SINGLEEXC: return 16;
    default: return 4;  // 2x2 dense / controlled block
  }
}

__host__ __device__ inline int operand_is_diag(int type) {
  return type == TQK_G_RZ || type == TQK_G_PHASE || type == TQK_G_CU1 || type == TQK_G_CRZ || type == TQK_G_RZZ;
}

// Operand of gate `type` (or its derivative w.r.t. parameter `dk`, dk >= 0) at params p.
__device__ void operand(int type, const double* p, int dk, C2* m) {
  const bool d = dk >= 0;
  switch (type) {
    case TQK_G_U3:
    case TQK_G_CU3:
    case TQK_G_CU: {  // [[c, -e^{il} s], [e^{if} s, e^{i(f+l)} c]] (x e^{ig} for cu)
      const double th = p[0], ph = p[1], la = p[2];
      double s, c;
      sincos(th / 2, &s, &c);
      double a00 = c, a01 = s, a10 = s, a11 = c;  // magnitudes before phases
      if (d && dk == 0) { a00 = -s / 2; a01 = c / 2; a10 = c / 2; a11 = -s / 2; }
      m[0] = mk(a00, 0);
      m[1] = scale(expi(la), -a01);
      m[2] = scale(expi(ph), a10);
      m[3] = scale(expi(ph + la), a11);
      if (d && dk == 1) { m[0] = mk(0, 0); m[1] = mk(0, 0); m[2] = mul_i(m[2]); m[3] = mul_i(m[3]); }
      if (d && dk == 2) { m[0] = mk(0, 0); m[2] = mk(0, 0); m[1] = mul_i(m[1]); m[3] = mul_i(m[3]); }
      if (type == TQK_G_CU) {
        const C2 g = expi(p[3]);
        if (d && dk == 3) {  // d/dgamma of e^{ig} U3 = i e^{ig} U3
          double s2, c2;
          sincos(th / 2, &s2, &c2);
          m[0] = mk(c2, 0);
          m[1] = scale(expi(la), -s2);
          m[2] = scale(expi(ph), s2);
          m[3] = scale(expi(ph + la), c2);
          for (int e = 0; e < 4; ++e) m[e] = mul_i(m[e]);
        }
        for (int e = 0; e < 4; ++e) m[e] = cmul2(m[e], g);
      }
      return;
    }
    case TQK_G_RX:
    case TQK_G_CRX: {
      double s, c;
      sincos(p[0] / 2, &s, &c);
      if (d) { const double t = c; c = -s / 2; s = t / 2; }
      m[0] = mk(c, 0); m[1] = mk(0, -s); m[2] = mk(0, -s); m[3] = mk(c, 0);
      return;
    }
    case TQK_G_RY:
    case TQK_G_CRY: {
      double s, c;
      sincos(p[0] / 2, &s, &c);
      if (d) { const double t = c; c = -s / 2; s = t / 2; }
      m[0] = mk(c, 0); m[1] = mk(-s, 0); m[2] = mk(s, 0); m[3] = mk(c, 0);
      return;
    }
    case TQK_G_RZ: {  // diag(e^{-it/2}, e^{it/2})
      m[0] = expi(-p[0] / 2);
      m[1] = expi(p[0] / 2);
      if (d) { m[0] = scale(mul_i(m[0]), -0.5); m[1] = scale(mul_i(m[1]), 0.5); }
      return;
    }
    case TQK_G_CRZ: {  // diag(1, 1, e^{-it/2}, e^{it/2})
      m[0] = mk(d ? 0 : 1, 0);
      m[1] = mk(d ? 0 : 1, 0);
      m[2] = expi(-p[0] / 2);
      m[3] = expi(p[0] / 2);
      if (d) { m[2] = scale(mul_i(m[2]), -0.5); m[3] = scale(mul_i(m[3]), 0.5); }
      return;
    }
    case TQK_G_RZZ: {  // diag(e^{-it/2}, e^{it/2}, e^{it/2}, e^{-it/2})
      const C2 a = expi(-p[0] / 2), b = expi(p[0] / 2);
      m[0] = a; m[1] = b; m[2] = b; m[3] = a;
      if (d) {
        m[0] = scale(mul_i(a), -0.5); m[3] = m[0];
        m[1] = scale(mul_i(b), 0.5); m[2] = m[1];
      }
      return;
    }
    case TQK_G_PHASE:
    case TQK_G_CU1: {
      m[0] = expi(p[0]);
      if (d) m[0] = mul_i(m[0]);
      return;
    }
    case TQK_G_ROT:
    case TQK_G_CROT: {  // RZ(om) RY(th) RZ(ph): a = (ph+om)/2, dd = (ph-om)/2
      const double ph = p[0], th = p[1], om = p[2];
      double s, c;
      sincos(th / 2, &s, &c);
      const double a = (ph + om) / 2, dd = (ph - om) / 2;
      double c0 = c, s0 = s;
      if (d && dk == 1) { c0 = -s / 2; s0 = c / 2; }
      m[0] = scale(expi(-a), c0);
      m[1] = scale(expi(dd), -s0);
      m[2] = scale(expi(-dd), s0);
      m[3] = scale(expi(a), c0);
      if (d && dk == 0) {
        m[0] = scale(mul_i(m[0]), -0.5); m[1] = scale(mul_i(m[1]), 0.5);
        m[2] = scale(mul_i(m[2]), -0.5); m[3] = scale(mul_i(m[3]), 0.5);
      }
      if (d && dk == 2) {
        m[0] = scale(mul_i(m[0]), -0.5); m[1] = scale(mul_i(m[1]), -0.5);
        m[2] = scale(mul_i(m[2]), 0.5); m[3] = scale(mul_i(m[3]), 0.5);
      }
      return;
    }
    case TQK_G_U2: {  // (1/sqrt2)[[1, -e^{il}], [e^{if}, e^{i(f+l)}]]
      const double r = 0.70710678118654752440;
      m[0] = mk(r, 0);
      m[1] = scale(expi(p[1]), -r);
      m[2] = scale(expi(p[0]), r);
      m[3] = scale(expi(p[0] + p[1]), r);
      if (d && dk == 0) { m[0] = mk(0, 0); m[1] = mk(0, 0); m[2] = mul_i(m[2]); m[3] = mul_i(m[3]); }
      if (d && dk == 1) { m[0] = mk(0, 0); m[2] = mk(0, 0); m[1] = mul_i(m[1]); m[3] = mul_i(m[3]); }
      return;
    }
    case TQK_G_R: {  // [[c, -i e^{-if} s], [-i e^{if} s, c]]
      double s, c;
      sincos(p[0] / 2, &s, &c);
      const C2 em = expi(-p[1]), ep = expi(p[1]);
      if (d && dk == 1) {
        m[0] = mk(0, 0); m[3] = mk(0, 0);
        m[1] = scale(em, -s);
        m[2] = scale(ep, s);
        return;
      }
      if (d) { const double t = c; c = -s / 2; s = t / 2; }
      m[0] = mk(c, 0); m[3] = mk(c, 0);
      m[1] = cmul2(mk(0, -s), em);
      m[2] = cmul2(mk(0, -s), ep);
      return;
    }
    case TQK_G_RXX:
    case TQK_G_RYY:
    case TQK_G_RZX:
    case TQK_G_SINGLEEXC: {
      double s, c;
      sincos(p[0] / 2, &s, &c);
      if (d) { const double t = c; c = -s / 2; s = t / 2; }
      for (int e = 0; e < 16; ++e) m[e] = mk(0, 0);
      const double one = d ? 0.0 : 1.0;
      if (type == TQK_G_RXX) {
        m[0] = m[5] = m[10] = m[15] = mk(c, 0);
        m[3] = m[6] = m[9] = m[12] = mk(0, -s);
      } else if (type == TQK_G_RYY) {
        m[0] = m[5] = m[10] = m[15] = mk(c, 0);
        m[3] = m[12] = mk(0, s);
        m[6] = m[9] = mk(0, -s);
      } else if (type == TQK_G_RZX) {
        m[0] = m[5] = m[10] = m[15] = mk(c, 0);
        m[1] = m[4] = mk(0, -s);
        m[11] = m[14] = mk(0, s);
      } else {
        m[0] = m[15] = mk(one, 0);
        m[5] = m[10] = mk(c, 0);
        m[6] = mk(-s, 0);
        m[9] = mk(s, 0);
      }
      return;
    }
    default:
      return;
  }
}

__device__ __forceinline__ void operand_inverse(int type, C2* m) {
  const int sz = operand_size(type);
  if (operand_is_diag(type)) {
    for (int e = 0; e < sz; ++e) m[e] = conj2(m[e]);
    return;
  }
  const int dim = sz == 16 ? 4 : 2;
  C2 t[16];
  for (int r = 0; r < dim; ++r)
    for (int c = 0; c < dim; ++c) t[r * dim + c] = conj2(m[c * dim + r]);
  for (int e = 0; e < sz; ++e) m[e] = t[e];
}

__device__ __forceinline__ double load_param(const tqk_gate_desc& g, int64_t b, int k) {
  const int64_t idx = b * g.p_row_stride + k * g.p_col_stride;
  return g.p_is_double ? static_cast<const double*>(g.p)[idx] : static_cast<double>(static_cast<const float*>(g.p)[idx]);
}

__global__ void k_gate_operands(const tqk_gate_desc* gates, int ngates) {
  const int gi = blockIdx.x;
  if (gi >= ngates) return;
  const tqk_gate_desc g = gates[gi];
  const int sz = operand_size(g.type);
  for (int64_t b = threadIdx.x; b < g.batch; b += blockDim.x) {
    double p[4];
    for (int k = 0; k < g.nparam && k < 4; ++k) p[k] = load_param(g, b, k);
    C2 m[16];
    operand(g.type, p, -1, m);
    if (g.inverse) operand_inverse(g.type, m);
    double2* o128 = static_cast<double2*>(g.op128) + b * sz;
    float2* o64 = static_cast<float2*>(g.op64) + b * sz;
    for (int e = 0; e < sz; ++e) {
      if (g.op128) o128[e] = make_double2(m[e].x, m[e].y);
      if (g.op64) o64[e] = make_float2(static_cast<float>(m[e].x), static_cast<float>(m[e].y));
    }
  }
}

// dL/dp_k = Re sum_e conj(G_e) dOp_e / dp_k, accumulated into grad buffers shaped like params.
__global__ void k_param_grads(const tqk_gate_desc* gates, int ngates) {
  const int gi = blockIdx.x;
  if (gi >= ngates) return;
  const tqk_gate_desc g = gates[gi];
  if (g.grad == nullptr || g.op_grad == nullptr) return;
  const double2* op_grad = static_cast<const double2*>(g.op_grad);
  const int sz = operand_size(g.type);
  for (int64_t b = threadIdx.x; b < g.batch; b += blockDim.x) {
    double p[4];
    for (int k = 0; k < g.nparam && k < 4; ++k) p[k] = load_param(g, b, k);
    const int64_t o = b * sz;
    for (int k = 0; k < g.nparam; ++k) {
      C2 dm[16];
      operand(g.type, p, k, dm);
      if (g.inverse) operand_inverse(g.type, dm);
      double acc = 0.0;
      for (int e = 0; e < sz; ++e) {
        const double2 G = op_grad[o + e];
        acc += G.x * dm[e].x + G.y * dm[e].y;  // Re(conj(G) dm)
      }
      atomicAdd(g.grad + b * g.p_row_stride + k * g.p_col_stride, acc);
    }
  }
}

// ------------------------------------------------------------------ block build / unbuild
// Rows of a 2^k x 2^k complex128 matrix in shared memory (row-major, ld = D); block wire
// i <-> row bit (k-1-i).  apply_op_rows applies op (or its adjoint) to every column.
template <typename C>
__device__ void apply_op_rows(C* U, int D, const tqk_block_op& op, const double2* opnd, bool adjoint) {
  const int nw = op.nw;
  const int kind = op.kind;
  const int nc = op.nctrl;
  uint32_t cmask = 0, tmask = 0;
  for (int j = 0; j < nc; ++j) cmask |= 1u << op.pos[j];
  for (int j = nc; j < nw; ++j) tmask |= 1u << op.pos[j];
  const uint32_t allmask = cmask | tmask;
  const int tid = threadIdx.x, nth = blockDim.x;
  if (kind == TQK_K_PHASE) {
    C ph = mkc<C>(opnd[0].x, opnd[0].y);
    if (adjoint) ph = conj2(ph);
    for (int e = tid; e < D * D; e += nth) {
      const int r = e / D;
      if ((static_cast<uint32_t>(r) & allmask) == allmask) U[e] = cmul2(ph, U[e]);
    }
  } else if (kind == TQK_K_DIAG) {
    for (int e = tid; e < D * D; e += nth) {
      const int r = e / D;
      int di = 0;
      for (int j = 0; j < nw; ++j) di = (di << 1) | ((r >> op.pos[j]) & 1);
      C dv = mkc<C>(opnd[di].x, opnd[di].y);
      if (adjoint) dv = conj2(dv);
      U[e] = cmul2(dv, U[e]);
    }
  } else if (kind == TQK_K_X) {
    const uint32_t want = op.ctrl_val ? cmask : 0u;
    const uint32_t tb = 1u << op.pos[nw - 1];
    for (int e = tid; e < D * D; e += nth) {
      const int r = e / D, c = e % D;
      if ((static_cast<uint32_t>(r) & tb) == 0 && (static_cast<uint32_t>(r) & cmask) == want) {
        const int r2 = r | tb;
        const C a = U[r * D + c], b2 = U[r2 * D + c];
        U[r * D + c] = b2;
        U[r2 * D + c] = a;
      }
    }
  } else if (kind == TQK_K_SWAP) {
    const uint32_t b0 = 1u << op.pos[nc], b1 = 1u << op.pos[nc + 1];
    for (int e = tid; e < D * D; e += nth) {
      const int r = e / D, c = e % D;
      if ((static_cast<uint32_t>(r) & cmask) == cmask && (r & b0) && !(r & b1)) {
        const int r2 = (r & ~b0) | b1;
        const C a = U[r * D + c], b2 = U[r2 * D + c];
        U[r * D + c] = b2;
        U[r2 * D + c] = a;
      }
    }
  } else {  // dense (all wires targets) or controlled block on the last nw-nc wires
    const int kt = nw - nc;
    const int dt = 1 << kt;
    C M[16];
    for (int a = 0; a < dt; ++a)
      for (int b = 0; b < dt; ++b) {
        const double2 v = adjoint ? opnd[b * dt + a] : opnd[a * dt + b];
        M[a * dt + b] = adjoint ? conj2(mkc<C>(v.x, v.y)) : mkc<C>(v.x, v.y);
      }
    // work item = (column, group of rows sharing all op bits = 0)
    const int groups = D >> nw;
    for (int w = tid; w < groups * D; w += nth) {
      const int c = w % D, g = w / D;
      // insert zeros at the op's bit positions
      uint32_t base = static_cast<uint32_t>(g);
      for (int q = 0; q < 6; ++q) {
        if (allmask & (1u << q)) base = ((base >> q) << (q + 1)) | (base & ((1u << q) - 1u));
      }
      base |= cmask;
      int rows[4];
      C x[4], y[4];
      for (int a = 0; a < dt; ++a) {
        uint32_t r = base;
        for (int j = 0; j < kt; ++j)
          if ((a >> (kt - 1 - j)) & 1) r |= 1u << op.pos[nc + j];
        rows[a] = static_cast<int>(r);
        x[a] = U[r * D + c];
      }
      for (int a = 0; a < dt; ++a) {
        C acc = mkc<C>(0, 0);
        for (int b = 0; b < dt; ++b) acc = cadd2(acc, cmul2(M[a * dt + b], x[b]));
        y[a] = acc;
      }
      for (int a = 0; a < dt; ++a) U[rows[a] * D + c] = y[a];
    }
  }
}

// Descriptor limits the block kernels rely on (shared memory holds a 64 x 64 block; an op
// touches at most 6 wires, a dense part at most 2 targets): a block or op outside them is
// skipped, never indexed (the host checks them before upload).
__device__ __forceinline__ bool block_ok(const tqk_block_desc& bl) { return bl.k >= 1 && bl.k <= 6 && bl.num_ops >= 0; }

__device__ __forceinline__ bool op_ok(const tqk_block_op& op, int k) {
  if (op.nw < 1 || op.nw > 6 || op.nctrl < 0 || op.nctrl > op.nw) return false;
  for (int j = 0; j < op.nw; ++j)
    if (op.pos[j] < 0 || op.pos[j] >= k) return false;
  const int kt = op.nw - op.nctrl;
  switch (op.kind) {
    case TQK_K_DENSE:
    case TQK_K_CTRL: return kt >= 1 && kt <= 2 && op.op_size >= (1 << kt) * (1 << kt);
    case TQK_K_X: return kt == 1;
    case TQK_K_SWAP: return kt == 2;
    case TQK_K_PHASE: return op.op_size >= 1;
    case TQK_K_DIAG: return op.op_size >= (1 << op.nw);
    default: return false;
  }
}

__global__ void k_block_build(const tqk_block_desc* blocks, const tqk_block_op* ops) {
  extern __shared__ double2 smem_u[];
  C2* U = reinterpret_cast<C2*>(smem_u);
  const tqk_block_desc bl = blocks[blockIdx.x];
  const int64_t b = blockIdx.y;
  if (b >= bl.batch || !block_ok(bl)) return;
  const int D = 1 << bl.k;
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) U[e] = mk((e / D) == (e % D) ? 1.0 : 0.0, 0.0);
  __syncthreads();
  for (int i = 0; i < bl.num_ops; ++i) {
    const tqk_block_op op = ops[bl.first_op + i];
    if (!op_ok(op, bl.k)) continue;  // uniform for the CTA
    const double2* opnd = static_cast<const double2*>(op.operand) + (op.batch > 1 ? b : 0) * op.op_size;
    apply_op_rows(U, D, op, opnd, false);
    __syncthreads();
  }
  double2* dst = static_cast<double2*>(bl.u) + b * D * D;
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) dst[e] = make_double2(U[e].x, U[e].y);
}

// grad of op (operand cotangent) = sum over rows/cols of X[row][col] conj(W[row'][col]) restricted
// to the op's structure; W = product of the ops before it, X = (ops after)^H dL/dU.
// One sweep per entry: ops outside the specialised shapes below.
template <typename C>
__device__ void op_cotangent_generic(const C* X, const C* W, int D, const tqk_block_op& op, double2* gout, bool accumulate) {
  const int nw = op.nw, nc = op.nctrl;
  uint32_t cmask = 0, tmask = 0;
  for (int j = 0; j < nc; ++j) cmask |= 1u << op.pos[j];
  for (int j = nc; j < nw; ++j) tmask |= 1u << op.pos[j];
  const uint32_t allmask = cmask | tmask;
  int nent, kt = nw - nc;
  if (op.kind == TQK_K_PHASE) nent = 1;
  else if (op.kind == TQK_K_DIAG) nent = 1 << nw;
  else nent = (1 << kt) * (1 << kt);
  __shared__ double red[32][2];
  for (int ent = 0; ent < nent; ++ent) {
    double ax = 0.0, ay = 0.0;
    for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
      const int r = e / D, c = e % D;
      int rr = -1;  // partner row (W side) for this X row
      if (op.kind == TQK_K_PHASE) {
        if ((static_cast<uint32_t>(r) & allmask) == allmask) rr = r;
      } else if (op.kind == TQK_K_DIAG) {
        int di = 0;
        for (int j = 0; j < nw; ++j) di = (di << 1) | ((r >> op.pos[j]) & 1);
        if (di == ent) rr = r;
      } else {
        if ((static_cast<uint32_t>(r) & cmask) == cmask) {
          const int dt = 1 << kt;
          const int a_want = ent / dt, b_want = ent % dt;
          int a = 0;
          for (int j = 0; j < kt; ++j) a = (a << 1) | ((r >> op.pos[nc + j]) & 1);
          if (a == a_want) {
            uint32_t r2 = static_cast<uint32_t>(r) & ~tmask;
            for (int j = 0; j < kt; ++j)
              if ((b_want >> (kt - 1 - j)) & 1) r2 |= 1u << op.pos[nc + j];
            rr = static_cast<int>(r2);
          }
        }
      }
      if (rr >= 0) {
        const C xv = X[r * D + c], wv = W[rr * D + c];
        ax += xv.x * wv.x + xv.y * wv.y;  // x * conj(w)
        ay += xv.y * wv.x - xv.x * wv.y;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      ax += __shfl_xor_sync(0xffffffffu, ax, o);
      ay += __shfl_xor_sync(0xffffffffu, ay, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { red[warp][0] = ax; red[warp][1] = ay; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double sx = 0, sy = 0;
      for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w) { sx += red[w][0]; sy += red[w][1]; }
      if (accumulate) {
        atomicAdd(&gout[ent].x, sx);
        atomicAdd(&gout[ent].y, sy);
      } else {
        gout[ent] = make_double2(sx, sy);
      }
    }
    __syncthreads();
  }
}

// Row r with zeros inserted at the (ascending) bit positions pos[0..m).
__device__ __forceinline__ int insert_zeros(int r, const int* pos, int m) {
  for (int j = 0; j < m; ++j) r = ((r >> pos[j]) << (pos[j] + 1)) | (r & ((1 << pos[j]) - 1));
  return r;
}

// Sum of NE complex partial sums over the block; entries added (or stored) into gout.
template <int NE>
__device__ void block_reduce_entries(double (&acc)[2 * NE], double2* gout, int nent, bool accumulate) {
  __shared__ double red[8][2 * 16];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < 2 * NE; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 2 * nent) {
    double t = 0.0;
    for (int w = 0; w < nwarps; ++w) t += red[w][threadIdx.x];
    double* g = reinterpret_cast<double*>(gout) + threadIdx.x;
    if (accumulate) atomicAdd(g, t);
    else *g = t;
  }
  __syncthreads();
}

// Cotangent of the op's operand from X (cotangent rows) and W (state rows):
// entry (a, b) = sum over rows r with the op's control bits set and target pattern a, and
// columns c, of X[r][c] conj(W[r with target pattern b][c]) (diagonal ops: a = b over
// all op bits; phase ops: the single all-ones pattern).  One sweep over (row with the op's
// bits cleared, column) pairs evaluates every entry.
template <int KT, typename C>
__device__ void cot_dense(const C* X, const C* W, int D, const tqk_block_op& op, double2* gout, bool accumulate) {
  using R = typename C::real;
  constexpr int DT = 1 << KT, NE = DT * DT;
  const int nc = op.nctrl;
  uint32_t cmask = 0;
  for (int j = 0; j < nc; ++j) cmask |= 1u << op.pos[j];
  int tbit[KT], tsorted[KT];
#pragma unroll
  for (int j = 0; j < KT; ++j) tbit[j] = op.pos[nc + j];  // j = 0 is the pattern's most significant bit
#pragma unroll
  for (int j = 0; j < KT; ++j) tsorted[j] = tbit[j];
  if (KT == 2 && tsorted[0] > tsorted[1]) {
    const int t = tsorted[0];
    tsorted[0] = tsorted[1];
    tsorted[1] = t;
  }
  int pat[DT];
#pragma unroll
  for (int a = 0; a < DT; ++a) {
    int r = 0;
#pragma unroll
    for (int j = 0; j < KT; ++j)
      if ((a >> (KT - 1 - j)) & 1) r |= 1 << tbit[j];
    pat[a] = r;
  }
  R acc[2 * NE];
#pragma unroll
  for (int q = 0; q < 2 * NE; ++q) acc[q] = R(0);
  const int nbase = D >> KT;
  for (int w = threadIdx.x; w < nbase * D; w += blockDim.x) {
    const int c = w % D;
    const int r = insert_zeros(w / D, tsorted, KT);
    if ((static_cast<uint32_t>(r) & cmask) != cmask) continue;
    C xs[DT], ws[DT];
#pragma unroll
    for (int a = 0; a < DT; ++a) {
      xs[a] = X[(r | pat[a]) * D + c];
      ws[a] = W[(r | pat[a]) * D + c];
    }
#pragma unroll
    for (int a = 0; a < DT; ++a)
#pragma unroll
      for (int b2 = 0; b2 < DT; ++b2) {
        acc[2 * (a * DT + b2)] += xs[a].x * ws[b2].x + xs[a].y * ws[b2].y;  // x * conj(w)
        acc[2 * (a * DT + b2) + 1] += xs[a].y * ws[b2].x - xs[a].x * ws[b2].y;
      }
  }
  double accd[2 * NE];
#pragma unroll
  for (int q = 0; q < 2 * NE; ++q) accd[q] = static_cast<double>(acc[q]);
  block_reduce_entries<NE>(accd, gout, NE, accumulate);
}

// Diagonal ops (entries = pattern over all NW op bits) and phase ops (one entry: all bits set).
template <int NW, typename C>
__device__ void cot_diag(const C* X, const C* W, int D, const tqk_block_op& op, double2* gout, bool accumulate,
                         bool phase) {
  using R = typename C::real;
  constexpr int DT = 1 << NW;
  int bit[NW], srt[NW];
#pragma unroll
  for (int j = 0; j < NW; ++j) srt[j] = bit[j] = op.pos[j];
  if (NW == 2 && srt[0] > srt[1]) {
    const int t = srt[0];
    srt[0] = srt[1];
    srt[1] = t;
  }
  int pat[DT];
#pragma unroll
  for (int a = 0; a < DT; ++a) {
    int r = 0;
#pragma unroll
    for (int j = 0; j < NW; ++j)
      if ((a >> (NW - 1 - j)) & 1) r |= 1 << bit[j];
    pat[a] = r;
  }
  R acc[2 * DT];
#pragma unroll
  for (int q = 0; q < 2 * DT; ++q) acc[q] = R(0);
  const int nbase = D >> NW;
  for (int w = threadIdx.x; w < nbase * D; w += blockDim.x) {
    const int c = w % D;
    const int r = insert_zeros(w / D, srt, NW);
#pragma unroll
    for (int a = 0; a < DT; ++a) {
      if (phase && a != DT - 1) continue;
      const C xv = X[(r | pat[a]) * D + c], wv = W[(r | pat[a]) * D + c];
      acc[2 * a] += xv.x * wv.x + xv.y * wv.y;
      acc[2 * a + 1] += xv.y * wv.x - xv.x * wv.y;
    }
  }
  if (phase) {  // the single entry sits at index DT - 1
    acc[0] = acc[2 * (DT - 1)];
    acc[1] = acc[2 * (DT - 1) + 1];
  }
  double accd[2 * DT];
#pragma unroll
  for (int q = 0; q < 2 * DT; ++q) accd[q] = static_cast<double>(acc[q]);
  block_reduce_entries<DT>(accd, gout, phase ? 1 : DT, accumulate);
}

template <typename C>
__device__ void op_cotangent(const C* X, const C* W, int D, const tqk_block_op& op, double2* gout, bool accumulate) {
  const int kt = op.nw - op.nctrl;
  const bool diag = op.kind == TQK_K_PHASE || op.kind == TQK_K_DIAG;
  if ((diag && (op.nw < 1 || op.nw > 4)) || (!diag && (kt < 1 || kt > 2))) {
    op_cotangent_generic(X, W, D, op, gout, accumulate);
  } else if (diag) {
    const bool phase = op.kind == TQK_K_PHASE;
    if (op.nw == 1) cot_diag<1, C>(X, W, D, op, gout, accumulate, phase);
    else if (op.nw == 2) cot_diag<2, C>(X, W, D, op, gout, accumulate, phase);
    else if (op.nw == 3) cot_diag<3, C>(X, W, D, op, gout, accumulate, phase);
    else cot_diag<4, C>(X, W, D, op, gout, accumulate, phase);
  } else if (kt == 1) {
    cot_dense<1, C>(X, W, D, op, gout, accumulate);
  } else {
    cot_dense<2, C>(X, W, D, op, gout, accumulate);
  }
}

__global__ void k_block_unbuild(const tqk_block_desc* blocks, const tqk_block_op* ops) {
  extern __shared__ double2 smem_u[];
  const tqk_block_desc bl = blocks[blockIdx.x];
  const int64_t b = blockIdx.y;
  if (b >= bl.batch || bl.gu == nullptr || !block_ok(bl)) return;
  const int D = 1 << bl.k;
  F2* W = reinterpret_cast<F2*>(smem_u);
  F2* X = W + D * D;
  const double2* us = static_cast<const double2*>(bl.u) + b * D * D;
  const double2* gs = static_cast<const double2*>(bl.gu) + b * D * D;
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    W[e] = mkc<F2>(us[e].x, us[e].y);
    X[e] = mkc<F2>(gs[e].x, gs[e].y);
  }
  __syncthreads();
  for (int i = bl.num_ops - 1; i >= 0; --i) {
    const tqk_block_op op = ops[bl.first_op + i];
    if (!op_ok(op, bl.k)) continue;  // uniform for the CTA
    const double2* opnd = static_cast<const double2*>(op.operand) + (op.batch > 1 ? b : 0) * op.op_size;
    apply_op_rows(W, D, op, opnd, true);  // W <- G^H W = product of the ops before op
    __syncthreads();
    if (op.grad != nullptr) {
      double2* gout = static_cast<double2*>(op.grad) + (op.batch > 1 ? b : 0) * op.op_size;
      op_cotangent(X, W, D, op, gout, true);
    }
    apply_op_rows(X, D, op, opnd, true);  // X <- G^H X
    __syncthreads();
  }
}

}  // namespace prog
}  // namespace tqk

using namespace tqk;

extern "C" int tqk_gate_operand_size(int type) { return prog::operand_size(type); }

extern "C" int tqk_gate_operands(const tqk_gate_desc* gates, int ngates, void* stream) {
  if (ngates <= 0) return TQK_OK;
  if (!gates) return fail(TQK_BAD_POINTER, "tqk_gate_operands: null gate table");
  prog::k_gate_operands<<<ngates, 32, 0, as_stream(stream)>>>(gates, ngates);
  return launch_status("tqk_gate_operands");
}

extern "C" int tqk_param_grads(const tqk_gate_desc* gates, int ngates, void* stream) {
  if (ngates <= 0) return TQK_OK;
  if (!gates) return fail(TQK_BAD_POINTER, "tqk_param_grads: null gate table");
  prog::k_param_grads<<<ngates, 32, 0, as_stream(stream)>>>(gates, ngates);
  return launch_status("tqk_param_grads");
}

static void set_block_smem_attrs() {
  static int done = 0;
  if (done) return;
  const int one = static_cast<int>(64 * 64 * sizeof(double2));
  cudaFuncSetAttribute(prog::k_block_build, cudaFuncAttributeMaxDynamicSharedMemorySize, one);
  cudaFuncSetAttribute(prog::k_block_unbuild, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * one);
  done = 1;
}

extern "C" int tqk_block_build(const tqk_block_desc* blocks, int nblocks, int max_batch, const tqk_block_op* ops,
                               void* stream) {
  if (nblocks <= 0) return TQK_OK;
  if (!blocks || !ops) return fail(TQK_BAD_POINTER, "tqk_block_build: null pointer");
  if (max_batch < 1 || max_batch > 65535) return fail(TQK_BAD_SHAPE, "tqk_block_build: batch %d", max_batch);
  set_block_smem_attrs();
  dim3 grid(nblocks, max_batch, 1);
  prog::k_block_build<<<grid, 256, 64 * 64 * sizeof(double2), as_stream(stream)>>>(blocks, ops);
  return launch_status("tqk_block_build");
}

extern "C" int tqk_block_unbuild(const tqk_block_desc* blocks, int nblocks, int max_batch, const tqk_block_op* ops,
                                 void* stream) {
  if (nblocks <= 0) return TQK_OK;
  if (!blocks || !ops) return fail(TQK_BAD_POINTER, "tqk_block_unbuild: null pointer");
  if (max_batch < 1 || max_batch > 65535) return fail(TQK_BAD_SHAPE, "tqk_block_unbuild: batch %d", max_batch);
  set_block_smem_attrs();
  dim3 grid(nblocks, max_batch, 1);
  prog::k_block_unbuild<<<grid, 256, 2 * 64 * 64 * sizeof(float2), as_stream(stream)>>>(blocks, ops);
  return launch_status("tqk_block_unbuild");
}
