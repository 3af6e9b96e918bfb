// staged.cu -- runs of low-qubit gates applied in one pass through shared memory.
//
// The plain method launches one kernel per gate, each streaming the touched amplitudes
// once through HBM.  A run of consecutive gates whose targets all lie in the lowest
// tile_bits bits of the amplitude index (wires n - tile_bits .. n - 1) can share one
// pass instead: a CTA loads a contiguous tile of 2^tile_bits amplitudes of one batch row
// into shared memory with 128-bit loads, applies every op of the run there, and stores
// the tile back.  Controls and the wires of diagonal ops may be anywhere: they are read
// from the amplitude's global index (tile base | local index).
//
// The adjoint pass holds the psi and lam tiles of the same amplitudes and walks the run
// in reverse: psi <- U^H psi, lam <- U^H lam and, for ops with a cotangent slot,
// sum lam_in conj(psi_out) accumulated per op (warp shuffles, then float64 in shared
// memory across every tile the CTA handles; one atomic per value per CTA at the end).
#include <stdint.h>

#include "common.cuh"

namespace tqk {
namespace staged {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

struct SOp {
  int32_t kind;           // TQK_S_*
  int32_t lb;             // DENSE1 / X: target bit (inside the tile)
  uint64_t cmask;         // DENSE1 / X: control bits; PHASE: bits that must all be set
  uint64_t cval;          // DENSE1 / X: required values of the control bits
  int32_t nd;             // DIAG: number of bits (1 or 2)
  int32_t dbits[2];       // DIAG: bit positions, most significant diag-index bit first
  int32_t pad;
  const float2* operand;  // DENSE1 [batch][4], PHASE [batch], DIAG [batch][2^nd]
  int64_t op_stride;      // float2 per row (0 when shared by every row)
  double* grad;           // complex128 cotangent (interleaved), or null
  int64_t grad_stride;    // doubles per row (0 when shared)
};

struct Params {
  float2* psi;
  float2* lam;
  int n;
  int m;                  // tile bits
  int nops;
  int64_t tiles;          // tiles per row
  SOp ops[TQK_STAGED_MAX_OPS];
};

__device__ __forceinline__ int diag_index(const SOp& o, uint64_t g) {
  int d = 0;
  for (int j = 0; j < o.nd; ++j) d = (d << 1) | (int)((g >> o.dbits[j]) & 1ull);
  return d;
}

// Forward application of one op to the tile (amp, 2^m amplitudes at global index base).
__device__ __forceinline__ void apply_fwd(const SOp& o, float2* amp, int m, uint64_t base, int64_t b) {
  const int tsz = 1 << m;
  if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X) {
    const int lb = o.lb;
    float2 m00, m01, m10, m11;
    if (o.kind == TQK_S_DENSE1) {
      const float2* M = o.operand + b * o.op_stride;
      m00 = __ldg(M);
      m01 = __ldg(M + 1);
      m10 = __ldg(M + 2);
      m11 = __ldg(M + 3);
    }
    for (int p = threadIdx.x; p < (tsz >> 1); p += kThreads) {
      const int i0 = ((p >> lb) << (lb + 1)) | (p & ((1 << lb) - 1));
      const int i1 = i0 | (1 << lb);
      if (((base | (uint64_t)i0) & o.cmask) != o.cval) continue;
      const float2 a0 = amp[i0], a1 = amp[i1];
      if (o.kind == TQK_S_X) {
        amp[i0] = a1;
        amp[i1] = a0;
      } else {
        amp[i0] = cfma(m00, a0, cmul(m01, a1));
        amp[i1] = cfma(m10, a0, cmul(m11, a1));
      }
    }
  } else if (o.kind == TQK_S_PHASE) {
    const float2 ph = __ldg(o.operand + b * o.op_stride);
    for (int l = threadIdx.x; l < tsz; l += kThreads)
      if (((base | (uint64_t)l) & o.cmask) == o.cmask) amp[l] = cmul(ph, amp[l]);
  } else {  // DIAG
    const float2* dv = o.operand + b * o.op_stride;
    for (int l = threadIdx.x; l < tsz; l += kThreads) amp[l] = cmul(__ldg(dv + diag_index(o, base | (uint64_t)l)), amp[l]);
  }
}

__global__ void __launch_bounds__(kThreads) k_staged(const __grid_constant__ Params p) {
  extern __shared__ float4 sm4[];
  float2* amp = reinterpret_cast<float2*>(sm4);
  const int64_t b = blockIdx.y;
  const int half = 1 << (p.m - 1);  // float4 per tile
  float2* row = p.psi + (b << p.n);
  for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x) {
    const uint64_t base = (uint64_t)t << p.m;
    const float4* src = reinterpret_cast<const float4*>(row + base);
    for (int i = threadIdx.x; i < half; i += kThreads) sm4[i] = src[i];
    __syncthreads();
    for (int j = 0; j < p.nops; ++j) {
      apply_fwd(p.ops[j], amp, p.m, base, b);
      __syncthreads();
    }
    float4* dst = reinterpret_cast<float4*>(row + base);
    for (int i = threadIdx.x; i < half; i += kThreads) dst[i] = sm4[i];
    __syncthreads();
  }
}

// Warp-reduce NV float partials and add the block's sum into acc[0..NV) (float64,
// shared memory).  Called by every thread; ends with the block synchronised.
template <int NV>
__device__ __forceinline__ void block_accumulate(float (&v)[NV], float (*red)[8], double* acc) {
#pragma unroll
  for (int j = 0; j < NV; ++j)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) red[warp][j] = v[j];
  __syncthreads();
  if (threadIdx.x < NV) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) s += (double)red[w][threadIdx.x];
    acc[threadIdx.x] += s;
  }
}

// One reverse step of op o on the psi / lam tiles; cotangent partials into acc (8 doubles).
__device__ __forceinline__ void apply_adj(const SOp& o, float2* ps, float2* ls, int m, uint64_t base, int64_t b,
                                          float (*red)[8], double* acc) {
  const int tsz = 1 << m;
  const bool grad = o.grad != nullptr;
  if (o.kind == TQK_S_X) {
    const int lb = o.lb;
    for (int p = threadIdx.x; p < (tsz >> 1); p += kThreads) {
      const int i0 = ((p >> lb) << (lb + 1)) | (p & ((1 << lb) - 1));
      const int i1 = i0 | (1 << lb);
      if (((base | (uint64_t)i0) & o.cmask) != o.cval) continue;
      float2 t = ps[i0];
      ps[i0] = ps[i1];
      ps[i1] = t;
      t = ls[i0];
      ls[i0] = ls[i1];
      ls[i1] = t;
    }
    return;
  }
  float g[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) g[j] = 0.f;
  if (o.kind == TQK_S_DENSE1) {
    const int lb = o.lb;
    const float2* M = o.operand + b * o.op_stride;
    const float2 m00 = __ldg(M), m01 = __ldg(M + 1), m10 = __ldg(M + 2), m11 = __ldg(M + 3);
    for (int p = threadIdx.x; p < (tsz >> 1); p += kThreads) {
      const int i0 = ((p >> lb) << (lb + 1)) | (p & ((1 << lb) - 1));
      const int i1 = i0 | (1 << lb);
      if (((base | (uint64_t)i0) & o.cmask) != o.cval) continue;
      const float2 a0 = ps[i0], a1 = ps[i1], l0 = ls[i0], l1 = ls[i1];
      // U^H: [conj m00, conj m10; conj m01, conj m11]
      const float2 y0 = cfma_conj(m00, a0, cfma_conj(m10, a1, make_float2(0.f, 0.f)));
      const float2 y1 = cfma_conj(m01, a0, cfma_conj(m11, a1, make_float2(0.f, 0.f)));
      ps[i0] = y0;
      ps[i1] = y1;
      ls[i0] = cfma_conj(m00, l0, cfma_conj(m10, l1, make_float2(0.f, 0.f)));
      ls[i1] = cfma_conj(m01, l0, cfma_conj(m11, l1, make_float2(0.f, 0.f)));
      if (grad) {  // g[r][c] += l_r conj(y_c)
        float2 v;
        v = cfma_bconj(l0, y0, make_float2(g[0], g[1]));
        g[0] = v.x, g[1] = v.y;
        v = cfma_bconj(l0, y1, make_float2(g[2], g[3]));
        g[2] = v.x, g[3] = v.y;
        v = cfma_bconj(l1, y0, make_float2(g[4], g[5]));
        g[4] = v.x, g[5] = v.y;
        v = cfma_bconj(l1, y1, make_float2(g[6], g[7]));
        g[6] = v.x, g[7] = v.y;
      }
    }
  } else if (o.kind == TQK_S_PHASE) {
    const float2 phc = cconj(__ldg(o.operand + b * o.op_stride));
    for (int l = threadIdx.x; l < tsz; l += kThreads) {
      if (((base | (uint64_t)l) & o.cmask) != o.cmask) continue;
      const float2 y = cmul(phc, ps[l]), lv = ls[l];
      ps[l] = y;
      ls[l] = cmul(phc, lv);
      if (grad) {
        const float2 v = cfma_bconj(lv, y, make_float2(g[0], g[1]));
        g[0] = v.x, g[1] = v.y;
      }
    }
  } else {  // DIAG (nd <= 2)
    const float2* dv = o.operand + b * o.op_stride;
    for (int l = threadIdx.x; l < tsz; l += kThreads) {
      const int d = diag_index(o, base | (uint64_t)l);
      const float2 c = cconj(__ldg(dv + d));
      const float2 y = cmul(c, ps[l]), lv = ls[l];
      ps[l] = y;
      ls[l] = cmul(c, lv);
      if (grad) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (j == d) {
            const float2 v = cfma_bconj(lv, y, make_float2(g[2 * j], g[2 * j + 1]));
            g[2 * j] = v.x, g[2 * j + 1] = v.y;
          }
      }
    }
  }
  if (grad) block_accumulate<8>(g, red, acc);
}

__global__ void __launch_bounds__(kThreads) k_staged_adj(const __grid_constant__ Params p) {
  extern __shared__ float4 sm4[];
  const int tsz = 1 << p.m;
  float2* ps = reinterpret_cast<float2*>(sm4);
  float2* ls = ps + tsz;
  __shared__ double gacc[TQK_STAGED_MAX_OPS][8];
  __shared__ float red[kWarps][8];
  for (int i = threadIdx.x; i < TQK_STAGED_MAX_OPS * 8; i += kThreads) gacc[i / 8][i % 8] = 0.0;
  const int64_t b = blockIdx.y;
  const int half = tsz >> 1;
  float2* prow = p.psi + (b << p.n);
  float2* lrow = p.lam + (b << p.n);
  float4* ps4 = sm4;
  float4* ls4 = sm4 + half;
  __syncthreads();
  for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x) {
    const uint64_t base = (uint64_t)t << p.m;
    const float4* sp = reinterpret_cast<const float4*>(prow + base);
    const float4* sl = reinterpret_cast<const float4*>(lrow + base);
    for (int i = threadIdx.x; i < half; i += kThreads) {
      ps4[i] = sp[i];
      ls4[i] = sl[i];
    }
    __syncthreads();
    for (int j = p.nops - 1; j >= 0; --j) {
      apply_adj(p.ops[j], ps, ls, p.m, base, b, red, gacc[j]);
      __syncthreads();
    }
    float4* dp = reinterpret_cast<float4*>(prow + base);
    float4* dl = reinterpret_cast<float4*>(lrow + base);
    for (int i = threadIdx.x; i < half; i += kThreads) {
      dp[i] = ps4[i];
      dl[i] = ls4[i];
    }
    __syncthreads();
  }
  // flush: one atomic per value per op with a cotangent slot
  for (int i = threadIdx.x; i < p.nops * 8; i += kThreads) {
    const SOp& o = p.ops[i / 8];
    const int v = i % 8;
    if (o.grad == nullptr || o.kind == TQK_S_X) continue;
    const int nv = o.kind == TQK_S_DENSE1 ? 8 : (o.kind == TQK_S_PHASE ? 2 : 2 << o.nd);
    if (v < nv) atomicAdd(o.grad + b * o.grad_stride + v, gacc[i / 8][v]);
  }
}

}  // namespace staged
}  // namespace tqk

using namespace tqk;

namespace {

int fill_staged(staged::Params& p, int64_t bsz, int n, const tqk_staged_op* ops, int nops, int tile_bits,
                bool adjoint, const char* what) {
  if (bsz < 1 || n < 1 || n > TQK_MAX_QUBITS) return fail(TQK_BAD_SHAPE, "%s: bsz=%lld n=%d", what, (long long)bsz, n);
  if (bsz > 65535) return fail(TQK_BAD_SHAPE, "%s: bsz %lld > 65535", what, (long long)bsz);
  if (tile_bits < 1 || tile_bits > TQK_STAGED_MAX_TILE_BITS || tile_bits > n)
    return fail(TQK_BAD_SHAPE, "%s: tile_bits %d (1..min(n, %d))", what, tile_bits, TQK_STAGED_MAX_TILE_BITS);
  if (nops < 0 || nops > TQK_STAGED_MAX_OPS)
    return fail(TQK_BAD_SHAPE, "%s: %d ops (at most %d per pass)", what, nops, TQK_STAGED_MAX_OPS);
  if (nops > 0 && ops == nullptr) return fail(TQK_BAD_POINTER, "%s: null op list", what);
  p.n = n;
  p.m = tile_bits;
  p.nops = nops;
  p.tiles = 1ll << (n - tile_bits);
  for (int j = 0; j < nops; ++j) {
    const tqk_staged_op& s = ops[j];
    staged::SOp& o = p.ops[j];
    o = staged::SOp{};
    o.kind = s.kind;
    if (s.nwires < 1 || s.nwires > TQK_STAGED_MAX_WIRES)
      return fail(TQK_BAD_WIRES, "%s: op %d has %d wires", what, j, s.nwires);
    uint64_t used = 0;
    int bits[TQK_STAGED_MAX_WIRES];
    for (int w = 0; w < s.nwires; ++w) {
      if (s.wires[w] < 0 || s.wires[w] >= n) return fail(TQK_BAD_WIRES, "%s: op %d wire %d out of range", what, j, s.wires[w]);
      bits[w] = n - 1 - s.wires[w];
      if (used & (1ull << bits[w])) return fail(TQK_BAD_WIRES, "%s: op %d repeats wire %d", what, j, s.wires[w]);
      used |= 1ull << bits[w];
    }
    if (s.batch != 1 && s.batch != bsz && s.kind != TQK_S_X)
      return fail(TQK_BAD_SHAPE, "%s: op %d operand batch %lld (1 or bsz)", what, j, (long long)s.batch);
    if (s.kind != TQK_S_X && s.operand == nullptr) return fail(TQK_BAD_POINTER, "%s: op %d null operand", what, j);
    o.operand = static_cast<const float2*>(s.operand);
    o.grad = adjoint ? s.grad : nullptr;
    switch (s.kind) {
      case TQK_S_DENSE1:
      case TQK_S_X: {
        // wires[0 .. nwires-1) controls, wires[nwires-1] target
        const int tb = bits[s.nwires - 1];
        if (tb >= tile_bits)
          return fail(TQK_BAD_WIRES, "%s: op %d target wire %d is outside the tile (bit %d >= %d)", what, j,
                      s.wires[s.nwires - 1], tb, tile_bits);
        o.lb = tb;
        o.cmask = used & ~(1ull << tb);
        o.cval = (s.kind == TQK_S_X && !s.ctrl_val) ? 0ull : o.cmask;
        o.op_stride = (s.kind == TQK_S_DENSE1 && s.batch > 1) ? 4 : 0;
        o.grad_stride = (s.batch > 1) ? 8 : 0;
        break;
      }
      case TQK_S_PHASE:
        o.cmask = used;
        o.op_stride = s.batch > 1 ? 1 : 0;
        o.grad_stride = s.batch > 1 ? 2 : 0;
        break;
      case TQK_S_DIAG:
        if (s.nwires > 2) return fail(TQK_UNSUPPORTED, "%s: op %d diagonal on %d wires (1 or 2)", what, j, s.nwires);
        o.nd = s.nwires;
        for (int w = 0; w < s.nwires; ++w) o.dbits[w] = bits[w];
        o.op_stride = s.batch > 1 ? (1 << s.nwires) : 0;
        o.grad_stride = s.batch > 1 ? (2 << s.nwires) : 0;
        break;
      default:
        return fail(TQK_BAD_SHAPE, "%s: op %d kind %d", what, j, s.kind);
    }
  }
  return TQK_OK;
}

int launch_staged(void* psi, void* lam, int64_t bsz, int n, const tqk_staged_op* ops, int nops, int tile_bits,
                  bool adjoint, void* stream, const char* what) {
  int rc = check_state(psi, bsz, n, what);
  if (rc) return rc;
  if (adjoint && (rc = check_state(lam, bsz, n, what))) return rc;
  staged::Params p;
  if ((rc = fill_staged(p, bsz, n, ops, nops, tile_bits, adjoint, what))) return rc;
  if (nops == 0) return TQK_OK;
  p.psi = static_cast<float2*>(psi);
  p.lam = static_cast<float2*>(lam);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = (adjoint ? 2 : 1) * (sizeof(float2) << tile_bits);
  auto kern = adjoint ? staged::k_staged_adj : staged::k_staged;
  static int attr_set[64][2] = {{0}};
  if (dev >= 0 && dev < 64 && !attr_set[dev][adjoint]) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>((adjoint ? 2 : 1) * (sizeof(float2) << TQK_STAGED_MAX_TILE_BITS)));
    attr_set[dev][adjoint] = 1;
  }
  int fit = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, staged::kThreads, smem) != cudaSuccess || fit < 1)
    fit = 1;
  // enough CTAs to fill the GPU (each loops over tiles of its row); the adjoint flushes
  // its cotangents once per CTA, so it stops at one wave
  const int64_t want = static_cast<int64_t>(sms) * fit * (adjoint ? 1 : 4);
  int64_t gx = (want + bsz - 1) / bsz;
  if (gx > p.tiles) gx = p.tiles;
  if (gx < 1) gx = 1;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(bsz), 1);
  kern<<<grid, staged::kThreads, smem, as_stream(stream)>>>(p);
  return launch_status(what);
}

}  // namespace

extern "C" int tqk_staged_apply(void* state, int64_t bsz, int n, const tqk_staged_op* ops, int nops, int tile_bits,
                                void* stream) {
  return launch_staged(state, nullptr, bsz, n, ops, nops, tile_bits, false, stream, "tqk_staged_apply");
}

extern "C" int tqk_staged_adjoint(void* psi, void* lam, int64_t bsz, int n, const tqk_staged_op* ops, int nops,
                                  int tile_bits, void* stream) {
  return launch_staged(psi, lam, bsz, n, ops, nops, tile_bits, true, stream, "tqk_staged_adjoint");
}
