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
// Tiles are contiguous, so one thread moves each with the bulk-copy engine (TMA:
// cp.async.bulk into shared memory on an mbarrier, cp.async.bulk back to HBM); the wait
// for a load is bounded and reports TQK_TIMEOUT through the caller's status word.
//
// The adjoint pass holds the psi and lam tiles of the same amplitudes and walks the run
// in reverse: psi <- U^H psi, lam <- U^H lam and, for ops with a cotangent slot,
// sum lam_in conj(psi_out) accumulated per op (warp shuffles, then float64 in shared
// memory across every tile the CTA handles; one atomic per value per CTA at the end).
#include <stdint.h>

#include "bulk.cuh"
#include "common.cuh"

namespace tqk {
namespace staged {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;

using namespace bulk;

// Thread 0: load `nreg` tile regions (bytes each) for use number `use` of the barrier; the
// previous tile's bulk stores must have finished reading the buffer first.  Returns false
// (and records TQK_TIMEOUT) if the load did not land in time.
__device__ __forceinline__ bool load_tile(uint64_t* bar, uint32_t use, int nreg, void* d0, const void* s0,
                                          void* d1, const void* s1, uint32_t bytes, int* status) {
  bulk_wait_read();
  mbar_expect(bar, bytes * nreg);
  bulk_load(d0, s0, bytes, bar);
  if (nreg > 1) bulk_load(d1, s1, bytes, bar);
  if (mbar_wait(bar, use & 1u)) return true;
  atomicExch(status, TQK_TIMEOUT);
  return false;
}

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
  int* status;            // TQK_TIMEOUT if a tile load did not complete
  SOp ops[TQK_STAGED_MAX_OPS];
};

// Per-tile view of an op: its control / phase condition split into the bits inside the
// tile (checked per amplitude, 32-bit) and the bits above it (uniform for the tile).
struct Local {
  bool active;      // the condition on the bits above the tile holds
  uint32_t lmask;   // condition bits inside the tile
  uint32_t lval;    // their required values
  int dsh[2];       // DIAG: local bit of diag-index bit j, or -1 (then dconst)
  int dconst;       // DIAG: diag-index bits that come from above the tile
};

__device__ __forceinline__ Local localise(const SOp& o, int m, uint64_t base) {
  Local L;
  const uint64_t lo = (1ull << m) - 1ull;
  if (o.kind == TQK_S_DIAG) {
    L.active = true;
    L.lmask = L.lval = 0;
    L.dconst = 0;
    for (int j = 0; j < 2; ++j) {
      L.dsh[j] = -1;
      if (j >= o.nd) continue;
      const int bit = o.dbits[j];
      const int place = o.nd - 1 - j;  // dbits[0] is the most significant diag-index bit
      if (bit < m) L.dsh[j] = bit;
      else if ((base >> bit) & 1ull) L.dconst |= 1 << place;
    }
    return L;
  }
  const uint64_t val = o.kind == TQK_S_PHASE ? o.cmask : o.cval;
  L.active = (base & (o.cmask & ~lo)) == (val & ~lo);
  L.lmask = static_cast<uint32_t>(o.cmask & lo);
  L.lval = static_cast<uint32_t>(val & lo);
  return L;
}

__device__ __forceinline__ int diag_local(const SOp& o, const Local& L, uint32_t l) {
  int d = L.dconst;
  if (L.dsh[0] >= 0) d |= static_cast<int>((l >> L.dsh[0]) & 1u) << (o.nd - 1);
  if (L.dsh[1] >= 0) d |= static_cast<int>((l >> L.dsh[1]) & 1u);
  return d;
}

// First index i0 (target bit lb clear) of pair-pair q: two adjacent pairs (i0, i0 + 2^lb)
// and (i0 + 1, i0 + 1 + 2^lb) when lb >= 1; one pair (2q, 2q + 1) when lb == 0.
__device__ __forceinline__ uint32_t pair_base(uint32_t q, int lb) {
  if (lb == 0) return q << 1;
  const uint32_t lowm = (1u << (lb - 1)) - 1u;
  return ((q >> (lb - 1)) << (lb + 1)) | ((q & lowm) << 1);
}

__device__ __forceinline__ void mat2(const float2 (&M)[4], float2& a0, float2& a1) {
  const float2 y0 = cfma(M[0], a0, cmul(M[1], a1));
  a1 = cfma(M[2], a0, cmul(M[3], a1));
  a0 = y0;
}

// Forward application of one op to the tile (amp, 2^m amplitudes at global index base).
__device__ __forceinline__ void apply_fwd(const SOp& o, float2* amp, int m, uint64_t base, int64_t b) {
  const Local L = localise(o, m, base);
  if (!L.active) return;  // uniform for the tile
  const int tsz = 1 << m;
  float4* amp4 = reinterpret_cast<float4*>(amp);
  if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X) {
    const int lb = o.lb;
    const bool x = o.kind == TQK_S_X;
    float2 M[4];
    if (!x) {
      const float2* src = o.operand + b * o.op_stride;
#pragma unroll
      for (int e = 0; e < 4; ++e) M[e] = __ldg(src + e);
    }
    const uint32_t nq = lb == 0 ? static_cast<uint32_t>(tsz >> 1) : static_cast<uint32_t>(tsz >> 2);
    for (uint32_t q = threadIdx.x; q < nq; q += kThreads) {
      const uint32_t i0 = pair_base(q, lb);
      if (lb == 0) {
        if ((i0 & L.lmask) != L.lval) continue;
        float4 v = amp4[i0 >> 1];
        float2 a0 = lo2(v), a1 = hi2(v);
        if (x) amp4[i0 >> 1] = pack4(a1, a0);
        else {
          mat2(M, a0, a1);
          amp4[i0 >> 1] = pack4(a0, a1);
        }
        continue;
      }
      const uint32_t i1 = i0 | (1u << lb);
      const bool ok0 = (i0 & L.lmask) == L.lval, ok1 = ((i0 | 1u) & L.lmask) == L.lval;
      if (!ok0 && !ok1) continue;
      float4 va = amp4[i0 >> 1], vb = amp4[i1 >> 1];
      float2 a0 = lo2(va), b0 = lo2(vb), a1 = hi2(va), b1 = hi2(vb);  // pairs (a0, b0), (a1, b1)
      if (x) {
        if (ok0) { const float2 t = a0; a0 = b0; b0 = t; }
        if (ok1) { const float2 t = a1; a1 = b1; b1 = t; }
      } else {
        if (ok0) mat2(M, a0, b0);
        if (ok1) mat2(M, a1, b1);
      }
      amp4[i0 >> 1] = pack4(a0, a1);
      amp4[i1 >> 1] = pack4(b0, b1);
    }
  } else if (o.kind == TQK_S_PHASE) {
    const float2 ph = __ldg(o.operand + b * o.op_stride);
    for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>(tsz >> 1); q += kThreads) {
      const uint32_t l = q << 1;
      const bool ok0 = (l & L.lmask) == L.lval, ok1 = ((l | 1u) & L.lmask) == L.lval;
      if (!ok0 && !ok1) continue;
      float4 v = amp4[q];
      float2 a0 = lo2(v), a1 = hi2(v);
      if (ok0) a0 = cmul(ph, a0);
      if (ok1) a1 = cmul(ph, a1);
      amp4[q] = pack4(a0, a1);
    }
  } else {  // DIAG
    const float2* dv = o.operand + b * o.op_stride;
    float2 D[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) D[e] = e < (1 << o.nd) ? __ldg(dv + e) : make_float2(0.f, 0.f);
    for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>(tsz >> 1); q += kThreads) {
      const uint32_t l = q << 1;
      float4 v = amp4[q];
      amp4[q] = pack4(cmul(D[diag_local(o, L, l)], lo2(v)), cmul(D[diag_local(o, L, l | 1u)], hi2(v)));
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_staged(const __grid_constant__ Params p) {
  extern __shared__ float4 sm4[];
  __shared__ uint64_t full;
  __shared__ int abort_flag;
  float2* amp = reinterpret_cast<float2*>(sm4);
  const int64_t b = blockIdx.y;
  const uint32_t bytes = static_cast<uint32_t>(sizeof(float2)) << p.m;
  float2* row = p.psi + (b << p.n);
  if (threadIdx.x == 0) {
    mbar_init(&full);
    abort_flag = 0;
  }
  __syncthreads();
  uint32_t use = 0;
  for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x, ++use) {
    const uint64_t base = (uint64_t)t << p.m;
    if (threadIdx.x == 0 && !load_tile(&full, use, 1, amp, row + base, nullptr, nullptr, bytes, p.status))
      abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;  // uniform
    for (int j = 0; j < p.nops; ++j) {
      apply_fwd(p.ops[j], amp, p.m, base, b);
      __syncthreads();
    }
    fence_async_smem();  // the ops' shared-memory writes, visible to the bulk store
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_store(row + base, amp, bytes);
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
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

__device__ __forceinline__ void acc_c(float (&g)[8], int slot, float2 l, float2 y) {  // g[slot] += l conj(y)
  const float2 v = cfma_bconj(l, y, make_float2(g[2 * slot], g[2 * slot + 1]));
  g[2 * slot] = v.x;
  g[2 * slot + 1] = v.y;
}

// Reverse step of a dense 2x2 on one pair: psi (a0, a1) <- U^H, lam (l0, l1) <- U^H, and
// the cotangent g[r][c] += lam_in_r conj(psi_out_c).
__device__ __forceinline__ void adj_pair(const float2 (&M)[4], float2& a0, float2& a1, float2& l0, float2& l1,
                                         bool grad, float (&g)[8]) {
  const float2 y0 = cfma_conj(M[0], a0, cfma_conj(M[2], a1, make_float2(0.f, 0.f)));
  const float2 y1 = cfma_conj(M[1], a0, cfma_conj(M[3], a1, make_float2(0.f, 0.f)));
  if (grad) {
    acc_c(g, 0, l0, y0);
    acc_c(g, 1, l0, y1);
    acc_c(g, 2, l1, y0);
    acc_c(g, 3, l1, y1);
  }
  const float2 z0 = cfma_conj(M[0], l0, cfma_conj(M[2], l1, make_float2(0.f, 0.f)));
  l1 = cfma_conj(M[1], l0, cfma_conj(M[3], l1, make_float2(0.f, 0.f)));
  l0 = z0;
  a0 = y0;
  a1 = y1;
}

// One reverse step of op o on the psi / lam tiles; cotangent partials into acc (8 doubles).
__device__ __forceinline__ void apply_adj(const SOp& o, float2* ps, float2* ls, int m, uint64_t base, int64_t b,
                                          float (*red)[8], double* acc) {
  const Local L = localise(o, m, base);
  if (!L.active) return;  // uniform for the tile
  const int tsz = 1 << m;
  const bool grad = o.grad != nullptr;
  float4* p4 = reinterpret_cast<float4*>(ps);
  float4* l4 = reinterpret_cast<float4*>(ls);
  float g[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) g[j] = 0.f;
  if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X) {
    const int lb = o.lb;
    const bool x = o.kind == TQK_S_X;
    float2 M[4];
    if (!x) {
      const float2* src = o.operand + b * o.op_stride;
#pragma unroll
      for (int e = 0; e < 4; ++e) M[e] = __ldg(src + e);
    }
    const uint32_t nq = lb == 0 ? static_cast<uint32_t>(tsz >> 1) : static_cast<uint32_t>(tsz >> 2);
    for (uint32_t q = threadIdx.x; q < nq; q += kThreads) {
      const uint32_t i0 = pair_base(q, lb);
      if (lb == 0) {
        if ((i0 & L.lmask) != L.lval) continue;
        float4 va = p4[i0 >> 1], vl = l4[i0 >> 1];
        float2 a0 = lo2(va), a1 = hi2(va), l0 = lo2(vl), l1 = hi2(vl);
        if (x) {
          p4[i0 >> 1] = pack4(a1, a0);
          l4[i0 >> 1] = pack4(l1, l0);
        } else {
          adj_pair(M, a0, a1, l0, l1, grad, g);
          p4[i0 >> 1] = pack4(a0, a1);
          l4[i0 >> 1] = pack4(l0, l1);
        }
        continue;
      }
      const uint32_t i1 = i0 | (1u << lb);
      const bool ok0 = (i0 & L.lmask) == L.lval, ok1 = ((i0 | 1u) & L.lmask) == L.lval;
      if (!ok0 && !ok1) continue;
      float4 pa = p4[i0 >> 1], pb = p4[i1 >> 1], la = l4[i0 >> 1], lb4 = l4[i1 >> 1];
      float2 a0 = lo2(pa), b0 = lo2(pb), a1 = hi2(pa), b1 = hi2(pb);
      float2 c0 = lo2(la), d0 = lo2(lb4), c1 = hi2(la), d1 = hi2(lb4);
      if (x) {
        if (ok0) { float2 t = a0; a0 = b0; b0 = t; t = c0; c0 = d0; d0 = t; }
        if (ok1) { float2 t = a1; a1 = b1; b1 = t; t = c1; c1 = d1; d1 = t; }
      } else {
        if (ok0) adj_pair(M, a0, b0, c0, d0, grad, g);
        if (ok1) adj_pair(M, a1, b1, c1, d1, grad, g);
      }
      p4[i0 >> 1] = pack4(a0, a1);
      p4[i1 >> 1] = pack4(b0, b1);
      l4[i0 >> 1] = pack4(c0, c1);
      l4[i1 >> 1] = pack4(d0, d1);
    }
    if (x) return;
  } else if (o.kind == TQK_S_PHASE) {
    const float2 phc = cconj(__ldg(o.operand + b * o.op_stride));
    for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>(tsz >> 1); q += kThreads) {
      const uint32_t l = q << 1;
      const bool ok0 = (l & L.lmask) == L.lval, ok1 = ((l | 1u) & L.lmask) == L.lval;
      if (!ok0 && !ok1) continue;
      float4 vp = p4[q], vl = l4[q];
      float2 a0 = lo2(vp), a1 = hi2(vp), c0 = lo2(vl), c1 = hi2(vl);
      if (ok0) {
        a0 = cmul(phc, a0);
        if (grad) acc_c(g, 0, c0, a0);
        c0 = cmul(phc, c0);
      }
      if (ok1) {
        a1 = cmul(phc, a1);
        if (grad) acc_c(g, 0, c1, a1);
        c1 = cmul(phc, c1);
      }
      p4[q] = pack4(a0, a1);
      l4[q] = pack4(c0, c1);
    }
  } else {  // DIAG (nd <= 2)
    const float2* dv = o.operand + b * o.op_stride;
    float2 D[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) D[e] = e < (1 << o.nd) ? cconj(__ldg(dv + e)) : make_float2(0.f, 0.f);
    for (uint32_t q = threadIdx.x; q < static_cast<uint32_t>(tsz >> 1); q += kThreads) {
      const uint32_t l = q << 1;
      const int d0 = diag_local(o, L, l), d1 = diag_local(o, L, l | 1u);
      float4 vp = p4[q], vl = l4[q];
      const float2 y0 = cmul(D[d0], lo2(vp)), y1 = cmul(D[d1], hi2(vp));
      if (grad) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (j == d0) acc_c(g, j, lo2(vl), y0);
          if (j == d1) acc_c(g, j, hi2(vl), y1);
        }
      }
      p4[q] = pack4(y0, y1);
      l4[q] = pack4(cmul(D[d0], lo2(vl)), cmul(D[d1], hi2(vl)));
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
  __shared__ uint64_t full;
  __shared__ int abort_flag;
  for (int i = threadIdx.x; i < TQK_STAGED_MAX_OPS * 8; i += kThreads) gacc[i / 8][i % 8] = 0.0;
  const int64_t b = blockIdx.y;
  const uint32_t bytes = static_cast<uint32_t>(sizeof(float2)) << p.m;
  float2* prow = p.psi + (b << p.n);
  float2* lrow = p.lam + (b << p.n);
  if (threadIdx.x == 0) {
    mbar_init(&full);
    abort_flag = 0;
  }
  __syncthreads();
  uint32_t use = 0;
  for (int64_t t = blockIdx.x; t < p.tiles; t += gridDim.x, ++use) {
    const uint64_t base = (uint64_t)t << p.m;
    if (threadIdx.x == 0 && !load_tile(&full, use, 2, ps, prow + base, ls, lrow + base, bytes, p.status))
      abort_flag = 1;
    __syncthreads();
    if (abort_flag) break;  // uniform
    for (int j = p.nops - 1; j >= 0; --j) {
      apply_adj(p.ops[j], ps, ls, p.m, base, b, red, gacc[j]);
      __syncthreads();
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_store(prow + base, ps, bytes);
      bulk_store(lrow + base, ls, bytes);
      bulk_commit();
    }
  }
  if (threadIdx.x == 0) bulk_wait_all();
  __syncthreads();
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
                  int* status, bool adjoint, void* stream, const char* what) {
  int rc = check_state(psi, bsz, n, what);
  if (rc) return rc;
  if (adjoint && (rc = check_state(lam, bsz, n, what))) return rc;
  staged::Params p;
  if ((rc = fill_staged(p, bsz, n, ops, nops, tile_bits, adjoint, what))) return rc;
  if (nops == 0) return TQK_OK;
  if (status == nullptr) return fail(TQK_BAD_POINTER, "%s: null status word", what);
  p.psi = static_cast<float2*>(psi);
  p.lam = static_cast<float2*>(lam);
  p.status = status;
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
  // (the adjoint grid is rounded down so every CTA is resident at once: a CTA past the
  // first wave would run its whole tile loop after the others)
  const int64_t want = static_cast<int64_t>(sms) * fit * (adjoint ? 1 : 4);
  int64_t gx = adjoint ? want / bsz : (want + bsz - 1) / bsz;
  if (gx > p.tiles) gx = p.tiles;
  if (gx < 1) gx = 1;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(bsz), 1);
  kern<<<grid, staged::kThreads, smem, as_stream(stream)>>>(p);
  return launch_status(what);
}

}  // namespace

extern "C" int tqk_staged_apply(void* state, int64_t bsz, int n, const tqk_staged_op* ops, int nops, int tile_bits,
                                int* status, void* stream) {
  return launch_staged(state, nullptr, bsz, n, ops, nops, tile_bits, status, false, stream, "tqk_staged_apply");
}

extern "C" int tqk_staged_adjoint(void* psi, void* lam, int64_t bsz, int n, const tqk_staged_op* ops, int nops,
                                  int tile_bits, int* status, void* stream) {
  return launch_staged(psi, lam, bsz, n, ops, nops, tile_bits, status, true, stream, "tqk_staged_adjoint");
}
