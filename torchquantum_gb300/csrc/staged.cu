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
// Inside a tile the run is applied in sweeps: up to 3 consecutive ops whose target bits
// number at most 3 (phase and diagonal ops join any sweep) act on cells of 8 amplitudes
// (the sweep's 3 cell bits in every combination) that one thread holds in registers, so
// the tile crosses shared memory once per sweep instead of once per op.
//
// Tiles are contiguous, so one thread moves each with the bulk-copy engine (TMA:
// cp.async.bulk into shared memory on an mbarrier, cp.async.bulk back to HBM); the wait
// for a load is bounded and reports TQK_TIMEOUT through the caller's status word.
//
// The adjoint pass holds the psi and lam tiles of the same amplitudes and walks the
// sweeps (and each sweep's ops) in reverse: psi <- U^H psi, lam <- U^H lam and, for ops
// with a cotangent slot, sum lam_in conj(psi_out) accumulated per op in registers over a
// thread's cells, then per sweep over the CTA (warp shuffles, float64 in shared memory
// across every tile the CTA handles; one atomic per value per CTA at the end).
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

// Consecutive ops applied in one shared-memory sweep: every op's target bit is one of the
// sweep's cell bits, so the ops act inside cells of 2^nd amplitudes (the cell bits set in
// every combination) that one thread holds in registers.
constexpr int kMaxSweepOps = 3;   // the adjoint keeps one cotangent accumulator set per op
constexpr int kCellDims = 3;      // cells of up to 8 amplitudes
struct Sweep {
  int32_t first, count;  // ops [first, first + count)
  int32_t nd;            // cell dimensions: min(3, tile bits)
  int32_t bits[kCellDims];  // cell bit positions, ascending
};

struct SOp {
  int32_t kind;           // TQK_S_*
  int32_t lb;             // DENSE1 / X: target bit (inside the tile)
  uint64_t cmask;         // DENSE1 / X: control bits; PHASE: bits that must all be set
  uint64_t cval;          // DENSE1 / X: required values of the control bits
  int32_t nd;             // DIAG: number of bits (1 or 2)
  int32_t dbits[2];       // DIAG: bit positions, most significant diag-index bit first
  int32_t dim;            // DENSE1 / X: position of lb among its sweep's cell bits
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
  int nsweeps;
  SOp ops[TQK_STAGED_MAX_OPS];
  Sweep sweeps[TQK_STAGED_MAX_OPS];
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

__device__ __forceinline__ void mat2(const float2 (&M)[4], float2& a0, float2& a1) {
  const float2 y0 = cfma(M[0], a0, cmul(M[1], a1));
  a1 = cfma(M[2], a0, cmul(M[3], a1));
  a0 = y0;
}

// Operands of the ops for batch row b, copied once per CTA into shared memory.
__device__ __forceinline__ void load_operands(const Params& p, int64_t b, float2 (*opnd)[4]) {
  for (int i = threadIdx.x; i < p.nops * 4; i += kThreads) {
    const SOp& o = p.ops[i >> 2];
    const int e = i & 3;
    const int cnt = o.kind == TQK_S_DENSE1 ? 4 : (o.kind == TQK_S_PHASE ? 1 : (o.kind == TQK_S_DIAG ? 1 << o.nd : 0));
    opnd[i >> 2][e] = e < cnt ? __ldg(o.operand + b * o.op_stride + e) : make_float2(0.f, 0.f);
  }
}

// In-tile indices of the 2^ND amplitudes of cell c: c with zeros inserted at the cell bits,
// then every combination of the cell bits (combination r sets cell bit d for bit d of r).
template <int ND>
__device__ __forceinline__ void cell_index(const Sweep& sw, uint32_t c, uint32_t (&idx)[1 << ND]) {
  uint32_t base = c;
#pragma unroll
  for (int d = 0; d < ND; ++d) {
    const int q = sw.bits[d];
    base = ((base >> q) << (q + 1)) | (base & ((1u << q) - 1u));
  }
#pragma unroll
  for (int r = 0; r < (1 << ND); ++r) {
    uint32_t v = base;
#pragma unroll
    for (int d = 0; d < ND; ++d)
      if ((r >> d) & 1) v |= 1u << sw.bits[d];
    idx[r] = v;
  }
}

// Cells with bit 0 among their bits hold amplitude pairs (r, r + 1) at adjacent even
// indices: 16-byte accesses; otherwise 8-byte accesses (consecutive lanes then address
// consecutive amplitudes).
template <int ND>
__device__ __forceinline__ void load_cell(const float2* t, const uint32_t (&idx)[1 << ND], bool vec,
                                          float2 (&a)[1 << ND]) {
  if (vec) {
#pragma unroll
    for (int r = 0; r < (1 << ND); r += 2) {
      const float4 v = *reinterpret_cast<const float4*>(t + idx[r]);
      a[r] = lo2(v);
      a[r + 1] = hi2(v);
    }
  } else {
#pragma unroll
    for (int r = 0; r < (1 << ND); ++r) a[r] = t[idx[r]];
  }
}

template <int ND>
__device__ __forceinline__ void store_cell(float2* t, const uint32_t (&idx)[1 << ND], bool vec,
                                           const float2 (&a)[1 << ND]) {
  if (vec) {
#pragma unroll
    for (int r = 0; r < (1 << ND); r += 2) *reinterpret_cast<float4*>(t + idx[r]) = pack4(a[r], a[r + 1]);
  } else {
#pragma unroll
    for (int r = 0; r < (1 << ND); ++r) t[idx[r]] = a[r];
  }
}

// Forward of a dense / X op on the cell's pairs along cell dimension K.
template <int ND, int K>
__device__ __forceinline__ void pairs_fwd(bool x, const float2 (&M)[4], const Local& L,
                                          const uint32_t (&idx)[1 << ND], float2 (&a)[1 << ND]) {
#pragma unroll
  for (int r = 0; r < (1 << ND); ++r) {
    if ((r >> K) & 1) continue;
    const int r1 = r | (1 << K);
    if ((idx[r] & L.lmask) != L.lval) continue;
    if (x) {
      const float2 t = a[r];
      a[r] = a[r1];
      a[r1] = t;
    } else {
      mat2(M, a[r], a[r1]);
    }
  }
}

template <int ND>
__device__ __forceinline__ void cell_fwd(const SOp& o, const Local& L, const float2* opd, const uint32_t (&idx)[1 << ND],
                                         float2 (&a)[1 << ND]) {
  if (!L.active) return;  // uniform for the tile
  if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X) {
    const bool x = o.kind == TQK_S_X;
    float2 M[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) M[e] = opd[e];
    if (o.dim == 0) pairs_fwd<ND, 0>(x, M, L, idx, a);
    else if (ND > 1 && o.dim == 1) pairs_fwd<ND, (ND > 1 ? 1 : 0)>(x, M, L, idx, a);
    else if (ND > 2) pairs_fwd<ND, (ND > 2 ? 2 : 0)>(x, M, L, idx, a);
  } else if (o.kind == TQK_S_PHASE) {
    const float2 ph = opd[0];
#pragma unroll
    for (int r = 0; r < (1 << ND); ++r)
      if ((idx[r] & L.lmask) == L.lval) a[r] = cmul(ph, a[r]);
  } else {  // DIAG
#pragma unroll
    for (int r = 0; r < (1 << ND); ++r) a[r] = cmul(opd[diag_local(o, L, idx[r])], a[r]);
  }
}

template <int ND>
__device__ __forceinline__ void sweep_fwd(const Params& p, const Sweep& sw, float2* amp, const Local* locs,
                                          const float2 (*opnd)[4]) {
  const uint32_t ncells = 1u << (p.m - ND);
  const bool vec = sw.bits[0] == 0;
  for (uint32_t c = threadIdx.x; c < ncells; c += kThreads) {
    uint32_t idx[1 << ND];
    cell_index<ND>(sw, c, idx);
    float2 a[1 << ND];
    load_cell<ND>(amp, idx, vec, a);
    for (int j = sw.first; j < sw.first + sw.count; ++j) cell_fwd<ND>(p.ops[j], locs[j], opnd[j], idx, a);
    store_cell<ND>(amp, idx, vec, a);
  }
}

__global__ void __launch_bounds__(kThreads) k_staged(const __grid_constant__ Params p) {
  extern __shared__ float4 sm4[];
  __shared__ uint64_t full;
  __shared__ int abort_flag;
  __shared__ Local locs[TQK_STAGED_MAX_OPS];
  __shared__ float2 opnd[TQK_STAGED_MAX_OPS][4];
  float2* amp = reinterpret_cast<float2*>(sm4);
  const int64_t b = blockIdx.y;
  const uint32_t bytes = static_cast<uint32_t>(sizeof(float2)) << p.m;
  float2* row = p.psi + (b << p.n);
  load_operands(p, b, opnd);
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
    if (threadIdx.x < p.nops) locs[threadIdx.x] = localise(p.ops[threadIdx.x], p.m, base);
    __syncthreads();
    if (abort_flag) break;  // uniform
    for (int s = 0; s < p.nsweeps; ++s) {
      const Sweep& sw = p.sweeps[s];
      if (sw.nd == 3) sweep_fwd<3>(p, sw, amp, locs, opnd);
      else if (sw.nd == 2) sweep_fwd<2>(p, sw, amp, locs, opnd);
      else sweep_fwd<1>(p, sw, amp, locs, opnd);
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

// Reverse of a dense / X op on the cell's pairs along cell dimension K (psi a, lam l).
template <int ND, int K>
__device__ __forceinline__ void pairs_adj(bool x, const float2 (&M)[4], const Local& L, const uint32_t (&idx)[1 << ND],
                                          float2 (&a)[1 << ND], float2 (&l)[1 << ND], bool grad, float (&g)[8]) {
#pragma unroll
  for (int r = 0; r < (1 << ND); ++r) {
    if ((r >> K) & 1) continue;
    const int r1 = r | (1 << K);
    if ((idx[r] & L.lmask) != L.lval) continue;
    if (x) {
      float2 t = a[r];
      a[r] = a[r1];
      a[r1] = t;
      t = l[r];
      l[r] = l[r1];
      l[r1] = t;
    } else {
      adj_pair(M, a[r], a[r1], l[r], l[r1], grad, g);
    }
  }
}

// One op's reverse step on a cell: psi <- U^H psi, lam <- U^H lam, cotangent partials in g.
template <int ND>
__device__ __forceinline__ void cell_adj(const SOp& o, const Local& L, const float2* opd, const uint32_t (&idx)[1 << ND],
                                         float2 (&a)[1 << ND], float2 (&l)[1 << ND], float (&g)[8]) {
  if (!L.active) return;  // uniform for the tile
  const bool grad = o.grad != nullptr;
  if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X) {
    const bool x = o.kind == TQK_S_X;
    float2 M[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) M[e] = opd[e];
    if (o.dim == 0) pairs_adj<ND, 0>(x, M, L, idx, a, l, grad, g);
    else if (ND > 1 && o.dim == 1) pairs_adj<ND, (ND > 1 ? 1 : 0)>(x, M, L, idx, a, l, grad, g);
    else if (ND > 2) pairs_adj<ND, (ND > 2 ? 2 : 0)>(x, M, L, idx, a, l, grad, g);
  } else if (o.kind == TQK_S_PHASE) {
    const float2 phc = cconj(opd[0]);
#pragma unroll
    for (int r = 0; r < (1 << ND); ++r) {
      if ((idx[r] & L.lmask) != L.lval) continue;
      a[r] = cmul(phc, a[r]);
      if (grad) acc_c(g, 0, l[r], a[r]);
      l[r] = cmul(phc, l[r]);
    }
  } else {  // DIAG (nd <= 2)
#pragma unroll
    for (int r = 0; r < (1 << ND); ++r) {
      const int d = diag_local(o, L, idx[r]);
      const float2 D = cconj(opd[d]);
      const float2 y = cmul(D, a[r]);
      if (grad) {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (j == d) acc_c(g, j, l[r], y);
      }
      a[r] = y;
      l[r] = cmul(D, l[r]);
    }
  }
}

// A sweep in reverse (its ops last to first on every cell), then each op's cotangent
// partials reduced over the CTA into its float64 accumulator.
template <int ND>
__device__ __forceinline__ void sweep_adj(const Params& p, const Sweep& sw, float2* ps, float2* ls, const Local* locs,
                                          const float2 (*opnd)[4], float (*red)[8], double (*gacc)[8]) {
  const uint32_t ncells = 1u << (p.m - ND);
  const bool vec = sw.bits[0] == 0;
  float g[kMaxSweepOps][8];
#pragma unroll
  for (int k = 0; k < kMaxSweepOps; ++k)
#pragma unroll
    for (int v = 0; v < 8; ++v) g[k][v] = 0.f;
  for (uint32_t c = threadIdx.x; c < ncells; c += kThreads) {
    uint32_t idx[1 << ND];
    cell_index<ND>(sw, c, idx);
    float2 a[1 << ND], l[1 << ND];
    load_cell<ND>(ps, idx, vec, a);
    load_cell<ND>(ls, idx, vec, l);
#pragma unroll
    for (int k = kMaxSweepOps - 1; k >= 0; --k)
      if (k < sw.count) cell_adj<ND>(p.ops[sw.first + k], locs[sw.first + k], opnd[sw.first + k], idx, a, l, g[k]);
    store_cell<ND>(ps, idx, vec, a);
    store_cell<ND>(ls, idx, vec, l);
  }
#pragma unroll
  for (int k = 0; k < kMaxSweepOps; ++k) {
    if (k >= sw.count) break;
    const SOp& o = p.ops[sw.first + k];
    if (o.grad != nullptr && o.kind != TQK_S_X && locs[sw.first + k].active)  // uniform
      block_accumulate<8>(g[k], red, gacc[sw.first + k]);
  }
}

__global__ void __launch_bounds__(kThreads, 2) k_staged_adj(const __grid_constant__ Params p) {
  extern __shared__ float4 sm4[];
  const int tsz = 1 << p.m;
  float2* ps = reinterpret_cast<float2*>(sm4);
  float2* ls = ps + tsz;
  __shared__ double gacc[TQK_STAGED_MAX_OPS][8];
  __shared__ float red[kWarps][8];
  __shared__ uint64_t full;
  __shared__ int abort_flag;
  __shared__ Local locs[TQK_STAGED_MAX_OPS];
  __shared__ float2 opnd[TQK_STAGED_MAX_OPS][4];
  for (int i = threadIdx.x; i < TQK_STAGED_MAX_OPS * 8; i += kThreads) gacc[i / 8][i % 8] = 0.0;
  const int64_t b = blockIdx.y;
  const uint32_t bytes = static_cast<uint32_t>(sizeof(float2)) << p.m;
  float2* prow = p.psi + (b << p.n);
  float2* lrow = p.lam + (b << p.n);
  load_operands(p, b, opnd);
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
    if (threadIdx.x < p.nops) locs[threadIdx.x] = localise(p.ops[threadIdx.x], p.m, base);
    __syncthreads();
    if (abort_flag) break;  // uniform
    for (int s = p.nsweeps - 1; s >= 0; --s) {
      const Sweep& sw = p.sweeps[s];
      if (sw.nd == 3) sweep_adj<3>(p, sw, ps, ls, locs, opnd, red, gacc);
      else if (sw.nd == 2) sweep_adj<2>(p, sw, ps, ls, locs, opnd, red, gacc);
      else sweep_adj<1>(p, sw, ps, ls, locs, opnd, red, gacc);
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

// Sweeps: consecutive ops (at most kMaxSweepOps) whose dense / X target bits number at most
// min(3, tile bits); phase and diagonal ops join any sweep.  Cell bits: the targets, then
// the lowest other tile bits, ascending; each dense / X op records its target's position.
void plan_sweeps(staged::Params& p) {
  const int nd = p.m < staged::kCellDims ? p.m : staged::kCellDims;
  p.nsweeps = 0;
  int j = 0;
  while (j < p.nops) {
    staged::Sweep& sw = p.sweeps[p.nsweeps++];
    sw.first = j;
    sw.count = 0;
    sw.nd = nd;
    uint32_t tmask = 0;
    while (j < p.nops && sw.count < staged::kMaxSweepOps) {
      const staged::SOp& o = p.ops[j];
      uint32_t t = tmask;
      if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X) t |= 1u << o.lb;
      if (__builtin_popcount(t) > nd) break;
      tmask = t;
      ++sw.count;
      ++j;
    }
    int nb = 0;
    for (int q = 0; q < p.m && nb < nd; ++q)  // targets first ...
      if ((tmask >> q) & 1u) sw.bits[nb++] = q;
    for (int q = 0; q < p.m && nb < nd; ++q)  // ... then the lowest other bits
      if (!((tmask >> q) & 1u)) sw.bits[nb++] = q;
    for (int a = 1; a < nd; ++a)  // ascending
      for (int c = a; c > 0 && sw.bits[c - 1] > sw.bits[c]; --c) {
        const int t = sw.bits[c];
        sw.bits[c] = sw.bits[c - 1];
        sw.bits[c - 1] = t;
      }
    for (int k = sw.first; k < sw.first + sw.count; ++k) {
      staged::SOp& o = p.ops[k];
      o.dim = 0;
      if (o.kind == TQK_S_DENSE1 || o.kind == TQK_S_X)
        for (int d = 0; d < nd; ++d)
          if (sw.bits[d] == o.lb) o.dim = d;
    }
  }
}

int launch_staged(void* psi, void* lam, int64_t bsz, int n, const tqk_staged_op* ops, int nops, int tile_bits,
                  int* status, bool adjoint, void* stream, const char* what) {
  int rc = check_state(psi, bsz, n, what);
  if (rc) return rc;
  if (adjoint && (rc = check_state(lam, bsz, n, what))) return rc;
  staged::Params p;
  if ((rc = fill_staged(p, bsz, n, ops, nops, tile_bits, adjoint, what))) return rc;
  if (nops == 0) return TQK_OK;
  plan_sweeps(p);
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
