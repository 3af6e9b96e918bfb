// batch.cu -- persistent runner for many independent circuits of different sizes.
//
// A circuit is a list of passes (tqk_batch_plan); a pass holds ops whose target bits lie
// in a tile of 2^tile_bits amplitudes (tile_mask, tile_bits 10..14 per launch), applied
// tile by tile in shared memory: gather the tile from the circuit's state, apply every op
// of the pass, scatter it back.  Circuits with n <= tile_bits are one tile and one pass:
// their whole life is in shared memory.  Diagonal ops (CZ, CZ ladders) and controls need
// no tile bit -- their signs split into per-tile constants and tile-local terms -- so the
// planner gives them to any pass.
//
// Work is one item per (circuit, pass, tile) (tqk_batch_items), handed out in waves of
// pass index by a global counter to persistent CTAs (1..8 per SM), so the tiles of a large
// circuit's pass run on many SMs at once.  An item of pass p > 0 waits (bounded) for the
// completion counter of pass p - 1; every item's dependencies are handed out before it,
// so the earliest unfinished item can always run.  A tile publishes its stores
// (__threadfence) before counting itself done; dependent tiles read through L2
// (ld.global.cg) since their SM's L1 may hold the previous pass's lines.  Last-pass tiles
// add their <Z> partial (float64 atomics) and the tile that completes a circuit stamps
// its completion time.
#include <stdint.h>

#include <vector>

#include "bulk.cuh"
#include "common.cuh"

namespace tqk {
namespace batch {

constexpr int kMaxTileBits = TQK_BATCH_TILE_BITS;
constexpr int kMinTileBits = 10;
constexpr int kLowReserve = 5;  // address bits 0-4 stay in every tile: warps read 256-byte runs
constexpr int kFirst = 1, kLast = 2;

struct Tabs {
  uint32_t lo[128];  // amplitude offset of tile index bits 0-6
  uint32_t hi[128];  // ... and bits 7-13
};

__device__ __forceinline__ uint32_t dep(const Tabs& t, uint32_t l) { return t.lo[l & 127] + t.hi[l >> 7]; }

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {  // a * b + c
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}

// 2x2 matrix m on local bit lb of the tile; if lc >= 0 only where local bit lc is set.
// Two adjacent pairs (i0, i0 + 2^lb), (i0 + 1, i0 + 1 + 2^lb) per 16-byte access when
// lb >= 1, one pair (2q, 2q + 1) per access when lb == 0.
template <int THREADS>
__device__ __forceinline__ void apply_1q(float2* amp, int tb, int lb, int lc, const float2* m) {
  float2 M[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) M[e] = __ldg(m + e);
  const uint32_t cm = lc >= 0 ? (1u << lc) : 0u;
  float4* amp4 = reinterpret_cast<float4*>(amp);
  if (lb == 0) {
    for (uint32_t q = threadIdx.x; q < (1u << (tb - 1)); q += THREADS) {
      const uint32_t i0 = q << 1;
      if ((i0 & cm) != cm) continue;
      const float4 v = amp4[q];
      const float2 a0 = lo2(v), a1 = hi2(v);
      amp4[q] = pack4(cfma(M[0], a0, cmul(M[1], a1)), cfma(M[2], a0, cmul(M[3], a1)));
    }
    return;
  }
  const uint32_t lowm = (1u << (lb - 1)) - 1u;
  for (uint32_t q = threadIdx.x; q < (1u << (tb - 2)); q += THREADS) {
    const uint32_t i0 = ((q >> (lb - 1)) << (lb + 1)) | ((q & lowm) << 1);
    const uint32_t i1 = i0 | (1u << lb);
    const bool ok0 = (i0 & cm) == cm, ok1 = ((i0 | 1u) & cm) == cm;
    if (!ok0 && !ok1) continue;
    const float4 va = amp4[i0 >> 1], vb = amp4[i1 >> 1];
    float2 a0 = lo2(va), b0 = lo2(vb), a1 = hi2(va), b1 = hi2(vb);
    if (ok0) {
      const float2 y = cfma(M[0], a0, cmul(M[1], b0));
      b0 = cfma(M[2], a0, cmul(M[3], b0));
      a0 = y;
    }
    if (ok1) {
      const float2 y = cfma(M[0], a1, cmul(M[1], b1));
      b1 = cfma(M[2], a1, cmul(M[3], b1));
      a1 = y;
    }
    amp4[i0 >> 1] = pack4(a0, a1);
    amp4[i1 >> 1] = pack4(b0, b1);
  }
}

// Negate the amplitudes whose local index l has odd parity of c0 + popc(l & lin) +
// popc(l & (l >> 1) & quad) (CZ and CZ ladders split into tile-local terms).
template <int THREADS>
__device__ __forceinline__ void apply_sign(float2* amp, int tb, int c0, uint32_t lin, uint32_t quad) {
  float4* amp4 = reinterpret_cast<float4*>(amp);
  for (uint32_t q = threadIdx.x; q < (1u << (tb - 1)); q += THREADS) {
    const uint32_t l0 = q << 1, l1 = l0 | 1u;
    const int s0 = (c0 + __popc(l0 & lin) + __popc(l0 & (l0 >> 1) & quad)) & 1;
    const int s1 = (c0 + __popc(l1 & lin) + __popc(l1 & (l1 >> 1) & quad)) & 1;
    if (!(s0 | s1)) continue;
    float4 v = amp4[q];
    if (s0) v.x = -v.x, v.y = -v.y;
    if (s1) v.z = -v.z, v.w = -v.w;
    amp4[q] = v;
  }
}

__device__ __forceinline__ int local_pos(uint32_t tmask, int b) { return __popc(tmask & ((1u << b) - 1u)); }

// Sign terms of CZ on global bits (bh, bl): both local -> a quadratic term only when the
// bits are adjacent in the tile (true for ladder neighbours), else handled as lin/const.
__device__ __forceinline__ void cz_terms(uint32_t tmask, uint32_t base, int b0, int b1, int& c0, uint32_t& lin,
                                         uint32_t& quad, uint32_t& pairs) {
  const bool in0 = (tmask >> b0) & 1u, in1 = (tmask >> b1) & 1u;
  if (in0 && in1) {
    const int p0 = local_pos(tmask, b0), p1 = local_pos(tmask, b1);
    const int lo = p0 < p1 ? p0 : p1, hi = p0 < p1 ? p1 : p0;
    if (hi == lo + 1) quad |= 1u << lo;
    else pairs |= (1u << lo) | (1u << hi);  // a general local pair (single CZ only)
  } else if (in0) {
    if ((base >> b1) & 1u) lin ^= 1u << local_pos(tmask, b0);
  } else if (in1) {
    if ((base >> b0) & 1u) lin ^= 1u << local_pos(tmask, b1);
  } else {
    c0 ^= static_cast<int>((base >> b0) & (base >> b1) & 1u);
  }
}

template <int THREADS>
__device__ void apply_op(const tqk_batch_op& op, float2* amp, int n, int tb, uint32_t tmask, uint32_t base,
                         const Tabs& tabs, const float2* mats) {
  switch (op.kind) {
    case TQK_B_DENSE1: {
      const int b = n - 1 - op.w0;
      apply_1q<THREADS>(amp, tb, local_pos(tmask, b), -1, mats + 4 * op.mat);
      break;
    }
    case TQK_B_CTRL1: {
      const int cb = n - 1 - op.w0, b = n - 1 - op.w1;
      const int lb = local_pos(tmask, b);
      if ((tmask >> cb) & 1u) {
        apply_1q<THREADS>(amp, tb, lb, local_pos(tmask, cb), mats + 4 * op.mat);
      } else if ((base >> cb) & 1u) {  // control outside the tile: set for the whole tile
        apply_1q<THREADS>(amp, tb, lb, -1, mats + 4 * op.mat);
      }
      break;
    }
    case TQK_B_CZ: {
      int c0 = 0;
      uint32_t lin = 0, quad = 0, pairs = 0;
      cz_terms(tmask, base, n - 1 - op.w0, n - 1 - op.w1, c0, lin, quad, pairs);
      if (pairs) {  // both bits in the tile but not adjacent: negate where both are set
        float4* amp4 = reinterpret_cast<float4*>(amp);
        for (uint32_t q = threadIdx.x; q < (1u << (tb - 1)); q += THREADS) {
          const uint32_t l0 = q << 1;
          const bool s0 = (l0 & pairs) == pairs, s1 = ((l0 | 1u) & pairs) == pairs;
          if (!(s0 || s1)) continue;
          float4 v = amp4[q];
          if (s0) v.x = -v.x, v.y = -v.y;
          if (s1) v.z = -v.z, v.w = -v.w;
          amp4[q] = v;
        }
      } else if (c0 | lin | quad) {
        apply_sign<THREADS>(amp, tb, c0, lin, quad);
      }
      break;
    }
    case TQK_B_CZ_LADDER: {
      int c0 = 0;
      uint32_t lin = 0, quad = 0, pairs = 0;
      for (int w = op.w0; w < op.w1; ++w) cz_terms(tmask, base, n - 1 - w, n - 2 - w, c0, lin, quad, pairs);
      if (c0 | lin | quad) apply_sign<THREADS>(amp, tb, c0, lin, quad);
      break;
    }
    default:
      break;
  }
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz

// THREADS threads per CTA, MINB CTAs per SM for the register budget; the tile holds up
// to 2^max_tb amplitudes (dynamic shared memory).
template <int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB)
    k_batch(const tqk_batch_circuit* circ, int ncirc, const tqk_batch_op* ops, const tqk_batch_pass* passes,
            const tqk_batch_item* items, long long n_items, const float2* mats, float2* states, int write_states,
            double* z_out, int* pass_done, unsigned long long* t_done, int* counter, int* status, int max_tb) {
  extern __shared__ float4 amp_raw[];  // 16-byte aligned: ops use float4 accesses
  float2* amp = reinterpret_cast<float2*>(amp_raw);
  __shared__ Tabs tabs;
  __shared__ long long s_i;
  __shared__ double red[THREADS / 32];
  __shared__ uint64_t full;  // bulk-copy (TMA) tile loads complete here
  __shared__ int abort_flag;
  if (t_done != nullptr && blockIdx.x == 0 && threadIdx.x == 0) t_done[ncirc] = global_ns();
  if (threadIdx.x == 0) {
    bulk::mbar_init(&full);
    abort_flag = 0;
  }
  uint32_t use = 0;  // loads completed on `full` so far
  for (;;) {
    if (threadIdx.x == 0) s_i = atomicAdd(counter, 1);
    __syncthreads();
    const long long i = s_i;
    __syncthreads();
    if (i >= n_items) break;
    const tqk_batch_item it = items[i];
    const tqk_batch_circuit C = circ[it.circuit];
    const tqk_batch_pass P = passes[it.pass];
    const int n = C.n;
    const uint32_t tmask = P.tile_mask;
    const int tb = __popc(tmask);
    if (tb > max_tb || tb < 1) {  // a plan made for a larger tile: record and skip the item
      if (threadIdx.x == 0) {
        atomicExch(status, TQK_BAD_SHAPE);
        atomicAdd(pass_done + it.pass, 1);
      }
      __syncthreads();
      continue;
    }
    const int tsz = 1 << tb;
    const int ntiles = 1 << (n - tb);
    const uint32_t omask = (n >= 32 ? 0xffffffffu : ((1u << n) - 1u)) & ~tmask;
    float2* st = states + (C.state_off >= 0 ? C.state_off : 0);
    if (!(P.flags & kFirst) && threadIdx.x == 0) {  // every tile of the previous pass must be stored
      const int prev_tiles = 1 << (n - __popc(passes[it.pass - 1].tile_mask));
      const volatile int* d = pass_done + it.pass - 1;
      const long long t0 = clock64();
      while (*d < prev_tiles) {
        if (clock64() - t0 > kWaitCycles) {
          atomicExch(status, TQK_TIMEOUT);
          break;
        }
      }
      __threadfence();
    }
    for (int t = threadIdx.x; t < 256; t += THREADS) {  // deposit tables of the tile bits
      const int part = t >> 7, x = t & 127;
      uint32_t v = 0;
      int j = 0;
      for (int b = 0; b < n; ++b) {
        if (!((tmask >> b) & 1u)) continue;
        const int k = j++ - 7 * part;
        if (k >= 0 && k < 7 && ((x >> k) & 1)) v |= 1u << b;
      }
      (part ? tabs.hi : tabs.lo)[x] = v;
    }
    uint32_t base = 0;
    for (int b = 0, j = 0; b < n; ++b) {
      if (!((omask >> b) & 1u)) continue;
      if ((it.tile >> j) & 1) base |= 1u << b;
      ++j;
    }
    __syncthreads();
    // Runs of 32 amplitudes (tile bits 0-4 are address bits 0-4) or the whole tile when it
    // is smaller: contiguous in HBM, moved by the bulk-copy engine.
    const int run = tsz < 32 ? tsz : 32;
    const int nruns = tsz / run;
    if (P.flags & kFirst) {
      for (int l = threadIdx.x; l < tsz; l += THREADS)
        amp[l] = make_float2((base == 0u && l == 0) ? 1.f : 0.f, 0.f);
    } else {
      if (threadIdx.x == 0) bulk::mbar_expect(&full, static_cast<uint32_t>(tsz * sizeof(float2)));
      __syncthreads();
      asm volatile("fence.proxy.async.global;" ::: "memory");  // the dependency flag was read by the generic proxy
      for (int r = threadIdx.x; r < nruns; r += THREADS)
        bulk::bulk_load(amp + r * run, st + base + dep(tabs, static_cast<uint32_t>(r * run)),
                        static_cast<uint32_t>(run * sizeof(float2)), &full);
      if (threadIdx.x == 0 && !bulk::mbar_wait(&full, use & 1u)) {
        atomicExch(status, TQK_TIMEOUT);
        abort_flag = 1;
      }
      ++use;
    }
    __syncthreads();
    if (abort_flag) break;  // uniform: a tile load never landed
    for (int oi = 0; oi < P.num_ops; ++oi) {
      apply_op<THREADS>(ops[P.first_op + oi], amp, n, tb, tmask, base, tabs, mats);
      __syncthreads();
    }
    if (P.flags & kLast) {
      const int zbit = n - 1 - C.z_wire;
      double zacc = 0.0;
      for (int l = threadIdx.x; l < tsz; l += THREADS) {
        const float2 a = amp[l];
        const double p2 = static_cast<double>(a.x) * a.x + static_cast<double>(a.y) * a.y;
        zacc += (((base + dep(tabs, l)) >> zbit) & 1u) ? -p2 : p2;
      }
      for (int o = 16; o > 0; o >>= 1) zacc += __shfl_xor_sync(0xffffffffu, zacc, o);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = zacc;
    }
    if (((P.flags & kLast) == 0 || write_states) && C.state_off >= 0) {
      bulk::fence_async_smem();  // the ops' shared-memory writes, visible to the bulk stores
      __syncthreads();
      bool mine = false;
      for (int r = threadIdx.x; r < nruns; r += THREADS) {
        bulk::bulk_store(st + base + dep(tabs, static_cast<uint32_t>(r * run)), amp + r * run,
                         static_cast<uint32_t>(run * sizeof(float2)));
        mine = true;
      }
      if (mine) {
        bulk::bulk_commit();
        bulk::bulk_wait_all();  // stored in HBM / L2 before the tile counts as done
        asm volatile("fence.proxy.async.global;" ::: "memory");
      }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      if (P.flags & kLast) {
        double sum = 0.0;
        for (int w = 0; w < THREADS / 32; ++w) sum += red[w];
        atomicAdd(z_out + it.circuit, sum);
        __threadfence();
      }
      const int old = atomicAdd(pass_done + it.pass, 1);
      if ((P.flags & kLast) && old == ntiles - 1 && t_done != nullptr) t_done[it.circuit] = global_ns();
    }
    __syncthreads();
  }
}

// Bits of an op's wires (all of them) and of its targets (the bits that must be in the tile).
void op_bits(const tqk_batch_op& op, int n, uint32_t* wires, uint32_t* targets) {
  auto bit = [n](int w) { return 1u << (n - 1 - w); };
  switch (op.kind) {
    case TQK_B_DENSE1:
      *wires = *targets = bit(op.w0);
      break;
    case TQK_B_CTRL1:
      *wires = bit(op.w0) | bit(op.w1);
      *targets = bit(op.w1);
      break;
    case TQK_B_CZ:
      *wires = bit(op.w0) | bit(op.w1);
      *targets = 0;
      break;
    default: {  // ladder
      uint32_t m = 0;
      for (int w = op.w0; w <= op.w1; ++w) m |= bit(w);
      *wires = m;
      *targets = 0;
    }
  }
}

}  // namespace batch
}  // namespace tqk

using namespace tqk;

extern "C" int tqk_batch_plan(tqk_batch_circuit* circuits, int ncirc, const tqk_batch_op* ops_in, int n_mats,
                              tqk_batch_op* ops_out, tqk_batch_pass* passes, int max_passes, int tile_bits) {
  const char* what = "tqk_batch_plan";
  if (ncirc < 0) return -fail(TQK_BAD_SHAPE, "%s: ncirc %d", what, ncirc);
  if (ncirc > 0 && (!circuits || !passes || !ops_out)) return -fail(TQK_BAD_POINTER, "%s: null pointer", what);
  if (tile_bits < batch::kMinTileBits || tile_bits > batch::kMaxTileBits)
    return -fail(TQK_BAD_SHAPE, "%s: tile_bits %d outside %d..%d", what, tile_bits, batch::kMinTileBits,
                 batch::kMaxTileBits);
  const int T = tile_bits;
  int np = 0;
  for (int ci = 0; ci < ncirc; ++ci) {
    tqk_batch_circuit& c = circuits[ci];
    const int n = c.n;
    if (n < 1 || n > TQK_BATCH_MAX_QUBITS) return -fail(TQK_TOO_MANY_QUBITS, "%s: circuit %d has n=%d", what, ci, n);
    if (c.z_wire < 0 || c.z_wire >= n) return -fail(TQK_BAD_WIRES, "%s: circuit %d z_wire %d", what, ci, c.z_wire);
    if (c.num_ops < 0 || c.first_op < 0 || (c.num_ops > 0 && !ops_in))
      return -fail(TQK_BAD_SHAPE, "%s: circuit %d op range", what, ci);
    for (int k = 0; k < c.num_ops; ++k) {
      const tqk_batch_op& op = ops_in[c.first_op + k];
      const bool two = op.kind == TQK_B_CTRL1 || op.kind == TQK_B_CZ || op.kind == TQK_B_CZ_LADDER;
      if (op.kind < TQK_B_DENSE1 || op.kind > TQK_B_CZ_LADDER)
        return -fail(TQK_BAD_SHAPE, "%s: circuit %d op %d kind %d", what, ci, k, op.kind);
      if (op.w0 < 0 || op.w0 >= n || (two && (op.w1 < 0 || op.w1 >= n)))
        return -fail(TQK_BAD_WIRES, "%s: circuit %d op %d wires out of range", what, ci, k);
      if ((op.kind == TQK_B_CTRL1 || op.kind == TQK_B_CZ) && op.w0 == op.w1)
        return -fail(TQK_BAD_WIRES, "%s: circuit %d op %d uses a wire twice", what, ci, k);
      if (op.kind == TQK_B_CZ_LADDER && op.w1 <= op.w0)
        return -fail(TQK_BAD_WIRES, "%s: circuit %d op %d ladder needs w0 < w1", what, ci, k);
      if ((op.kind == TQK_B_DENSE1 || op.kind == TQK_B_CTRL1) && (op.mat < 0 || op.mat >= n_mats))
        return -fail(TQK_BAD_SHAPE, "%s: circuit %d op %d matrix index %d (have %d)", what, ci, k, op.mat, n_mats);
    }
    c.first_pass = np;
    const uint32_t full = (n >= 32) ? 0xffffffffu : ((1u << n) - 1u);
    if (n <= T) {  // one tile, one pass
      if (np >= max_passes) return -fail(TQK_SCRATCH_TOO_SMALL, "%s: more than %d passes", what, max_passes);
      for (int k = 0; k < c.num_ops; ++k) ops_out[c.first_op + k] = ops_in[c.first_op + k];
      passes[np++] = {c.first_op, c.num_ops, full, batch::kFirst | batch::kLast};
    } else {
      if (c.state_off < 0) return -fail(TQK_BAD_POINTER, "%s: circuit %d (n=%d) needs a state buffer", what, ci, n);
      const uint32_t low = (1u << batch::kLowReserve) - 1u;
      std::vector<int> pending(c.num_ops), rest;
      for (int k = 0; k < c.num_ops; ++k) pending[k] = c.first_op + k;
      int out = c.first_op;
      do {
        uint32_t tile = low, blocked = 0;
        const int start = out;
        rest.clear();
        for (int idx : pending) {
          uint32_t wb, tg;
          batch::op_bits(ops_in[idx], n, &wb, &tg);
          if ((wb & blocked) == 0u && __builtin_popcount(tile | tg) <= T) {
            tile |= tg;
            ops_out[out++] = ops_in[idx];
          } else {  // stays for a later pass; later ops on these wires must wait too
            blocked |= wb;
            rest.push_back(idx);
          }
        }
        for (int b = 0; b < n && __builtin_popcount(tile) < T; ++b) tile |= 1u << b;  // fill with low bits
        if (np >= max_passes) return -fail(TQK_SCRATCH_TOO_SMALL, "%s: more than %d passes", what, max_passes);
        passes[np++] = {start, out - start, tile & full, 0};
        pending.swap(rest);
      } while (!pending.empty());
      passes[c.first_pass].flags |= batch::kFirst;
      passes[np - 1].flags |= batch::kLast;
    }
    c.num_passes = np - c.first_pass;
  }
  return np;
}

extern "C" int64_t tqk_batch_items(const tqk_batch_circuit* circuits, int ncirc, const tqk_batch_pass* passes,
                                   tqk_batch_item* items, int64_t max_items) {
  const char* what = "tqk_batch_items";
  if (ncirc < 0) return -fail(TQK_BAD_SHAPE, "%s: ncirc %d", what, ncirc);
  if (ncirc > 0 && (!circuits || !passes || !items)) return -fail(TQK_BAD_POINTER, "%s: null pointer", what);
  int max_np = 0;
  for (int c = 0; c < ncirc; ++c) max_np = circuits[c].num_passes > max_np ? circuits[c].num_passes : max_np;
  int64_t k = 0;
  for (int w = 0; w < max_np; ++w) {
    for (int c = 0; c < ncirc; ++c) {
      if (w >= circuits[c].num_passes) continue;
      const int pi = circuits[c].first_pass + w;
      const int ntiles = 1 << (circuits[c].n - __builtin_popcount(passes[pi].tile_mask));
      for (int t = 0; t < ntiles; ++t) {
        if (k >= max_items) return -fail(TQK_SCRATCH_TOO_SMALL, "%s: more than %lld items", what, (long long)max_items);
        items[k++] = {c, pi, t, 0};
      }
    }
  }
  return k;
}

namespace {
// Kernel variants: (threads per CTA, CTAs per SM the register budget is sized for).
template <int THREADS, int MINB>
int launch_batch(const tqk_batch_circuit* circuits, int ncirc, const tqk_batch_op* ops, const tqk_batch_pass* passes,
                 const tqk_batch_item* items, int64_t n_items, const void* mats, void* states, int write_states,
                 double* z_out, int* pass_done, uint64_t* t_done, int* counter, int* status, int tile_bits,
                 int ctas_per_sm, cudaStream_t stream) {
  auto kern = batch::k_batch<THREADS, MINB>;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = sizeof(float2) << tile_bits;
  // attributes are set once per device and variant (before any stream capture: the
  // first launch of a variant on a device must not be captured)
  static int attr_set[64] = {0};
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(float2) << batch::kMaxTileBits));
    attr_set[dev] = 1;
  }
  int fit = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kern, THREADS, smem) != cudaSuccess || fit < 1) fit = 1;
  const int per_sm = ctas_per_sm < fit ? ctas_per_sm : fit;
  const int64_t slots = static_cast<int64_t>(sms) * per_sm;
  const int grid = static_cast<int>(n_items < slots ? n_items : slots);
  kern<<<grid, THREADS, smem, stream>>>(circuits, ncirc, ops, passes, items, n_items,
                                        static_cast<const float2*>(mats), static_cast<float2*>(states), write_states,
                                        z_out, pass_done, reinterpret_cast<unsigned long long*>(t_done), counter,
                                        status, tile_bits);
  return launch_status("tqk_batch_run");
}
}  // namespace

extern "C" int tqk_batch_run(const tqk_batch_circuit* circuits, int ncirc, const tqk_batch_op* ops,
                             const tqk_batch_pass* passes, const tqk_batch_item* items, int64_t n_items,
                             const void* mats, void* states, int write_states, double* z_out, int* pass_done,
                             uint64_t* t_done, int* counter, int* status, const tqk_batch_config* config,
                             void* stream) {
  const char* what = "tqk_batch_run";
  if (ncirc <= 0 || n_items <= 0) return TQK_OK;
  if (!circuits || !passes || !items || !z_out || !pass_done || !counter || !status)
    return fail(TQK_BAD_POINTER, "%s: null pointer", what);
  if (n_items > 0x7fffffff) return fail(TQK_BAD_SHAPE, "%s: too many items", what);
  tqk_batch_config cfg = {TQK_BATCH_TILE_BITS, 512, 1, 0};
  if (config) cfg = *config;
  if (cfg.tile_bits < batch::kMinTileBits || cfg.tile_bits > batch::kMaxTileBits)
    return fail(TQK_BAD_SHAPE, "%s: tile_bits %d outside %d..%d", what, cfg.tile_bits, batch::kMinTileBits,
                batch::kMaxTileBits);
  if (cfg.ctas_per_sm < 1 || cfg.ctas_per_sm > 8)
    return fail(TQK_BAD_SHAPE, "%s: ctas_per_sm %d outside 1..8", what, cfg.ctas_per_sm);
  cudaStream_t s = as_stream(stream);
#define TQK_BATCH_ARGS circuits, ncirc, ops, passes, items, n_items, mats, states, write_states, z_out, pass_done, \
                       t_done, counter, status, cfg.tile_bits, cfg.ctas_per_sm, s
  switch (cfg.threads) {
    case 512:
      return launch_batch<512, 1>(TQK_BATCH_ARGS);
    case 256:
      return cfg.ctas_per_sm >= 4 ? launch_batch<256, 4>(TQK_BATCH_ARGS) : launch_batch<256, 2>(TQK_BATCH_ARGS);
    case 128:
      return launch_batch<128, 8>(TQK_BATCH_ARGS);
    default:
      return fail(TQK_BAD_SHAPE, "%s: threads %d (128, 256 or 512)", what, cfg.threads);
  }
#undef TQK_BATCH_ARGS
}
