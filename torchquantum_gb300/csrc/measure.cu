// measure.cu -- probabilities and Pauli-string expectation values.
//
// <psi|P|psi> for P = (x) sigma_w is evaluated from two bit masks over the in-row
// index: xmask (X or Y on the wire) and zmask (Z or Y), with
//   (P psi)_i = i^{#Y} (-1)^{popcount((i ^ x) & z)} psi_{i ^ x}.
// Strings that all share one xmask are evaluated 8 at a time in one pass over the state
// (each amplitude pair (i, i^x) is read once for all of them).  Strings with several
// xmasks are grouped and each group is one coset pass (k_coset): the row is cut into
// cosets of the span of the group's xmasks, staged in shared memory (16-byte cp.async copies), so
// all partners are read on chip and DRAM reads the state once per group.  Each thread
// accumulates in float32, blocks reduce in float64 and write one partial per (row,
// block or coset, string) to scratch; a second kernel adds the partials in a fixed
// order, so results are bitwise reproducible run to run.  The backward seed
// sum_s c_s P_s psi (k_coset<true>) uses the same coset passes.
#include <atomic>
#include <mutex>
#include <vector>

#include "bulk.cuh"
#include "common.cuh"

namespace tqk {

constexpr int kMaxStringsPerPass = 8;

// Blocks per row for the reduction passes: enough to fill the GPU, bounded so the
// partials stay small.  Depends only on (bsz, n) so scratch size is a pure function.
static int64_t reduce_blocks_per_row(int64_t bsz, int n) {
  const int64_t amps = 1ll << n;
  const int64_t want = (152 * 8 + bsz - 1) / bsz;        // ~8 blocks of 256 per SM overall
  const int64_t cap = (amps / 4 + 255) / 256;            // at least one float4 pair per thread
  int64_t b = want < cap ? want : cap;
  return b < 1 ? 1 : b;
}

template <int NV>
__device__ __forceinline__ void block_reduce_store(float (&v)[NV], double* dst, int count) {
  __shared__ double red[32][NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) red[warp][j] = (double)v[j];
  }
  __syncthreads();
  if (warp == 0 && lane < count) {
    double s = 0.0;
    for (int w = 0; w < nwarps; ++w) s += red[w][lane];
    dst[lane] = s;
  }
}

struct ExpvalParams {
  const float2* state;
  int n;
  uint64_t x;
  int hbit;                       // highest set bit of x (x != 0)
  int ns;                         // strings in this pass
  uint64_t z[kMaxStringsPerPass];
  int ny[kMaxStringsPerPass];     // number of Y mod 4
  int col[kMaxStringsPerPass];    // output column of each string
  int m;                          // total strings (partial row stride)
  int64_t work;                   // work items per row
  double* partial;                // [bsz][gridDim.x][m]
};


// Sign algebra of one pass.  All strings of a pass share the X-mask x; the pass visits
// even indices i (bit 0 clear) and their partners i ^ x.  Per string (z its Z-mask, ny
// its number of Y factors mod 4, so popcount(x & z) = ny mod 2):
//   (-1)^popcount((i ^ x) & z)       = (-1)^popcount(i & z) * (-1)^ny,
//   (-1)^popcount(((i + 1) ^ x) & z) = (-1)^popcount((i ^ x) & z) * (-1)^(z & 1).
// The pair (a = psi[i], b = psi[i ^ x]) contributes conj(a) (P psi)_i + conj(b) (P psi)_{i^x}
//   = 2 (-1)^popcount(i & z) F[ny] * (ny odd ? Im : Re)(conj(a) b),  F = (1, 1, -1, -1),
// so a pass needs one popcount per string for two pairs instead of four.
__device__ __forceinline__ float flip_if_odd(float v, uint32_t parity_bits) {  // v * (-1)^popcount
  return __int_as_float(__float_as_int(v) ^ static_cast<int>(parity_bits << 31));
}
template <typename I>
__device__ __forceinline__ uint32_t popc_t(I v) {
  if constexpr (sizeof(I) == 8) return static_cast<uint32_t>(__popcll(v));
  else return static_cast<uint32_t>(__popc(v));
}

// Per-string constants of a pass, kept in registers.
template <int NS, typename I>
struct PassStrings {
  I z[NS];
  float f[NS];       // 2 F[ny] (diagonal pass: 1)
  uint32_t odd[NS];  // ny odd: take the imaginary part
  float z0[NS];      // (-1)^(z & 1)
  __device__ __forceinline__ void load(const ExpvalParams& p, float scale) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      const int ny = s < p.ns ? p.ny[s] : 0;
      z[s] = s < p.ns ? static_cast<I>(p.z[s]) : I(0);
      f[s] = ny >= 2 ? -scale : scale;
      odd[s] = static_cast<uint32_t>(ny & 1);
      z0[s] = (z[s] & I(1)) ? -1.f : 1.f;
    }
  }
};

// x == 0: diagonal strings, contribution |psi_i|^2 * (-1)^{popcount(i & z)}
// NS: strings the pass's accumulators hold (1, 2, 4 or 8 >= p.ns): fewer registers for
// the common one-string pass, so more warps -- more loads in flight -- per SM.
// I: index type (32-bit for rows of up to 2^31 amplitudes).
template <int NS, typename I>
__global__ void __launch_bounds__(256) k_expval_diag(const ExpvalParams p) {
  const int64_t b = blockIdx.y;
  const float2* row = p.state + (b << p.n);
  PassStrings<NS, I> ps;
  ps.load(p, 1.f);
  float acc[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) acc[s] = 0.f;
  const I work = static_cast<I>(p.work), stride = static_cast<I>(gridDim.x * blockDim.x);
  for (I t = static_cast<I>(blockIdx.x * blockDim.x + threadIdx.x); t < work; t += stride) {
    const I i = t * 2;
    const float4 v = ld4(row + i);
    const float p0 = v.x * v.x + v.y * v.y, p1 = v.z * v.z + v.w * v.w;
#pragma unroll
    for (int s = 0; s < NS; ++s)
      if (s < p.ns) acc[s] += flip_if_odd(fmaf(ps.z0[s], p1, p0), popc_t<I>(i & ps.z[s]));
  }
  block_reduce_store<NS>(acc, p.partial + (b * gridDim.x + blockIdx.x) * kMaxStringsPerPass, p.ns);
}

// x != 0: pairs (i, i^x) with bit hbit of i clear.
template <bool LOWX, int NS, typename I>  // LOWX: x == 1 (the pair is one float4)
__global__ void __launch_bounds__(256) k_expval_pair(const ExpvalParams p) {
  const int64_t b = blockIdx.y;
  const float2* row = p.state + (b << p.n);
  PassStrings<NS, I> ps;
  ps.load(p, 2.f);
  float acc[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) acc[s] = 0.f;
  const I x = static_cast<I>(p.x);
  const int hb = p.hbit;
  const I lomask = (I(1) << hb) - I(1);
  const bool sw = (x & I(1)) != 0;
  const I work = static_cast<I>(p.work), stride = static_cast<I>(gridDim.x * blockDim.x);
  for (I t = static_cast<I>(blockIdx.x * blockDim.x + threadIdx.x); t < work; t += stride) {
    if (LOWX) {
      const I i = t * 2;  // bit 0 clear, partner i + 1
      const float4 v = ld4(row + i);
      const float ur = v.x * v.z + v.y * v.w, ui = v.x * v.w - v.y * v.z;  // conj(a) b
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s < p.ns) acc[s] += flip_if_odd(ps.f[s] * (ps.odd[s] ? ui : ur), popc_t<I>(i & ps.z[s]));
    } else {
      const I g = t * 2;  // two consecutive groups: i, i + 1 (hbit >= 1, so i is even)
      const I i = ((g >> hb) << (hb + 1)) | (g & lomask);
      const float4 v = ld4(row + i);
      const float4 w = ld4(row + ((i ^ x) & ~I(1)));
      const float2 a0 = lo2(v), a1 = hi2(v);
      const float2 b0 = sw ? hi2(w) : lo2(w), b1 = sw ? lo2(w) : hi2(w);
      const float ur0 = a0.x * b0.x + a0.y * b0.y, ui0 = a0.x * b0.y - a0.y * b0.x;
      const float ur1 = a1.x * b1.x + a1.y * b1.y, ui1 = a1.x * b1.y - a1.y * b1.x;
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s < p.ns) {
          const float c = ps.odd[s] ? fmaf(ps.z0[s], ui1, ui0) : fmaf(ps.z0[s], ur1, ur0);
          acc[s] += flip_if_odd(ps.f[s] * c, popc_t<I>(i & ps.z[s]));
        }
    }
  }
  block_reduce_store<NS>(acc, p.partial + (b * gridDim.x + blockIdx.x) * kMaxStringsPerPass, p.ns);
}

// The two kernels above store block partials contiguously as [row][block][slot];
// this kernel reduces them in block order into out[row*m + col].
// Launch the pass kernel with the smallest accumulator count that holds p.ns strings.
template <int NS, typename I>
void launch_expval_ns(const ExpvalParams& p, dim3 grid, cudaStream_t st) {
  if (p.x == 0) k_expval_diag<NS, I><<<grid, 256, 0, st>>>(p);
  else if (p.x == 1ull) k_expval_pair<true, NS, I><<<grid, 256, 0, st>>>(p);
  else k_expval_pair<false, NS, I><<<grid, 256, 0, st>>>(p);
}

template <typename I>
void launch_expval_i(const ExpvalParams& p, dim3 grid, cudaStream_t st) {
  if (p.ns <= 1) launch_expval_ns<1, I>(p, grid, st);
  else if (p.ns <= 2) launch_expval_ns<2, I>(p, grid, st);
  else if (p.ns <= 4) launch_expval_ns<4, I>(p, grid, st);
  else launch_expval_ns<8, I>(p, grid, st);
}

inline void launch_expval(const ExpvalParams& p, dim3 grid, cudaStream_t st) {
  if (p.n <= 31) launch_expval_i<uint32_t>(p, grid, st);
  else launch_expval_i<uint64_t>(p, grid, st);
}

struct FinishCols {
  int c[kMaxStringsPerPass];
};

// One CTA of kFinishThreads per row: thread t sums the partials k = t, t + kFinishThreads,
// ... of every slot, then a fixed tree in shared memory adds the threads' sums (the same
// order on every call, so the results are deterministic).
constexpr int kFinishThreads = 128;

__global__ void __launch_bounds__(kFinishThreads) k_expval_finish(const double* partial, int64_t nblk, int ns,
                                                                  int slot_stride, const FinishCols cols, int m,
                                                                  double* out, int64_t bsz) {
  __shared__ double red[kMaxStringsPerPass][kFinishThreads];
  const int64_t b = blockIdx.x;
  double acc[kMaxStringsPerPass];
#pragma unroll
  for (int s = 0; s < kMaxStringsPerPass; ++s) acc[s] = 0.0;
  for (int64_t k = threadIdx.x; k < nblk; k += kFinishThreads) {
    const double* pk = partial + (b * nblk + k) * slot_stride;
#pragma unroll
    for (int s = 0; s < kMaxStringsPerPass; ++s)
      if (s < ns) acc[s] += pk[s];
  }
#pragma unroll
  for (int s = 0; s < kMaxStringsPerPass; ++s) red[s][threadIdx.x] = acc[s];
  __syncthreads();
  for (int half = kFinishThreads / 2; half > 0; half >>= 1) {
    if (threadIdx.x < half)
      for (int s = 0; s < ns; ++s) red[s][threadIdx.x] += red[s][threadIdx.x + half];
    __syncthreads();
  }
  if (threadIdx.x < ns) out[b * m + cols.c[threadIdx.x]] = red[threadIdx.x][0];
}

// ------------------------------------------------------------------ coset passes
// Strings with different X-masks are evaluated from shared memory: the in-row index space
// is cut into cosets of the subgroup the strings' X-masks span, one coset per pipeline
// stage, so every partner amplitude psi[i ^ x_s] of every string of the group is read on
// chip and DRAM reads each amplitude once per pass.
//
// Chunks: the lowest c index bits stay contiguous (runs of 2^c amplitudes, copied in
// 16-byte pieces: bulk copies of runs this short are limited by the copy engine's
// per-request cost, not by bandwidth).  The high parts x_s >> c of the group's X-masks span an r-dimensional space;
// b_0..b_{r-1} is its reduced echelon basis (pivot bits p_0 < ... < p_{r-1}, each present
// in its own basis vector only).  Coset t of a row is rep(t) + span{b_k} over the high
// index bits, rep(t) = t with zeros inserted at the pivot bits; stage slot a (r bits)
// holds the chunk at high index h(t, a) = rep(t) ^ sum_k a_k b_k, so a stage is 2^(c + r)
// amplitudes.  In stage coordinates u = (a << c) | l the partner of u under string s is
// u ^ xs_s, xs_s = (a_s << c) | (x_s mod 2^c), a_s the basis coefficients of x_s >> c.
// Signs: for the in-row index i of u, parity(i & z_s) = rho_s(t) ^ parity(u & gam_s) with
// gam_s = (beta_s << c) | (z_s mod 2^c), beta_s bit k = parity(b_k & (z_s >> c)) and
// rho_s(t) = parity(rep(t) & (z_s >> c)).
// Grouping (host): strings are taken in order while some c in [min(4, T), T] has
// c + r <= T, T = min(n, 13), and the group holds at most 8 strings; the widest such c is
// used, which makes c + r = T: every stage is 2^T amplitudes (64 KB at n >= 13) and a row
// has 2^(n - T) cosets.
//
// CTA: sixteen warps and three stages.  At the top of each iteration every thread issues
// its 16-byte cp.async pieces of the coset two iterations ahead into the stage the previous
// iteration finished reading, and arrives on that stage's full mbarrier once they land;
// then all wait for the current stage.  Expvals: each warp sums its segment of the strings'
// pair visits in float32, the CTA reduces in float64 and writes one partial per (coset,
// string); the partials are summed per row in a fixed order (k_expval_finish).  Backward
// seed: each thread forms sum_s c_s (P_s psi)_u for two amplitudes and stores them to the
// output row (added to what is there for groups after the first).
// Every mbarrier wait is bounded: on expiry the CTA records TQK_TIMEOUT in the status
// word, stops issuing copies and waiting, writes NaN expval partials (the seed skips its
// stores), waits (bounded) for its copies in flight and exits.
constexpr int kCosetTileBits = 13;
constexpr int kCosetMinChunkBits = 4;
constexpr int kCosetMaxRank = kCosetTileBits - kCosetMinChunkBits;
constexpr int kCosetStages = 3;
constexpr int kCosetWarps = 16;
constexpr int kCosetThreads = 32 * kCosetWarps;

struct CosetParams {
  const float2* state;
  float2* out;       // seed: output rows; expvals: unused
  const float* coef; // seed: [bsz][m] weights; column col[s]
  double* partial;   // expvals: [bsz * cosets][kMaxStringsPerPass]
  int* status;
  int64_t bsz, cosets;  // cosets per row = 2^(n - c - r)
  int n, c, r, tb;      // tb = c + r
  int m, accumulate, ns;
  uint32_t basis[kCosetMaxRank];
  int piv[kCosetMaxRank];  // ascending
  uint32_t xs[kMaxStringsPerPass], gam[kMaxStringsPerPass], zh[kMaxStringsPerPass];
  uint32_t fl[kMaxStringsPerPass];   // constant sign bit (expvals: ny >> 1; seed: (ny & 1) ^ (ny >> 1))
  uint32_t odd[kMaxStringsPerPass];  // ny & 1
  uint32_t kind[kMaxStringsPerPass]; // expvals: 0 diagonal (xs = 0), 1 xs = 1, 2 other, 3 padding
  uint32_t hb[kMaxStringsPerPass];   // expvals, kind 2: highest set bit of xs
  int col[kMaxStringsPerPass];
};

__device__ __forceinline__ void mbar_init_count(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bulk::smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bulk::smem_addr(bar)) : "memory");
}
__device__ __forceinline__ float4 lds4(const float2* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(bulk::smem_addr(dst)), "l"(src) : "memory");
}
// Arrive on bar once every cp.async this thread issued so far has landed (the barrier's
// expected count includes this thread).
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bulk::smem_addr(bar)) : "memory");
}

// rep(t): t with a zero inserted at each pivot bit (ascending)
__device__ __forceinline__ uint32_t coset_rep(uint32_t t, const CosetParams& p) {
  for (int k = 0; k < p.r; ++k) {
    const int q = p.piv[k];
    t = ((t >> q) << (q + 1)) | (t & ((1u << q) - 1u));
  }
  return t;
}

// The coset stages (dynamic shared memory), indexed as float4 pairs of amplitudes so that
// every access below is a 32-bit shared-memory load.
extern __shared__ __align__(128) float4 coset_stage4[];

// One string's sum over a warp's segment of a staged coset (stage base b4, in float4 units;
// the lane visits j = j0, j0 + 32, ... < j1), each amplitude pair (u, u + 1) with bit h of u
// clear (j counts those pairs) against its partner pair
// ((u ^ x) & ~1); SW: x is odd, so the partner pair is in swapped order; ODD: odd number of Y
// factors (imaginary part).  Returns the thread's float32 partial of the half sum.
template <bool SW, bool ODD>
__device__ __forceinline__ float coset_string_sum(uint32_t b4, uint32_t j0, uint32_t j1, uint32_t h, uint32_t x,
                                                  uint32_t gam, uint32_t rho) {
  const uint32_t lo = (1u << h) - 1u;
  const uint32_t g1 = gam & 1u;
  const uint32_t x4 = x >> 1;  // partner pair index = (u >> 1) ^ (x >> 1)
  float a = 0.f;
#pragma unroll 4
  for (uint32_t j = j0; j < j1; j += 32) {
    // pair index of u: j with a zero inserted at bit h - 1 (u = 2 x pair index, h >= 1)
    const uint32_t pu = ((j >> (h - 1)) << h) | (j & (lo >> 1));
    const float4 v = coset_stage4[b4 + pu];
    const float4 w = coset_stage4[b4 + (pu ^ x4)];
    const float2 a0 = lo2(v), a1 = hi2(v);
    const float2 b0 = SW ? hi2(w) : lo2(w), b1 = SW ? lo2(w) : hi2(w);
    const float c0 = ODD ? a0.x * b0.y - a0.y * b0.x : a0.x * b0.x + a0.y * b0.y;
    const float c1 = ODD ? a1.x * b1.y - a1.y * b1.x : a1.x * b1.x + a1.y * b1.y;
    a += flip_if_odd(c0 + flip_if_odd(c1, g1), static_cast<uint32_t>(__popc((pu << 1) & gam)) + rho);
  }
  return a;
}

// Diagonal string (x = 0): sum of +-|psi_u|^2 over every pair of the coset.
__device__ __forceinline__ float coset_diag_sum(uint32_t b4, uint32_t j0, uint32_t j1, uint32_t gam, uint32_t rho) {
  const uint32_t g1 = gam & 1u;
  float a = 0.f;
  for (uint32_t j = j0; j < j1; j += 32) {
    const float4 v = coset_stage4[b4 + j];
    const float p0 = v.x * v.x + v.y * v.y, p1 = v.z * v.z + v.w * v.w;
    a += flip_if_odd(p0 + flip_if_odd(p1, g1), static_cast<uint32_t>(__popc((j << 1) & gam)) + rho);
  }
  return a;
}

// x = 1: each pair (u, u + 1) is its own partner; the u-side term (counted twice by the caller).
__device__ __forceinline__ float coset_x1_sum(uint32_t b4, uint32_t j0, uint32_t j1, bool odd, uint32_t gam,
                                              uint32_t rho) {
  float a = 0.f;
  for (uint32_t j = j0; j < j1; j += 32) {
    const float4 v = coset_stage4[b4 + j];
    const float c0 = odd ? v.x * v.w - v.y * v.z : v.x * v.z + v.y * v.w;
    a += flip_if_odd(c0, static_cast<uint32_t>(__popc((j << 1) & gam)) + rho);
  }
  return a;
}

// Stage `st` <- the coset of pipeline iteration `item` (one call per thread: its 16-byte
// pieces k = tid, tid + threads, ..., then an arrive on the stage's full barrier once they
// have landed).  Slot a of the stage holds the chunk at high index rep ^ slot_hi[a].
__device__ __forceinline__ void coset_issue(const CosetParams& p, int64_t item, int st, const uint32_t* slot_hi,
                                            uint64_t* full) {
  const uint32_t tile = 1u << p.tb;
  const int64_t b = item / p.cosets;
  const uint32_t rep = coset_rep(static_cast<uint32_t>(item - b * p.cosets), p);
  const uint32_t pmask = (1u << (p.c - 1)) - 1u;  // 16-byte pieces per chunk, minus one
  const float2* row = p.state + (static_cast<uint64_t>(b) << p.n);
  float2* dst = reinterpret_cast<float2*>(coset_stage4) + static_cast<size_t>(st) * tile;
  for (uint32_t k = threadIdx.x; k < (tile >> 1); k += kCosetThreads) {
    const uint32_t a = k >> (p.c - 1), off = (k & pmask) << 1;
    cp_async16(dst + (static_cast<size_t>(a) << p.c) + off,
               row + (static_cast<uint64_t>(rep ^ slot_hi[a]) << p.c) + off);
  }
  cp_async_arrive(&full[st]);
}

// Backward seed, one string over a thread's output pairs of a staged coset: pair k is
// q0 + k * kCosetThreads (local index u = 2q), its partner pair (q ^ x4) in the stage.  The
// sign (-1)^popcount(u & gam) splits into the thread's part (bits of 2 q0, folded into cft)
// and the part from k * 2 kCosetThreads, the same for every thread; SW: x odd (the partner
// pair is in swapped order); ODD: odd number of Y factors.
constexpr int kSeedPairs = (1 << kCosetTileBits) / 2 / kCosetThreads;

template <bool SW, bool ODD, bool FULL>
__device__ __forceinline__ void seed_string(float2 (&o)[kSeedPairs][2], uint32_t b4, uint32_t q0, uint32_t npairs,
                                            uint32_t x4, uint32_t gam, float cft) {
  const uint32_t g1 = gam & 1u;
  // FULL (tiles of 2^13 amplitudes): every thread has all its pairs, so the loads of all
  // of them can be issued before the first product
  float4 w[kSeedPairs];
#pragma unroll
  for (int k = 0; k < kSeedPairs; ++k) {
    const uint32_t q = q0 + static_cast<uint32_t>(k) * kCosetThreads;
    w[k] = (FULL || q < npairs) ? coset_stage4[b4 + (q ^ x4)] : make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int k = 0; k < kSeedPairs; ++k) {
    const uint32_t q = q0 + static_cast<uint32_t>(k) * kCosetThreads;
    if (!FULL && q >= npairs) break;  // tiles of fewer than 2^13 amplitudes
    const uint32_t up = static_cast<uint32_t>(__popc((static_cast<uint32_t>(k) * 2u * kCosetThreads) & gam));
    const float c0 = flip_if_odd(cft, up), c1 = flip_if_odd(cft, up + g1);
    const float2 b0 = SW ? hi2(w[k]) : lo2(w[k]), b1 = SW ? lo2(w[k]) : hi2(w[k]);
    if (ODD) {
      o[k][0].x = fmaf(-c0, b0.y, o[k][0].x);
      o[k][0].y = fmaf(c0, b0.x, o[k][0].y);
      o[k][1].x = fmaf(-c1, b1.y, o[k][1].x);
      o[k][1].y = fmaf(c1, b1.x, o[k][1].y);
    } else {
      o[k][0].x = fmaf(c0, b0.x, o[k][0].x);
      o[k][0].y = fmaf(c0, b0.y, o[k][0].y);
      o[k][1].x = fmaf(c1, b1.x, o[k][1].x);
      o[k][1].y = fmaf(c1, b1.y, o[k][1].y);
    }
  }
}

template <bool SEED, int NS>
__global__ void __launch_bounds__(kCosetThreads, 1) k_coset(const CosetParams p) {
  __shared__ __align__(8) uint64_t full[kCosetStages];
  __shared__ uint32_t slot_hi[1 << kCosetMaxRank];  // sum_k a_k b_k for slot a
  __shared__ float red[2][kCosetWarps][kMaxStringsPerPass];
  __shared__ int quit;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t tile = 1u << p.tb;
  for (int a = threadIdx.x; a < (1 << p.r); a += kCosetThreads) {
    uint32_t h = 0;
    for (int k = 0; k < p.r; ++k)
      if ((a >> k) & 1) h ^= p.basis[k];
    slot_hi[a] = h;
  }
  if (threadIdx.x == 0) {
    for (int st = 0; st < kCosetStages; ++st) mbar_init_count(&full[st], kCosetThreads);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    quit = 0;
  }
  __syncthreads();
  const int64_t total = p.bsz * p.cosets;
  volatile int* vquit = &quit;
  // prologue: the first kCosetStages - 1 cosets in flight
  int64_t issued = 0;  // pipeline iterations whose loads this CTA issued
  for (; issued < kCosetStages - 1 && blockIdx.x + issued * gridDim.x < total; ++issued)
    coset_issue(p, blockIdx.x + issued * gridDim.x, static_cast<int>(issued), slot_hi, full);
  // expvals: pair visits of all strings in a coset (tile / 4 per string, tile / 2 for x = 0
  // or 1; strings past ns are padding)
  uint32_t visits = 0;
  for (int s = 0; s < p.ns; ++s) visits += p.kind[s] == 3u ? 0u : (p.kind[s] == 2u ? tile >> 2 : tile >> 1);
  const uint32_t lmask = (1u << p.c) - 1u;
  int it = 0;
  for (int64_t item = blockIdx.x; item < total; item += gridDim.x, ++it) {
    const int st = it % kCosetStages;
    // every thread finished reading the stage of iteration it - 1 (the barrier that closed
    // it): refill it with the coset kCosetStages - 1 iterations ahead
    const int64_t ahead = item + static_cast<int64_t>(kCosetStages - 1) * gridDim.x;
    if (ahead < total && *vquit == 0) {
      coset_issue(p, ahead, static_cast<int>(issued % kCosetStages), slot_hi, full);
      ++issued;
    }
    const int64_t b = item / p.cosets;
    const uint32_t rep = coset_rep(static_cast<uint32_t>(item - b * p.cosets), p);
    bool ok = *vquit == 0;
    if (ok && !bulk::mbar_wait(&full[st], static_cast<uint32_t>(it / kCosetStages) & 1u)) {
      ok = false;
      if (lane == 0) {
        atomicExch(p.status, TQK_TIMEOUT);
        *vquit = 1;
      }
    }
    const uint32_t b4 = static_cast<uint32_t>(st) * (tile >> 1);  // stage start, float4 units
    if (ok && SEED) {
      // string by string over the thread's output pairs (outputs in registers), then one
      // store per pair; each string's orientation and Y parity are fixed for its loop
      const uint32_t npairs = tile >> 1, q0 = threadIdx.x;
      float2 o[kSeedPairs][2];
#pragma unroll
      for (int k = 0; k < kSeedPairs; ++k) o[k][0] = o[k][1] = make_float2(0.f, 0.f);
#pragma unroll 1
      for (int s = 0; s < p.ns; ++s) {
        const uint32_t x = p.xs[s], gam_s = p.gam[s];
        const uint32_t rho_s = (static_cast<uint32_t>(__popc(rep & p.zh[s])) ^ p.fl[s]) & 1u;
        const float cft = flip_if_odd(__ldg(p.coef + b * p.m + p.col[s]),
                                      static_cast<uint32_t>(__popc((q0 << 1) & gam_s)) + rho_s);
        const uint32_t x4 = x >> 1;
        const int variant = ((x & 1u) ? 2 : 0) + (p.odd[s] ? 1 : 0);
        if (npairs == static_cast<uint32_t>(kSeedPairs * kCosetThreads)) {
          if (variant == 3) seed_string<true, true, true>(o, b4, q0, npairs, x4, gam_s, cft);
          else if (variant == 2) seed_string<true, false, true>(o, b4, q0, npairs, x4, gam_s, cft);
          else if (variant == 1) seed_string<false, true, true>(o, b4, q0, npairs, x4, gam_s, cft);
          else seed_string<false, false, true>(o, b4, q0, npairs, x4, gam_s, cft);
        } else {
          if (variant == 3) seed_string<true, true, false>(o, b4, q0, npairs, x4, gam_s, cft);
          else if (variant == 2) seed_string<true, false, false>(o, b4, q0, npairs, x4, gam_s, cft);
          else if (variant == 1) seed_string<false, true, false>(o, b4, q0, npairs, x4, gam_s, cft);
          else seed_string<false, false, false>(o, b4, q0, npairs, x4, gam_s, cft);
        }
      }
#pragma unroll
      for (int k = 0; k < kSeedPairs; ++k) {
        const uint32_t q = q0 + static_cast<uint32_t>(k) * kCosetThreads;
        if (q >= npairs) break;
        const uint32_t u = q << 1;
        float2* dst = p.out + (static_cast<uint64_t>(b) << p.n) +
                      (static_cast<uint64_t>(rep ^ slot_hi[u >> p.c]) << p.c) + (u & lmask);
        float2 o0 = o[k][0], o1 = o[k][1];
        if (p.accumulate) {
          const float4 old = ld4(dst);
          o0.x += old.x;
          o0.y += old.y;
          o1.x += old.z;
          o1.y += old.w;
        }
        st4(dst, pack4(o0, o1));
      }
    } else if (ok) {
      // expvals: the visits of all strings in a row (tile / 4 pairs per string, tile / 2 for
      // x = 0 or 1) are cut into one contiguous segment per warp, so a warp takes one or two
      // strings, each with its orientation and Y parity fixed for the loop.  A pair of
      // amplitude pairs (u, u + 1) / ((u ^ xs) & ~1) is visited once, from the side whose bit
      // hb (the highest of xs) is clear -- enumerated directly by inserting a zero at hb --
      // and counted twice (P is Hermitian: both sides contribute the same real part).
      const uint32_t per = ((visits + kCosetWarps - 1) / kCosetWarps + 31u) & ~31u;
      const uint32_t w0 = static_cast<uint32_t>(warp) * per, w1 = min(visits, w0 + per);
      // the warp's row of red: zero, then the sums of the strings its segment touches (one
      // string body in the code, looped at run time, instead of one per string)
      if (lane < NS) red[it & 1][warp][lane] = 0.f;
      __syncwarp();
      uint32_t f0 = 0;
#pragma unroll 1
      for (int s = 0; s < p.ns && f0 < w1; ++s) {
        const uint32_t ks = p.kind[s];
        const uint32_t f1 = f0 + (ks == 3u ? 0u : (ks == 2u ? tile >> 2 : tile >> 1));
        const uint32_t lo = max(f0, w0), hi = min(f1, w1);
        if (lo < hi) {  // uniform for the warp
          const uint32_t j0 = lo - f0 + lane, j1 = hi - f0;
          const uint32_t xs_s = p.xs[s], gam_s = p.gam[s], hb_s = p.hb[s], odd_s = p.odd[s];
          const uint32_t rho_s = (static_cast<uint32_t>(__popc(rep & p.zh[s])) ^ p.fl[s]) & 1u;
          float a;
          if (ks == 0u) a = coset_diag_sum(b4, j0, j1, gam_s, rho_s);
          else if (ks == 1u) a = 2.f * coset_x1_sum(b4, j0, j1, odd_s != 0u, gam_s, rho_s);
          else if (xs_s & 1u)
            a = 2.f * (odd_s ? coset_string_sum<true, true>(b4, j0, j1, hb_s, xs_s, gam_s, rho_s)
                             : coset_string_sum<true, false>(b4, j0, j1, hb_s, xs_s, gam_s, rho_s));
          else
            a = 2.f * (odd_s ? coset_string_sum<false, true>(b4, j0, j1, hb_s, xs_s, gam_s, rho_s)
                             : coset_string_sum<false, false>(b4, j0, j1, hb_s, xs_s, gam_s, rho_s));
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
          if (lane == 0) red[it & 1][warp][s] = a;
        }
        f0 = f1;
      }
    } else if (!SEED) {
      if (lane < NS) red[it & 1][warp][lane] = 0.f;  // a stage that never arrived: its partials are NaN below
    }
    __syncthreads();  // the stage is read: the next iteration may refill it
    if (!SEED && warp == 0 && lane < p.ns) {
      double sum = 0.0;
      for (int w = 0; w < kCosetWarps; ++w) sum += static_cast<double>(red[it & 1][w][lane]);
      p.partial[item * kMaxStringsPerPass + lane] = (*vquit == 0) ? sum : __longlong_as_double(0x7ff8000000000000ll);
    }
  }
  // after a timeout, wait (bounded) for this CTA's copies still in flight before exiting
  if (quit && threadIdx.x == 0) {
    for (int64_t k = issued - (kCosetStages - 1); k < issued; ++k)
      if (k >= 0) bulk::mbar_wait(&full[k % kCosetStages], static_cast<uint32_t>(k / kCosetStages) & 1u);
  }
}

// Host plan of one coset pass.
struct CosetGroup {
  int c, r, ns;
  uint32_t basis[kCosetMaxRank];
  int piv[kCosetMaxRank];
  int idx[kMaxStringsPerPass];
};

// Reduced echelon basis of the vectors (GF(2)); returns the rank, or -1 past max_rank.
static int gf2_reduced_basis(const uint32_t* v, int cnt, uint32_t* basis, int* piv, int max_rank) {
  int r = 0;
  for (int i = 0; i < cnt; ++i) {
    uint32_t x = v[i];
    for (int k = 0; k < r; ++k)
      if ((x >> piv[k]) & 1u) x ^= basis[k];
    if (x == 0) continue;
    if (r == max_rank) return -1;
    const int q = 31 - __builtin_clz(x);
    for (int k = 0; k < r; ++k)
      if ((basis[k] >> q) & 1u) basis[k] ^= x;
    basis[r] = x;
    piv[r] = q;
    ++r;
  }
  for (int i = 1; i < r; ++i)  // ascending pivots
    for (int j = i; j > 0 && piv[j - 1] > piv[j]; --j) {
      const int tp = piv[j];
      piv[j] = piv[j - 1];
      piv[j - 1] = tp;
      const uint32_t tb = basis[j];
      basis[j] = basis[j - 1];
      basis[j - 1] = tb;
    }
  return r;
}

// Rank of {x_j >> c} (j in idx), or -1 when it exceeds max_rank.
static int coset_rank(const uint64_t* xmask, const int* idx, int cnt, int c, int max_rank, uint32_t* basis,
                      int* piv) {
  uint32_t v[kMaxStringsPerPass];
  for (int i = 0; i < cnt; ++i) v[i] = static_cast<uint32_t>(xmask[idx[i]] >> c);
  return gf2_reduced_basis(v, cnt, basis, piv, max_rank);
}

// Greedy grouping of the strings (in order) into coset passes; fills the groups' c and
// basis.  n <= 34, so x >> c fits 32 bits for c >= 4 (and c = n for n <= 4).
static void coset_plan(int n, const uint64_t* xmask, int m, std::vector<CosetGroup>& groups) {
  const int T = n < kCosetTileBits ? n : kCosetTileBits;
  const int cmin = T < kCosetMinChunkBits ? T : kCosetMinChunkBits;
  groups.clear();
  CosetGroup g;
  g.ns = 0;
  uint32_t basis[kCosetMaxRank];
  int piv[kCosetMaxRank];
  for (int j = 0; j < m; ++j) {
    if (g.ns > 0) {
      g.idx[g.ns] = j;
      const bool fits = g.ns < kMaxStringsPerPass && coset_rank(xmask, g.idx, g.ns + 1, cmin, T - cmin, basis, piv) >= 0;
      if (!fits) {
        groups.push_back(g);
        g.ns = 0;
      }
    }
    g.idx[g.ns++] = j;
  }
  if (g.ns > 0) groups.push_back(g);
  for (CosetGroup& gr : groups) {
    int c = cmin;
    while (c < T && coset_rank(xmask, gr.idx, gr.ns, c + 1, T - (c + 1), basis, piv) >= 0) ++c;
    gr.c = c;
    gr.r = coset_rank(xmask, gr.idx, gr.ns, c, T - c, gr.basis, gr.piv);
  }
}

static int coset_tile_bits(int n) { return n < kCosetTileBits ? n : kCosetTileBits; }

// Stage coordinates of the group's strings; per-string sign constants.
static void coset_params(const CosetGroup& g, int n, const uint64_t* xmask, const uint64_t* zmask, bool seed,
                         CosetParams& p) {
  p.n = n;
  p.c = g.c;
  p.r = g.r;
  p.tb = g.c + g.r;
  p.cosets = 1ll << (n - p.tb);
  p.ns = g.ns;
  for (int k = 0; k < kCosetMaxRank; ++k) {
    p.basis[k] = k < g.r ? g.basis[k] : 0u;
    p.piv[k] = k < g.r ? g.piv[k] : 0;
  }
  const uint32_t lmask = (1u << g.c) - 1u;
  for (int s = 0; s < kMaxStringsPerPass; ++s) {
    if (s >= g.ns) {
      p.xs[s] = p.gam[s] = p.zh[s] = p.fl[s] = p.odd[s] = p.hb[s] = 0u;
      p.kind[s] = 3u;
      p.col[s] = 0;
      continue;
    }
    const int j = g.idx[s];
    const uint32_t xh = static_cast<uint32_t>(xmask[j] >> g.c), zh = static_cast<uint32_t>(zmask[j] >> g.c);
    uint32_t a = 0, beta = 0;
    for (int k = 0; k < g.r; ++k) {
      if ((xh >> g.piv[k]) & 1u) a |= 1u << k;
      if (__builtin_popcount(g.basis[k] & zh) & 1) beta |= 1u << k;
    }
    const int ny = __builtin_popcountll(xmask[j] & zmask[j]) & 3;
    p.xs[s] = (a << g.c) | (static_cast<uint32_t>(xmask[j]) & lmask);
    p.gam[s] = (beta << g.c) | (static_cast<uint32_t>(zmask[j]) & lmask);
    p.zh[s] = zh;
    p.odd[s] = static_cast<uint32_t>(ny & 1);
    p.fl[s] = seed ? static_cast<uint32_t>((ny & 1) ^ (ny >> 1)) : static_cast<uint32_t>(ny >> 1);
    p.kind[s] = p.xs[s] == 0u ? 0u : (p.xs[s] == 1u ? 1u : 2u);
    p.hb[s] = p.xs[s] == 0u ? 0u : static_cast<uint32_t>(31 - __builtin_clz(p.xs[s]));
    p.col[s] = j;
  }
}

template <bool SEED, int NS>
static int launch_coset_ns(const CosetParams& p, cudaStream_t st) {
  static std::atomic<uint64_t> configured{0};  // devices whose attribute is set
  const size_t smem = static_cast<size_t>(kCosetStages) * (8ull << p.tb);
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & 63);
  if (!(configured.load() & bit)) {
    // the largest dynamic request (2^13-amplitude stages)
    if (cudaFuncSetAttribute(k_coset<SEED, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(kCosetStages * (8ull << kCosetTileBits))) != cudaSuccess)
      return fail(TQK_CUDA_ERROR, "coset pass: cannot reserve %d bytes of shared memory",
                  static_cast<int>(kCosetStages * (8ull << kCosetTileBits)));
    configured.fetch_or(bit);
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t total = p.bsz * p.cosets;
  const int64_t grid = total < sms ? total : sms;
  k_coset<SEED, NS><<<static_cast<unsigned>(grid), kCosetThreads, smem, st>>>(p);
  return TQK_OK;
}

template <bool SEED>
static int launch_coset(const CosetParams& p, cudaStream_t st) {
  if (p.ns <= 1) return launch_coset_ns<SEED, 1>(p, st);
  if (p.ns <= 2) return launch_coset_ns<SEED, 2>(p, st);
  if (p.ns <= 4) return launch_coset_ns<SEED, 4>(p, st);
  return launch_coset_ns<SEED, 8>(p, st);
}

__global__ void __launch_bounds__(256) k_probs(const float2* state, float* out, int64_t total_half) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_half) return;
  const float4 v = ld4(state + t * 2);
  reinterpret_cast<float2*>(out)[t] = make_float2(v.x * v.x + v.y * v.y, v.z * v.z + v.w * v.w);
}

}  // namespace tqk

using namespace tqk;

extern "C" int tqk_probs(const void* state, int64_t bsz, int n, float* out, void* stream) {
  int rc = check_state(state, bsz, n, "tqk_probs");
  if (rc) return rc;
  if (out == nullptr || (reinterpret_cast<uintptr_t>(out) & 7u))
    return fail(TQK_BAD_POINTER, "tqk_probs: out must be non-null and 8-byte aligned");
  const int64_t total_half = (bsz << n) >> 1;
  const int threads = 256;
  k_probs<<<(unsigned)((total_half + threads - 1) / threads), threads, 0, as_stream(stream)>>>(
      static_cast<const float2*>(state), out, total_half);
  return launch_status("tqk_probs");
}

extern "C" int64_t tqk_pauli_expval_scratch_bytes(int64_t bsz, int n, int m) {
  // partials per pass, reused by every pass (the stream orders them): the per-X-mask pass
  // writes [bsz][blocks per row][8], a coset pass [bsz][2^(n - T)][8] (one per coset)
  (void)m;
  const int64_t nblk = reduce_blocks_per_row(bsz, n);
  const int64_t cosets = 1ll << (n - coset_tile_bits(n));
  const int64_t per_row = nblk > cosets ? nblk : cosets;
  return bsz * per_row * kMaxStringsPerPass * static_cast<int64_t>(sizeof(double));
}

extern "C" int tqk_pauli_expval(const void* state, int64_t bsz, int n, const uint64_t* xmask, const uint64_t* zmask,
                                int m, double* out, void* scratch, int64_t scratch_bytes, int* status,
                                void* stream) {
  const char* what = "tqk_pauli_expval";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (m <= 0) return TQK_OK;
  if (!xmask || !zmask || !out) return fail(TQK_BAD_POINTER, "%s: null mask/output pointer", what);
  if (status == nullptr) return fail(TQK_BAD_POINTER, "%s: null status word", what);
  if (scratch == nullptr || scratch_bytes < tqk_pauli_expval_scratch_bytes(bsz, n, m))
    return fail(TQK_SCRATCH_TOO_SMALL, "%s: scratch of %lld bytes needed", what,
                (long long)tqk_pauli_expval_scratch_bytes(bsz, n, m));
  const uint64_t lim = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
  for (int j = 0; j < m; ++j)
    if ((xmask[j] | zmask[j]) & ~lim) return fail(TQK_BAD_WIRES, "%s: string %d has bits beyond n_wires=%d", what, j, n);
  cudaStream_t st = as_stream(stream);
  const int64_t nblk = reduce_blocks_per_row(bsz, n);
  double* partial = static_cast<double*>(scratch);
  bool several = false;
  for (int j = 1; j < m && !several; ++j) several = xmask[j] != xmask[0];
  if (several) {
    // strings with different X-masks: coset passes (every partner read on chip)
    std::vector<CosetGroup> groups;
    coset_plan(n, xmask, m, groups);
    for (const CosetGroup& g : groups) {
      CosetParams p;
      coset_params(g, n, xmask, zmask, false, p);
      p.state = static_cast<const float2*>(state);
      p.out = nullptr;
      p.coef = nullptr;
      p.partial = partial;
      p.status = status;
      p.bsz = bsz;
      p.m = m;
      p.accumulate = 0;
      if ((rc = launch_coset<false>(p, st))) return rc;
      if ((rc = launch_status(what))) return rc;
      FinishCols cols;
      for (int s = 0; s < kMaxStringsPerPass; ++s) cols.c[s] = s < g.ns ? g.idx[s] : 0;
      k_expval_finish<<<(unsigned)bsz, kFinishThreads, 0, st>>>(partial, p.cosets, g.ns, kMaxStringsPerPass, cols,
                                                                m, out, bsz);
      if ((rc = launch_status(what))) return rc;
    }
    return TQK_OK;
  }
  std::vector<int> done(m, 0);
  for (int j0 = 0; j0 < m; ++j0) {
    if (done[j0]) continue;
    ExpvalParams p;
    p.state = static_cast<const float2*>(state);
    p.n = n;
    p.x = xmask[j0];
    p.ns = 0;
    p.m = kMaxStringsPerPass;
    p.partial = partial;
    FinishCols cols;
    for (int j = j0; j < m && p.ns < kMaxStringsPerPass; ++j) {
      if (done[j] || xmask[j] != p.x) continue;
      done[j] = 1;
      p.z[p.ns] = zmask[j];
      p.ny[p.ns] = __builtin_popcountll(xmask[j] & zmask[j]) & 3;
      cols.c[p.ns] = j;
      p.col[p.ns] = j;
      p.ns++;
    }
    for (int s = p.ns; s < kMaxStringsPerPass; ++s) {
      p.z[s] = 0;
      p.ny[s] = 0;
      p.col[s] = 0;
      cols.c[s] = 0;
    }
    dim3 grid((unsigned)nblk, (unsigned)bsz, 1);
    // block partials land at partial[(b*nblk + blk)*kMax + s]
    if (p.x == 0) {
      p.work = (1ll << n) >> 1;
    } else {
      p.hbit = 63 - __builtin_clzll(p.x);
      p.work = p.x == 1ull ? (1ll << n) >> 1 : (1ll << n) >> 2;
    }
    launch_expval(p, grid, st);
    if ((rc = launch_status(what))) return rc;
    k_expval_finish<<<(unsigned)bsz, kFinishThreads, 0, st>>>(partial, nblk, p.ns, kMaxStringsPerPass,
                                                                      cols, m, out, bsz);
    if ((rc = launch_status(what))) return rc;
  }
  return TQK_OK;
}

extern "C" int tqk_pauli_apply_sum(const void* state, int64_t bsz, int n, const uint64_t* xmask,
                                   const uint64_t* zmask, int m, const float* coef, void* out, int* status,
                                   void* stream) {
  const char* what = "tqk_pauli_apply_sum";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(out, bsz, n, what))) return rc;
  if (m <= 0) return fail(TQK_BAD_SHAPE, "%s: need at least one string", what);
  if (!xmask || !zmask || !coef) return fail(TQK_BAD_POINTER, "%s: null pointer", what);
  if (status == nullptr) return fail(TQK_BAD_POINTER, "%s: null status word", what);
  if (out == state) return fail(TQK_BAD_POINTER, "%s: out must not alias the state", what);
  const uint64_t lim = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
  for (int j = 0; j < m; ++j)
    if ((xmask[j] | zmask[j]) & ~lim) return fail(TQK_BAD_WIRES, "%s: string %d has bits beyond n_wires=%d", what, j, n);
  cudaStream_t st = as_stream(stream);
  std::vector<CosetGroup> groups;
  coset_plan(n, xmask, m, groups);
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    CosetParams p;
    coset_params(groups[gi], n, xmask, zmask, true, p);
    p.state = static_cast<const float2*>(state);
    p.out = static_cast<float2*>(out);
    p.coef = coef;
    p.partial = nullptr;
    p.status = status;
    p.bsz = bsz;
    p.m = m;
    p.accumulate = gi > 0;
    if ((rc = launch_coset<true>(p, st))) return rc;
    if ((rc = launch_status(what))) return rc;
  }
  return TQK_OK;
}

// ------------------------------------------------------------------ no-allocation variant
// tqk_pauli_expval_noalloc: the same computation as tqk_pauli_expval for callers that
// cannot hand the library a scratch buffer: a host program binding the C ABI from
// another language over FFI with only raw pointers to its own buffers and no device
// allocator to draw from, or a service that runs inside a fixed device-memory budget
// where the library must not call cudaMalloc.  Its block partials live in the
// file-scope array below instead of caller scratch, so the call allocates nothing,
// neither device memory nor host heap.  It always makes one pass per distinct X-mask.
//
// Limits: the partials must fit kNoAllocScratchBytes (1 MiB): bsz * blocks_per_row * 8
// doubles, where blocks_per_row = min(ceil(1216 / bsz), ceil(2^n / 1024)) -- so any
// bsz <= 16384 fits at n <= 10, and at every n up to bsz = 1216 (bsz * 1216 rounded up
// to a multiple of bsz stays below 16384 rows of partials); and at most
// kNoAllocMaxStrings strings per call.  Larger calls are rejected with
// TQK_SCRATCH_TOO_SMALL / TQK_BAD_SHAPE before any launch.
//
// Every call shares the one array per device and it keeps the last call's contents.
// Nothing in it needs to start at zero: every partial a call reads back was written
// earlier in the same call.  Calls whose kernels overlap on the GPU (different
// streams, or different host threads without ordering) race on the array.
//
// Set-up: the first call on each device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it, keyed by the CUDA
// context that was current; make that first call before any stream capture.  A call
// made in a different context of the device (after cudaDeviceReset, or under another
// context made current by the driver API) looks the address up again.  The cache is
// safe to fill from several host threads at once.
namespace tqk {

constexpr int64_t kNoAllocScratchBytes = 1 << 20;
constexpr int kNoAllocMaxStrings = 4096;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kNoAllocScratchBytes / sizeof(double)];

// Partials the pass loop below writes: one region of [bsz][blocks_per_row][8] doubles,
// reused by every pass (the stream orders them).
static int64_t noalloc_partial_bytes(int64_t bsz, int n) {
  return bsz * reduce_blocks_per_row(bsz, n) * kMaxStringsPerPass * static_cast<int64_t>(sizeof(double));
}

// Identity of the context current on this thread (0 when none is current or the driver
// entry points are unavailable, in which case the address is looked up on every call).
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);

static unsigned long long current_context_id() {
  static std::once_flag once;
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  if (get_current == nullptr || get_id == nullptr) return 0;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || ctx == nullptr) return 0;
  unsigned long long id = 0;
  if (get_id(ctx, &id) != 0) return 0;
  return id;
}

struct NoAllocSlot {
  std::atomic<unsigned long long> ctx{0};  // context the address was looked up in
  std::atomic<void*> ptr{nullptr};
};
static NoAllocSlot g_noalloc_slot[kNoAllocMaxDevices];
static std::mutex g_noalloc_mutex;

static int noalloc_scratch(void** out, const char* what) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(TQK_CUDA_ERROR, "%s: cudaGetDevice failed", what);
  if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(TQK_UNSUPPORTED, "%s: device %d beyond %d", what, dev,
                                                        kNoAllocMaxDevices);
  NoAllocSlot& slot = g_noalloc_slot[dev];
  const unsigned long long ctx = current_context_id();
  if (ctx != 0 && slot.ctx.load(std::memory_order_acquire) == ctx) {
    *out = slot.ptr.load(std::memory_order_acquire);
    return TQK_OK;
  }
  std::lock_guard<std::mutex> guard(g_noalloc_mutex);
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
  if (e != cudaSuccess || p == nullptr)
    return fail(TQK_CUDA_ERROR, "%s: cudaGetSymbolAddress failed: %s", what, cudaGetErrorString(e));
  // the lookup makes the device's primary context current if none was: key by the
  // context seen afterwards; the address is published before the key
  slot.ptr.store(p, std::memory_order_release);
  slot.ctx.store(current_context_id(), std::memory_order_release);
  *out = p;
  return TQK_OK;
}

}  // namespace tqk

extern "C" int64_t tqk_pauli_expval_noalloc_capacity(void) { return tqk::kNoAllocScratchBytes; }

extern "C" int tqk_pauli_expval_noalloc(const void* state, int64_t bsz, int n, const uint64_t* xmask,
                                        const uint64_t* zmask, int m, double* out, void* stream) {
  const char* what = "tqk_pauli_expval_noalloc";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (m <= 0) return TQK_OK;
  if (m > kNoAllocMaxStrings)
    return fail(TQK_BAD_SHAPE, "%s: %d strings exceed the limit of %d per call", what, m, kNoAllocMaxStrings);
  if (!xmask || !zmask || !out) return fail(TQK_BAD_POINTER, "%s: null mask/output pointer", what);
  const int64_t need = noalloc_partial_bytes(bsz, n);
  if (need > kNoAllocScratchBytes)
    return fail(TQK_SCRATCH_TOO_SMALL, "%s: needs %lld bytes of partials, the static array holds %lld (reduce bsz)",
                what, (long long)need, (long long)kNoAllocScratchBytes);
  const uint64_t lim = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
  for (int j = 0; j < m; ++j)
    if ((xmask[j] | zmask[j]) & ~lim) return fail(TQK_BAD_WIRES, "%s: string %d has bits beyond n_wires=%d", what, j, n);
  void* scratch = nullptr;
  if ((rc = noalloc_scratch(&scratch, what))) return rc;
  cudaStream_t st = as_stream(stream);
  const int64_t nblk = reduce_blocks_per_row(bsz, n);
  double* partial = static_cast<double*>(scratch);
  unsigned char done[kNoAllocMaxStrings];
  for (int j = 0; j < m; ++j) done[j] = 0;
  for (int j0 = 0; j0 < m; ++j0) {
    if (done[j0]) continue;
    ExpvalParams p;
    p.state = static_cast<const float2*>(state);
    p.n = n;
    p.x = xmask[j0];
    p.ns = 0;
    p.m = kMaxStringsPerPass;
    p.partial = partial;
    FinishCols cols;
    for (int j = j0; j < m && p.ns < kMaxStringsPerPass; ++j) {
      if (done[j] || xmask[j] != p.x) continue;
      done[j] = 1;
      p.z[p.ns] = zmask[j];
      p.ny[p.ns] = __builtin_popcountll(xmask[j] & zmask[j]) & 3;
      cols.c[p.ns] = j;
      p.col[p.ns] = j;
      p.ns++;
    }
    for (int s = p.ns; s < kMaxStringsPerPass; ++s) {
      p.z[s] = 0;
      p.ny[s] = 0;
      p.col[s] = 0;
      cols.c[s] = 0;
    }
    dim3 grid(static_cast<unsigned>(nblk), static_cast<unsigned>(bsz), 1);
    if (p.x == 0) {
      p.work = (1ll << n) >> 1;
    } else {
      p.hbit = 63 - __builtin_clzll(p.x);
      p.work = p.x == 1ull ? (1ll << n) >> 1 : (1ll << n) >> 2;
    }
    launch_expval(p, grid, st);
    if ((rc = launch_status(what))) return rc;
    k_expval_finish<<<static_cast<unsigned>(bsz), kFinishThreads, 0, st>>>(partial, nblk, p.ns,
                                                                               kMaxStringsPerPass, cols, m, out, bsz);
    if ((rc = launch_status(what))) return rc;
  }
  return TQK_OK;
}
