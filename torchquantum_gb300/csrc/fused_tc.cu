// fused_tc.cu -- fused k=6 block application on the 5th-generation tensor cores.
//
// A fused block is a dense 64x64 complex unitary U on 6 target bits.  For every
// column c (an assignment of the other n-6 bits) the 64 amplitudes x_c are replaced by
// U x_c.  As a real GEMM: D[i][n] = sum_K A[i][K] B[n][K] with
//   A[i][2j+p]  = (Re, Im)_p of amplitude (target pattern j, column c0+i)   (M = 128 columns)
//   B[2j'+p'][2j+p] = real embedding of U: [[Re U, -Im U], [Im U, Re U]]      (N = 128, K = 128)
//   D[i][2j'+p']  = (Re, Im)_p' of (U x_{c0+i})_j'.
// Precision: both operands are split into bf16 hi + lo parts and three products
// (hi.hi + hi.lo + lo.hi) accumulate in fp32 in tensor memory, which recovers ~16
// mantissa bits per product from bf16 inputs.
//
// Data path per persistent CTA (one per SM; 256 threads):
//   * B (U's hi/lo images, 64 KB, prepared once per block by k_tc_prep) stays in shared
//     memory; it is reloaded only when a per-row U changes with the batch row.
//   * A tiles are double-buffered (2 x 64 KB).  Thread lanes map to consecutive columns,
//     each thread loads 4 amplitudes (4 consecutive target patterns) per (row, quad),
//     splits them and writes one 16-byte chunk per image into the SWIZZLE_128B K-major
//     layout (conflict-free: 8 consecutive rows hit 8 distinct chunks).
//   * One thread issues 24 tcgen05.mma (3 products x 8 K-steps of 16) into one of two
//     128-column TMEM accumulators and commits to an mbarrier.
//   * The epilogue reads the accumulator with tcgen05.ld (lanes = columns) and writes
//     complex results straight to global memory, lanes on consecutive columns.
//   Loads of tile t+1 overlap the MMAs of tile t; the epilogue of tile t overlaps the
//   MMAs of tile t+1.
// Every mbarrier wait is bounded (clock-based); on a timeout the kernel records
// TQK_TIMEOUT in *status, stops issuing work, waits (bounded) for MMAs in flight,
// frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace tqk {
namespace tc {

constexpr int kThreads = 256;
constexpr int kTileCols = 128;          // M of the MMA
constexpr int kImgBytes = 32768;        // one 128 x 128 bf16 operand image
constexpr int kKBlockBytes = 16384;     // 128 rows x 128 B (64 bf16 of K)
constexpr uint32_t kTmemCols = 256;     // two 128-column fp32 accumulators
constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on an mbarrier phase; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > kWaitCycles) return false;
  }
  return true;
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// SWIZZLE_128B K-major shared-memory matrix descriptor (sm_100 format): start address
// >> 4 in bits [0,14), leading byte offset (unused for swizzled K-major) in [16,30),
// stride byte offset >> 4 = 1024 B between 8-row atoms in [32,46), version 1 at bit 46,
// layout type 2 (128-byte swizzle) in bits [61,64).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(1) << 16;
  d |= static_cast<uint64_t>(1024 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(2) << 61;
  return d;
}

// Instruction descriptor, kind::f16: D fp32 (bit 4), A and B bf16 (bits 7, 10),
// both K-major, N>>3 at bit 17, M>>4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of the 16-byte chunk holding K elements [8*chunk, 8*chunk+8) of row r in
// a 128-row SWIZZLE_128B K-major image (K = 128: chunk 0..15)
__device__ __forceinline__ uint32_t sw128_off(int r, int chunk) {
  const int kb = chunk >> 3, c = chunk & 7;
  return kb * kKBlockBytes + (r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4);
}

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void split4(const float2 (&a)[4], uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    __nv_bfloat162 hv = __floats2bfloat162_rn(a[r].x, a[r].y);
    const float2 hf = __bfloat1622float2(hv);
    h[r] = *reinterpret_cast<uint32_t*>(&hv);
    l[r] = pack_bf2(a[r].x - hf.x, a[r].y - hf.y);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void issue_mma(uint32_t d_tmem, uint32_t a_s, uint32_t b_s) {
  constexpr uint32_t idesc = idesc_bf16(128, 128);
  // (A image, B image): hi.hi, hi.lo, lo.hi
  const uint32_t ao[3] = {0u, 0u, static_cast<uint32_t>(kImgBytes)};
  const uint32_t bo[3] = {0u, static_cast<uint32_t>(kImgBytes), 0u};
#pragma unroll
  for (int prod = 0; prod < 3; ++prod) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const uint32_t koff = (s >> 2) * kKBlockBytes + (s & 3) * 32;
      mma_bf16(d_tmem, desc_sw128(a_s + ao[prod] + koff), desc_sw128(b_s + bo[prod] + koff), idesc,
               (prod > 0 || s > 0) ? 1u : 0u);
    }
  }
}

// MN-major SWIZZLE_128B descriptor over a [column][128 (j,p)] tile image: the two
// 64-element (j,p) halves are 16 KB apart (LBO), 8-column groups 1024 B apart (SBO).
__device__ __forceinline__ uint64_t desc_sw128_mn(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(kKBlockBytes >> 4) << 16;
  d |= static_cast<uint64_t>(1024 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(2) << 61;
  return d;
}

// Cross term of the adjoint tile: D_M[m][n] += sum over the tile's 64 columns of
// lam~[m] psi~[n]; lam rows are tile rows 64..127, psi rows 0..63 (K = column, MN-major).
__device__ __forceinline__ void issue_cross(uint32_t d_tmem, uint32_t a_s, bool first) {
  constexpr uint32_t idesc = idesc_bf16(128, 128) | (1u << 15) | (1u << 16);
  const uint32_t lam_s = a_s + 64 * 128, psi_s = a_s;
  const uint32_t ao[3] = {0u, 0u, static_cast<uint32_t>(kImgBytes)};
  const uint32_t bo[3] = {0u, static_cast<uint32_t>(kImgBytes), 0u};
#pragma unroll
  for (int prod = 0; prod < 3; ++prod) {
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const uint32_t koff = s * 2048;
      mma_bf16(d_tmem, desc_sw128_mn(lam_s + ao[prod] + koff), desc_sw128_mn(psi_s + bo[prod] + koff), idesc,
               (first && prod == 0 && s == 0) ? 0u : 1u);
    }
  }
}

__device__ __forceinline__ void cp_async16(uint32_t saddr, const void* gptr) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr), "l"(gptr) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Stage layout: per state a region of 4096 / 2048 16-byte chunks (compressed address
// order, chunk c holds amplitudes 2c, 2c+1); chunk c is stored at c ^ ((c >> 5) & 31)
// so that column-strided reads of the conversion spread over the banks.
__device__ __forceinline__ uint32_t stage_chunk(uint32_t c) { return c ^ ((c >> 5) & 31u); }

// Tile geometry.  APPLY: 128 columns of one state.  ADJ: 64 columns of psi (rows 0..63)
// and the same 64 columns of lam (rows 64..127).
template <bool ADJ>
struct TileGeom {
  static constexpr int kCols = ADJ ? 64 : 128;       // columns per state
  static constexpr int kBits = ADJ ? 12 : 13;        // compressed bits per state
  static constexpr int kChunks = 1 << (kBits - 1);   // 16-byte chunks per state
  static constexpr int kStateBytes = kChunks * 16;   // 32 KB / 64 KB
};

struct TcParams {
  float2* psi;               // state (APPLY) / psi (ADJ)
  float2* lam;               // ADJ only
  int n;
  BitInsert ins;             // the 6 target bits
  uint64_t off[64];          // amplitude offset of target pattern j (j bit 5 = tb[0])
  int sbits[13];             // tile bits (targets + lowest column bits), ascending
  int col_pos[7];            // position in the compressed index of column bit b
  int tgt_pos[6];            // position in the compressed index of target bit tb[jb]
  const uint8_t* uimg;       // [u_batch][2 images][32 KB] (U for APPLY, U^H for ADJ)
  int64_t u_batch;
  int64_t tiles_per_row;
  int64_t tiles;
  double* mr_out;            // ADJ: [u_batch][128][128] cross term, or null
  int* status;
};

__device__ __forceinline__ uint64_t scatter_bits(uint32_t u, const int* sbits, int nb) {
  uint64_t a = 0;
  for (int b = 0; b < nb; ++b)
    if ((u >> b) & 1u) a |= 1ull << sbits[b];
  return a;
}

struct TcShared {
  uint64_t off[64];          // target pattern offsets
  uint32_t uj[64];           // compressed-index contribution of target pattern j
  uint64_t schunk[16];       // scatter of 512*s (chunk offsets of the cp.async loop)
};

template <bool ADJ>
__device__ __forceinline__ void issue_loads(const TcParams& p, int64_t t, uint32_t stage_s, uint64_t a_tid,
                                            const TcShared& sh) {
  using G = TileGeom<ADJ>;
  const int64_t b = t / p.tiles_per_row;
  const int64_t c0 = (t % p.tiles_per_row) * G::kCols;
  const uint64_t tbase = insert_zero_bits(static_cast<uint64_t>(c0), p.ins) + (static_cast<uint64_t>(b) << p.n);
#pragma unroll
  for (int s = 0; s < 16; ++s) {
    const int st = ADJ ? (s >> 3) : 0;
    const int sl = ADJ ? (s & 7) : s;
    const float2* base = st ? p.lam : p.psi;
    const uint32_t c = static_cast<uint32_t>(threadIdx.x + kThreads * sl);
    const float2* g = base + tbase + a_tid + sh.schunk[sl];
    cp_async16(stage_s + st * G::kStateBytes + stage_chunk(c) * 16, g);
  }
  cp_async_commit();
}

// stage (fp32, compressed order) -> A images (bf16 hi/lo, SWIZZLE_128B K-major)
template <bool ADJ>
__device__ __forceinline__ void convert(const uint8_t* stage, uint8_t* abuf, uint32_t ucol, int row,
                                        const TcShared& sh) {
  using G = TileGeom<ADJ>;
  const int st = ADJ ? (row >> 6) : 0;
  const float2* sp = reinterpret_cast<const float2*>(stage + st * G::kStateBytes);
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int q = (threadIdx.x >> 7) + 2 * s;
    float2 a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint32_t u = ucol | sh.uj[4 * q + r];
      a[r] = sp[stage_chunk(u >> 1) * 2 + (u & 1u)];
    }
    uint4 hi, lo;
    split4(a, hi, lo);
    const uint32_t o = sw128_off(row, q);
    *reinterpret_cast<uint4*>(abuf + o) = hi;
    *reinterpret_cast<uint4*>(abuf + kImgBytes + o) = lo;
  }
}

template <bool ADJ>
__device__ __forceinline__ void epilogue(const TcParams& p, int64_t t, uint32_t d_tmem, uint64_t ibase,
                                         const TcShared& sh) {
  using G = TileGeom<ADJ>;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = warp & 3, half = warp >> 2;
  const int64_t b = t / p.tiles_per_row;
  const int64_t c0 = (t % p.tiles_per_row) * G::kCols;
  const int row = sub * 32 + lane;
  const int st = ADJ ? (row >> 6) : 0;
  float2* base = (st ? p.lam : p.psi) + (b << p.n) + insert_zero_bits(static_cast<uint64_t>(c0), p.ins) + ibase;
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const int col = half * 64 + part * 32;
    uint32_t r[32];
    tmem_ld32(d_tmem + (static_cast<uint32_t>(sub * 32) << 16) + col, r);
    tmem_wait_ld();
#pragma unroll
    for (int v = 0; v < 16; ++v) {
      const int j = (col >> 1) + v;
      base[sh.off[j]] = make_float2(__uint_as_float(r[2 * v]), __uint_as_float(r[2 * v + 1]));
    }
  }
}

__device__ __forceinline__ void flush_cross(double* dst, uint32_t d_tmem) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = warp & 3, half = warp >> 2;
  const int m = sub * 32 + lane;
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const int col = half * 64 + part * 32;
    uint32_t r[32];
    tmem_ld32(d_tmem + (static_cast<uint32_t>(sub * 32) << 16) + col, r);
    tmem_wait_ld();
#pragma unroll
    for (int v = 0; v < 32; ++v) atomicAdd(dst + m * 128 + col + v, static_cast<double>(__uint_as_float(r[v])));
  }
}

__device__ __forceinline__ void load_u(const TcParams& p, int64_t b, uint8_t* bimg) {
  const uint4* src = reinterpret_cast<const uint4*>(p.uimg + (p.u_batch > 1 ? b : 0) * 2 * kImgBytes);
  uint4* dst = reinterpret_cast<uint4*>(bimg);
  for (int i = threadIdx.x; i < 2 * kImgBytes / 16; i += kThreads) dst[i] = src[i];
}

// One kernel for the forward block application (ADJ = false) and the adjoint step
// (ADJ = true).  Shared memory: U (or U^H) image 64 KB, A image 64 KB, raw stage 64 KB.
// TMEM: two 128-column accumulators for the block product (+ one for the cross term).
// Per iteration t: the loads of tile t+2 go out (cp.async) right after tile t+1 is
// converted and its MMAs issued, so one full iteration hides their latency; the
// epilogue of tile t overlaps the MMAs of tile t+1.
template <bool ADJ>
__global__ void __launch_bounds__(kThreads, 1) k_tc(const TcParams p) {
  using G = TileGeom<ADJ>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* bimg = smem;                          // 64 KB
  uint8_t* abuf = smem + 2 * kImgBytes;          // 64 KB
  uint8_t* stage = abuf + 2 * kImgBytes;         // 64 KB
  TcShared* sh = reinterpret_cast<TcShared*>(stage + 2 * kImgBytes);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sh + 1);  // 2 mbarriers
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);

  const int64_t per = (p.tiles + gridDim.x - 1) / gridDim.x;
  const int64_t t_begin = blockIdx.x * per;
  const int64_t t_end = min(p.tiles, t_begin + per);
  if (t_begin >= t_end) return;  // uniform for the block

  const uint32_t ncols_tmem = ADJ ? 512u : 256u;
  if (threadIdx.x < 64) {
    const int j = threadIdx.x;
    sh->off[j] = p.off[j];
    uint32_t u = 0;
    for (int jb = 0; jb < 6; ++jb)
      if ((j >> (5 - jb)) & 1) u |= 1u << p.tgt_pos[jb];
    sh->uj[j] = u;
  }
  if (threadIdx.x < 16) sh->schunk[threadIdx.x] = scatter_bits(512u * threadIdx.x, p.sbits, G::kBits);
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(ncols_tmem)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  // per-thread constants
  const uint64_t a_tid = scatter_bits(2u * threadIdx.x, p.sbits, G::kBits);
  const int crow = threadIdx.x & 127;                 // conversion row
  const int ccol = ADJ ? (crow & 63) : crow;          // its column within the state
  uint32_t ucol = 0;
  for (int bb = 0; bb < (ADJ ? 6 : 7); ++bb)
    if ((ccol >> bb) & 1) ucol |= 1u << p.col_pos[bb];
  const int erow = (threadIdx.x >> 5 & 3) * 32 + (threadIdx.x & 31);  // epilogue row
  const uint64_t ibase = insert_zero_bits(static_cast<uint64_t>(ADJ ? (erow & 63) : erow), p.ins);

  int64_t cur_b = t_begin / p.tiles_per_row;
  load_u(p, cur_b, bimg);
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t d_m = tmem + 256;
  const uint32_t b_s = smem_u32(bimg), a_s = smem_u32(abuf), stage_s = smem_u32(stage);
  const bool want_cross = ADJ && p.mr_out != nullptr;
  bool first_cross = true;

  // prologue: tile t_begin -> A -> D[0]; loads of t_begin+1 in flight
  issue_loads<ADJ>(p, t_begin, stage_s, a_tid, *sh);
  cp_async_wait_all();
  __syncthreads();
  convert<ADJ>(stage, abuf, ucol, crow, *sh);
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    issue_mma(tmem, a_s, b_s);
    if (want_cross) issue_cross(d_m, a_s, true);
    mma_commit(&bars[0]);
  }
  if (want_cross) first_cross = false;
  // stage is free again once every thread's conversion is done (barrier above)
  if (t_begin + 1 < t_end) issue_loads<ADJ>(p, t_begin + 1, stage_s, a_tid, *sh);
  uint32_t phase[2] = {0u, 0u};
  int inflight[2] = {1, 0};
  int aborted = 0;

  for (int64_t t = t_begin; t < t_end; ++t) {
    const int buf = static_cast<int>((t - t_begin) & 1);
    const bool more = t + 1 < t_end;
    if (more) cp_async_wait_all();
    int timed_out = 0;
    const bool waiting = !aborted && inflight[buf];
    if (waiting) timed_out = mbar_wait(&bars[buf], phase[buf]) ? 0 : 1;
    const int any_timeout = __syncthreads_or(timed_out);
    if (waiting && !any_timeout) {
      phase[buf] ^= 1u;
      inflight[buf] = 0;
    }
    if (any_timeout) {
      if (threadIdx.x == 0) atomicExch(p.status, TQK_TIMEOUT);
      aborted = 1;
    }
    tc_fence_after();
    if (more && !aborted) {
      const int64_t nb = (t + 1) / p.tiles_per_row;
      if (nb != cur_b) {  // a new batch row: flush its cross term, reload a per-row U
        if (want_cross) {
          flush_cross(p.mr_out + (p.u_batch > 1 ? cur_b : 0) * 128 * 128, d_m);
          first_cross = true;
        }
        if (p.u_batch > 1) load_u(p, nb, bimg);
        cur_b = nb;
      }
      convert<ADJ>(stage, abuf, ucol, crow, *sh);
      fence_proxy_async();
      tc_fence_before();
      __syncthreads();
      if (threadIdx.x == 0) {
        tc_fence_after();
        issue_mma(tmem + static_cast<uint32_t>((buf ^ 1) * 128), a_s, b_s);
        if (want_cross) issue_cross(d_m, a_s, first_cross);
        mma_commit(&bars[buf ^ 1]);
      }
      first_cross = false;
      inflight[buf ^ 1] = 1;
      if (t + 2 < t_end) issue_loads<ADJ>(p, t + 2, stage_s, a_tid, *sh);
    }
    if (!aborted) epilogue<ADJ>(p, t, tmem + static_cast<uint32_t>(buf * 128), ibase, *sh);
    tc_fence_before();
    __syncthreads();
  }
  cp_async_wait_all();
  for (int bsel = 0; bsel < 2; ++bsel)
    if (inflight[bsel]) mbar_wait(&bars[bsel], phase[bsel]);
  tc_fence_after();
  if (want_cross && !aborted && !first_cross) flush_cross(p.mr_out + (p.u_batch > 1 ? cur_b : 0) * 128 * 128, d_m);
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem) : "memory");
  }
}

// U (complex128 [u_batch][64][64], row-major) -> hi/lo bf16 images of the real
// embedding in the SWIZZLE_128B K-major layout expected by k_tc_apply (B operand:
// row n = 2j'+p', K = 2j+p).  One thread per (batch, row n, 16-byte chunk).
__global__ void k_tc_prep(const double2* u, int64_t u_batch, uint8_t* img) {
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= u_batch * 128 * 16) return;
  const int64_t b = idx / (128 * 16);
  const int n = static_cast<int>((idx / 16) % 128);
  const int chunk = static_cast<int>(idx % 16);
  const int jo = n >> 1, po = n & 1;
  const double2* ub = u + b * 64 * 64;
  float hv[8], lv[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int kk = chunk * 8 + e;
    const int j = kk >> 1, pi = kk & 1;
    const double2 z = ub[jo * 64 + j];
    // [[Re, -Im], [Im, Re]]
    double v;
    if (po == 0) v = (pi == 0) ? z.x : -z.y;
    else v = (pi == 0) ? z.y : z.x;
    const __nv_bfloat16 h = __double2bfloat16(v);
    hv[e] = __bfloat162float(h);
    lv[e] = static_cast<float>(v - static_cast<double>(hv[e]));
  }
  uint4 hi = make_uint4(pack_bf2(hv[0], hv[1]), pack_bf2(hv[2], hv[3]), pack_bf2(hv[4], hv[5]), pack_bf2(hv[6], hv[7]));
  uint4 lo = make_uint4(pack_bf2(lv[0], lv[1]), pack_bf2(lv[2], lv[3]), pack_bf2(lv[4], lv[5]), pack_bf2(lv[6], lv[7]));
  uint8_t* base = img + b * 2 * kImgBytes;
  const uint32_t o = sw128_off(n, chunk);
  *reinterpret_cast<uint4*>(base + o) = hi;
  *reinterpret_cast<uint4*>(base + kImgBytes + o) = lo;
}

}  // namespace tc
}  // namespace tqk

using namespace tqk;

extern "C" int64_t tqk_fused_image_bytes(int64_t u_batch) { return u_batch * 2 * tc::kImgBytes; }

extern "C" int tqk_fused_prepare(const void* u, int64_t u_batch, void* image, void* stream) {
  if (!u || !image) return fail(TQK_BAD_POINTER, "tqk_fused_prepare: null pointer");
  if ((reinterpret_cast<uintptr_t>(image) & 15u) != 0)
    return fail(TQK_BAD_POINTER, "tqk_fused_prepare: image must be 16-byte aligned");
  if (u_batch < 1) return fail(TQK_BAD_SHAPE, "tqk_fused_prepare: u_batch must be >= 1");
  const int64_t work = u_batch * 128 * 16;
  tc::k_tc_prep<<<static_cast<unsigned>((work + 255) / 256), 256, 0, as_stream(stream)>>>(
      static_cast<const double2*>(u), u_batch, static_cast<uint8_t*>(image));
  return launch_status("tqk_fused_prepare");
}

namespace {

int tc_setup(tqk::tc::TcParams& p, int64_t bsz, int n, const int32_t* wires, bool adj, const char* what) {
  using namespace tqk;
  int tb[6];
  uint64_t used = 0;
  int rc = wires_to_bits(n, wires, 6, tb, &used, what);
  if (rc) return rc;
  p.n = n;
  p.ins = make_insert(used);
  for (int j = 0; j < 64; ++j) {
    uint64_t o = 0;
    for (int jb = 0; jb < 6; ++jb)
      if ((j >> (5 - jb)) & 1) o |= 1ull << tb[jb];
    p.off[j] = o;
  }
  // tile bits: the 6 targets + the lowest 7 (apply) / 6 (adjoint) column bits
  const int ncolbits = adj ? 6 : 7;
  int colbits[7];
  int nc = 0;
  for (int q = 0; q < n && nc < ncolbits; ++q)
    if (!(used & (1ull << q))) colbits[nc++] = q;
  uint64_t smask = used;
  for (int i = 0; i < nc; ++i) smask |= 1ull << colbits[i];
  int ns = 0;
  for (int q = 0; q < 64 && ns < 13; ++q)
    if (smask & (1ull << q)) p.sbits[ns++] = q;
  for (int i = ns; i < 13; ++i) p.sbits[i] = 0;
  auto pos_of = [&](int bit) {
    for (int i = 0; i < ns; ++i)
      if (p.sbits[i] == bit) return i;
    return -1;
  };
  for (int i = 0; i < 7; ++i) p.col_pos[i] = i < nc ? pos_of(colbits[i]) : 0;
  for (int jb = 0; jb < 6; ++jb) p.tgt_pos[jb] = pos_of(tb[jb]);
  const int cols = adj ? 64 : 128;
  p.tiles_per_row = (1ll << (n - 6)) / cols;
  p.tiles = p.tiles_per_row * bsz;
  return TQK_OK;
}

int tc_launch(const tqk::tc::TcParams& p, bool adj, void* stream, const char* what) {
  using namespace tqk;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 1024 + 6 * tc::kImgBytes + sizeof(tc::TcShared) + 2 * 8 + 16;
  static int attr_dev[2] = {-1, -1};
  if (attr_dev[adj] != dev) {
    if (adj) cudaFuncSetAttribute(tc::k_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    else cudaFuncSetAttribute(tc::k_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    attr_dev[adj] = dev;
  }
  const int64_t grid = p.tiles < sms ? p.tiles : sms;
  if (adj) tc::k_tc<true><<<static_cast<unsigned>(grid), tc::kThreads, smem, as_stream(stream)>>>(p);
  else tc::k_tc<false><<<static_cast<unsigned>(grid), tc::kThreads, smem, as_stream(stream)>>>(p);
  return launch_status(what);
}

}  // namespace

extern "C" int tqk_fused_adjoint(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires,
                                 const void* image_h, int64_t u_batch, double* mr_out, int* status, void* stream) {
  const char* what = "tqk_fused_adjoint";
  int rc = check_state(psi, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(lam, bsz, n, what))) return rc;
  if ((rc = check_batch(u_batch, bsz, what))) return rc;
  if (!image_h || !status) return fail(TQK_BAD_POINTER, "%s: null image/status", what);
  if (n < 13) return fail(TQK_UNSUPPORTED, "%s: needs n_wires >= 13 (got %d)", what, n);
  tc::TcParams p;
  p.psi = static_cast<float2*>(psi);
  p.lam = static_cast<float2*>(lam);
  p.uimg = static_cast<const uint8_t*>(image_h);
  p.u_batch = u_batch;
  p.mr_out = mr_out;
  p.status = status;
  if ((rc = tc_setup(p, bsz, n, wires, true, what))) return rc;
  return tc_launch(p, true, stream, what);
}

extern "C" int tqk_fused_apply(void* state, int64_t bsz, int n, const int32_t* wires, const void* image,
                               int64_t u_batch, int* status, void* stream) {
  const char* what = "tqk_fused_apply";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_batch(u_batch, bsz, what))) return rc;
  if (!image || !status) return fail(TQK_BAD_POINTER, "%s: null image/status", what);
  if ((reinterpret_cast<uintptr_t>(image) & 15u) != 0) return fail(TQK_BAD_POINTER, "%s: image alignment", what);
  if (n < 13) return fail(TQK_UNSUPPORTED, "%s: needs n_wires >= 13 (got %d)", what, n);
  tc::TcParams p;
  p.psi = static_cast<float2*>(state);
  p.lam = nullptr;
  p.uimg = static_cast<const uint8_t*>(image);
  p.u_batch = u_batch;
  p.mr_out = nullptr;
  p.status = status;
  if ((rc = tc_setup(p, bsz, n, wires, false, what))) return rc;
  return tc_launch(p, false, stream, what);
}
