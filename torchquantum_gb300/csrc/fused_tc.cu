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

struct ApplyParams {
  float2* state;
  int n;
  int64_t bsz;
  BitInsert ins;             // the 6 target bits
  uint64_t off[64];          // amplitude offset of target pattern j (j bit 5 = tb[0])
  const uint8_t* uimg;       // [u_batch][2 images][32 KB]
  int64_t u_batch;
  int64_t tiles_per_row;
  int64_t tiles;
  int* status;
};

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

// Load tile t (128 columns x 64 patterns) from global, split, write A images at abuf.
__device__ __forceinline__ void produce(const ApplyParams& p, int64_t t, uint8_t* abuf, const uint64_t* offs) {
  const int64_t b = t / p.tiles_per_row;
  const int64_t c0 = (t % p.tiles_per_row) * kTileCols;
  const float2* row = p.state + (b << p.n);
  // 2048 (column, quad) pairs; lanes on consecutive columns
#pragma unroll
  for (int e = threadIdx.x; e < kTileCols * 16; e += kThreads) {
    const int i = e & (kTileCols - 1);
    const int q = e >> 7;
    const uint64_t base = insert_zero_bits(static_cast<uint64_t>(c0 + i), p.ins);
    float2 a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = row[base + offs[4 * q + r]];
    uint4 hi, lo;
    split4(a, hi, lo);
    const uint32_t o = sw128_off(i, q);
    *reinterpret_cast<uint4*>(abuf + o) = hi;
    *reinterpret_cast<uint4*>(abuf + kImgBytes + o) = lo;
  }
}

__device__ __forceinline__ void load_u(const ApplyParams& p, int64_t b, uint8_t* bimg) {
  const uint4* src = reinterpret_cast<const uint4*>(p.uimg + (p.u_batch > 1 ? b : 0) * 2 * kImgBytes);
  uint4* dst = reinterpret_cast<uint4*>(bimg);
  for (int i = threadIdx.x; i < 2 * kImgBytes / 16; i += kThreads) dst[i] = src[i];
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

__device__ __forceinline__ void epilogue(const ApplyParams& p, int64_t t, uint32_t d_tmem, const uint64_t* offs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = warp & 3, half = warp >> 2;
  const int64_t b = t / p.tiles_per_row;
  const int64_t c0 = (t % p.tiles_per_row) * kTileCols;
  const int i = sub * 32 + lane;
  float2* row = p.state + (b << p.n);
  const uint64_t base = insert_zero_bits(static_cast<uint64_t>(c0 + i), p.ins);
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const int col = half * 64 + part * 32;
    uint32_t r[32];
    tmem_ld32(d_tmem + (static_cast<uint32_t>(sub * 32) << 16) + col, r);
    tmem_wait_ld();
#pragma unroll
    for (int v = 0; v < 16; ++v) {
      const int j = (col >> 1) + v;
      row[base + offs[j]] = make_float2(__uint_as_float(r[2 * v]), __uint_as_float(r[2 * v + 1]));
    }
  }
}

__global__ void __launch_bounds__(kThreads, 1) k_tc_apply(const ApplyParams p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* bimg = smem;                         // 64 KB: U hi, U lo
  uint8_t* abuf0 = smem + 2 * kImgBytes;        // 64 KB each: tile hi, tile lo
  uint8_t* abuf1 = abuf0 + 2 * kImgBytes;
  uint64_t* offs = reinterpret_cast<uint64_t*>(abuf1 + 2 * kImgBytes);  // 64 entries
  uint64_t* bars = offs + 64;                   // 2 mbarriers
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);

  const int64_t per = (p.tiles + gridDim.x - 1) / gridDim.x;
  const int64_t t_begin = blockIdx.x * per;
  const int64_t t_end = min(p.tiles, t_begin + per);
  if (t_begin >= t_end) return;  // uniform for the block

  if (threadIdx.x < 64) offs[threadIdx.x] = p.off[threadIdx.x];
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {  // warp 0 owns the tensor memory
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  int64_t cur_b = t_begin / p.tiles_per_row;
  load_u(p, cur_b, bimg);
  __syncthreads();  // offsets, barriers, tmem slot visible
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t b_s = smem_u32(bimg);
  uint8_t* abufs[2] = {abuf0, abuf1};
  uint32_t phase[2] = {0u, 0u};
  int aborted = 0;

  // prologue: tile t_begin -> A[0] -> D[0]
  produce(p, t_begin, abufs[0], offs);
  fence_proxy_async();
  __syncthreads();
  if (threadIdx.x == 0) {
    tc_fence_after();
    issue_mma(tmem, smem_u32(abufs[0]), b_s);
    mma_commit(&bars[0]);
  }
  int inflight[2] = {1, 0};

  for (int64_t t = t_begin; t < t_end; ++t) {
    const int buf = static_cast<int>((t - t_begin) & 1);
    const bool more = t + 1 < t_end;
    if (more && !aborted) produce(p, t + 1, abufs[buf ^ 1], offs);
    // MMA(t) complete?  (a wait that gives up leaves the MMA marked in flight so the
    // drain below waits for it again, bounded, before the tensor memory is freed)
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
      if (p.u_batch > 1 && nb != cur_b) {  // per-row U: all MMAs have completed here
        load_u(p, nb, bimg);
        cur_b = nb;
      }
      fence_proxy_async();
      tc_fence_before();
      __syncthreads();
      if (threadIdx.x == 0) {
        tc_fence_after();
        issue_mma(tmem + static_cast<uint32_t>((buf ^ 1) * 128), smem_u32(abufs[buf ^ 1]), b_s);
        mma_commit(&bars[buf ^ 1]);
      }
      inflight[buf ^ 1] = 1;
    }
    if (!aborted) epilogue(p, t, tmem + static_cast<uint32_t>(buf * 128), offs);
    tc_fence_before();
    __syncthreads();
  }
  // drain: bounded wait for anything still in flight, then free tensor memory
  for (int bsel = 0; bsel < 2; ++bsel)
    if (inflight[bsel]) mbar_wait(&bars[bsel], phase[bsel]);
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// ------------------------------------------------------------------ adjoint step
// One reverse step of the adjoint method for a fused block, per tile of 128 columns:
//   psi <- U^H psi, lam <- U^H lam   (two K-major GEMMs against the image of U^H)
//   Mr += Lam~^T Psi~                 (the cross term, reduced over the tile's columns)
// where Lam~ / Psi~ are the tiles' real embeddings [column][2j+p].  The cross GEMM
// reads the same swizzled tiles as MN-major operands (M = N = 128 = (j, p), K = the
// tile's columns, 16 per instruction: start address + 2048 B per K step, LBO = 16 KB
// between the two 64-element (j, p) halves, SBO = 1024 B between 8-column groups).
// Mr is flushed to float64 (atomicAdd into mr_out[row or 0][128][128]) at the end and
// whenever a per-row U changes with the batch row; the host forms
//   M[j][j'] = sum lam[j] conj(psi[j'])  from Mr, and the cotangent of U as M U.
// Single-buffered: shared memory holds U^H (64 KB) and the psi and lam tiles (64 KB each).
struct AdjParams {
  float2* psi;
  float2* lam;
  int n;
  BitInsert ins;
  uint64_t off[64];
  const uint8_t* uimg;   // image of U^H
  int64_t u_batch;
  int64_t tiles_per_row;
  int64_t tiles;
  double* mr_out;        // [u_batch][128][128] or null (no gradient)
  int* status;
};

__device__ __forceinline__ void produce_rows(const float2* row, int64_t c0, const BitInsert& ins, uint8_t* abuf,
                                             const uint64_t* offs) {
#pragma unroll
  for (int e = threadIdx.x; e < kTileCols * 16; e += kThreads) {
    const int i = e & (kTileCols - 1);
    const int q = e >> 7;
    const uint64_t base = insert_zero_bits(static_cast<uint64_t>(c0 + i), ins);
    float2 a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = row[base + offs[4 * q + r]];
    uint4 hi, lo;
    split4(a, hi, lo);
    const uint32_t o = sw128_off(i, q);
    *reinterpret_cast<uint4*>(abuf + o) = hi;
    *reinterpret_cast<uint4*>(abuf + kImgBytes + o) = lo;
  }
}

__device__ __forceinline__ void epilogue_rows(float2* row, int64_t c0, const BitInsert& ins, uint32_t d_tmem,
                                              const uint64_t* offs) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = warp & 3, half = warp >> 2;
  const int i = sub * 32 + lane;
  const uint64_t base = insert_zero_bits(static_cast<uint64_t>(c0 + i), ins);
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const int col = half * 64 + part * 32;
    uint32_t r[32];
    tmem_ld32(d_tmem + (static_cast<uint32_t>(sub * 32) << 16) + col, r);
    tmem_wait_ld();
#pragma unroll
    for (int v = 0; v < 16; ++v) {
      const int j = (col >> 1) + v;
      row[base + offs[j]] = make_float2(__uint_as_float(r[2 * v]), __uint_as_float(r[2 * v + 1]));
    }
  }
}

// MN-major SWIZZLE_128B descriptor over a [column][128 (j,p)] tile image.
__device__ __forceinline__ uint64_t desc_sw128_mn(uint32_t saddr) {
  uint64_t d = 0;
  d |= static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(kKBlockBytes >> 4) << 16;
  d |= static_cast<uint64_t>(1024 >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  d |= static_cast<uint64_t>(2) << 61;
  return d;
}

__device__ __forceinline__ void issue_cross(uint32_t d_tmem, uint32_t lam_s, uint32_t psi_s, bool first) {
  // kind::f16, D fp32, bf16 A/B, A and B MN-major (bits 15, 16), M = N = 128
  constexpr uint32_t idesc = idesc_bf16(128, 128) | (1u << 15) | (1u << 16);
  const uint32_t ao[3] = {0u, 0u, static_cast<uint32_t>(kImgBytes)};
  const uint32_t bo[3] = {0u, static_cast<uint32_t>(kImgBytes), 0u};
#pragma unroll
  for (int prod = 0; prod < 3; ++prod) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const uint32_t koff = s * 2048;
      mma_bf16(d_tmem, desc_sw128_mn(lam_s + ao[prod] + koff), desc_sw128_mn(psi_s + bo[prod] + koff), idesc,
               (first && prod == 0 && s == 0) ? 0u : 1u);
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

__global__ void __launch_bounds__(kThreads, 1) k_tc_adjoint(const AdjParams p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* bimg = smem;                        // U^H hi, lo
  uint8_t* apsi = smem + 2 * kImgBytes;        // psi tile hi, lo
  uint8_t* alam = apsi + 2 * kImgBytes;        // lam tile hi, lo
  uint64_t* offs = reinterpret_cast<uint64_t*>(alam + 2 * kImgBytes);
  uint64_t* bar = offs + 64;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);

  const int64_t per = (p.tiles + gridDim.x - 1) / gridDim.x;
  const int64_t t_begin = blockIdx.x * per;
  const int64_t t_end = min(p.tiles, t_begin + per);
  if (t_begin >= t_end) return;

  if (threadIdx.x < 64) offs[threadIdx.x] = p.off[threadIdx.x];
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512u)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  int64_t cur_b = t_begin / p.tiles_per_row;
  {
    const uint4* src = reinterpret_cast<const uint4*>(p.uimg + (p.u_batch > 1 ? cur_b : 0) * 2 * kImgBytes);
    uint4* dst = reinterpret_cast<uint4*>(bimg);
    for (int i = threadIdx.x; i < 2 * kImgBytes / 16; i += kThreads) dst[i] = src[i];
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t d_psi = tmem, d_lam = tmem + 128, d_m = tmem + 256;
  const uint32_t b_s = smem_u32(bimg), psi_s = smem_u32(apsi), lam_s = smem_u32(alam);
  uint32_t phase = 0;
  int aborted = 0, inflight = 0;
  bool first_cross = true;

  for (int64_t t = t_begin; t < t_end && !aborted; ++t) {
    const int64_t b = t / p.tiles_per_row;
    const int64_t c0 = (t % p.tiles_per_row) * kTileCols;
    if (p.u_batch > 1 && b != cur_b) {
      // per-row U: flush the cross term of the previous row, reload U^H
      if (p.mr_out && !first_cross) {
        tc_fence_after();
        flush_cross(p.mr_out + cur_b * 128 * 128, d_m);
        first_cross = true;
      }
      const uint4* src = reinterpret_cast<const uint4*>(p.uimg + b * 2 * kImgBytes);
      uint4* dst = reinterpret_cast<uint4*>(bimg);
      for (int i = threadIdx.x; i < 2 * kImgBytes / 16; i += kThreads) dst[i] = src[i];
      cur_b = b;
    }
    float2* prow = p.psi + (b << p.n);
    float2* lrow = p.lam + (b << p.n);
    produce_rows(prow, c0, p.ins, apsi, offs);
    produce_rows(lrow, c0, p.ins, alam, offs);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      issue_mma(d_psi, psi_s, b_s);
      issue_mma(d_lam, lam_s, b_s);
      if (p.mr_out) issue_cross(d_m, lam_s, psi_s, first_cross);
      mma_commit(bar);
    }
    inflight = 1;
    first_cross = false;
    const int timed_out = mbar_wait(bar, phase) ? 0 : 1;
    if (__syncthreads_or(timed_out)) {
      if (threadIdx.x == 0) atomicExch(p.status, TQK_TIMEOUT);
      aborted = 1;
      break;
    }
    phase ^= 1u;
    inflight = 0;
    tc_fence_after();
    epilogue_rows(prow, c0, p.ins, d_psi, offs);
    epilogue_rows(lrow, c0, p.ins, d_lam, offs);
    tc_fence_before();
    __syncthreads();
  }
  if (aborted && inflight) mbar_wait(bar, phase);
  if (!aborted && p.mr_out && !first_cross) {
    tc_fence_after();
    flush_cross(p.mr_out + (p.u_batch > 1 ? cur_b : 0) * 128 * 128, d_m);
  }
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
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

extern "C" int tqk_fused_adjoint(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires,
                                 const void* image_h, int64_t u_batch, double* mr_out, int* status, void* stream) {
  const char* what = "tqk_fused_adjoint";
  int rc = check_state(psi, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(lam, bsz, n, what))) return rc;
  if ((rc = check_batch(u_batch, bsz, what))) return rc;
  if (!image_h || !status) return fail(TQK_BAD_POINTER, "%s: null image/status", what);
  if (n < 13) return fail(TQK_UNSUPPORTED, "%s: needs n_wires >= 13 (got %d)", what, n);
  int tb[6];
  uint64_t used = 0;
  if ((rc = wires_to_bits(n, wires, 6, tb, &used, what))) return rc;
  tc::AdjParams p;
  p.psi = static_cast<float2*>(psi);
  p.lam = static_cast<float2*>(lam);
  p.n = n;
  p.ins = make_insert(used);
  for (int j = 0; j < 64; ++j) {
    uint64_t o = 0;
    for (int jb = 0; jb < 6; ++jb)
      if ((j >> (5 - jb)) & 1) o |= 1ull << tb[jb];
    p.off[j] = o;
  }
  p.uimg = static_cast<const uint8_t*>(image_h);
  p.u_batch = u_batch;
  p.tiles_per_row = (1ll << (n - 6)) / tc::kTileCols;
  p.tiles = p.tiles_per_row * bsz;
  p.mr_out = mr_out;
  p.status = status;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 1024 + 6 * tc::kImgBytes + 64 * 8 + 8 + 16;
  static int attr_dev = -1;
  if (attr_dev != dev) {
    cudaFuncSetAttribute(tc::k_tc_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    attr_dev = dev;
  }
  const int64_t grid = p.tiles < sms ? p.tiles : sms;
  tc::k_tc_adjoint<<<static_cast<unsigned>(grid), tc::kThreads, smem, as_stream(stream)>>>(p);
  return launch_status(what);
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
  int tb[6];
  uint64_t used = 0;
  if ((rc = wires_to_bits(n, wires, 6, tb, &used, what))) return rc;
  tc::ApplyParams p;
  p.state = static_cast<float2*>(state);
  p.n = n;
  p.bsz = bsz;
  p.ins = make_insert(used);
  for (int j = 0; j < 64; ++j) {
    uint64_t o = 0;
    for (int jb = 0; jb < 6; ++jb)
      if ((j >> (5 - jb)) & 1) o |= 1ull << tb[jb];
    p.off[j] = o;
  }
  p.uimg = static_cast<const uint8_t*>(image);
  p.u_batch = u_batch;
  p.tiles_per_row = (1ll << (n - 6)) / tc::kTileCols;
  p.tiles = p.tiles_per_row * bsz;
  p.status = status;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 1024 + 6 * tc::kImgBytes + 64 * 8 + 2 * 8 + 16;
  static int attr_dev = -1;
  if (attr_dev != dev) {
    cudaFuncSetAttribute(tc::k_tc_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    attr_dev = dev;
  }
  const int64_t grid = p.tiles < sms ? p.tiles : sms;
  tc::k_tc_apply<<<static_cast<unsigned>(grid), tc::kThreads, smem, as_stream(stream)>>>(p);
  return launch_status(what);
}
