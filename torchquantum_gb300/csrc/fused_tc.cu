// fused_tc.cu -- fused k=6 block application on the 5th-generation tensor cores.
//
// A fused block is a dense 64x64 complex unitary U on 6 target bits.  For every column
// c (an assignment of the other n-6 bits) the 64 amplitudes x_c become U x_c.  A tile
// of 128 columns is the A operand of two real GEMMs (M = 128 columns, K = 128):
//   A[i][64p + j]   = part p (0 = Re, 1 = Im) of amplitude (target pattern j, column i)
//   B[j'][64p + j]  = part p of U[j'][j]                      (64 rows, one image)
//   D_re[i][j'] = sum_j Re x Re U - Im x Im U  : K-block 0 of A x K-block 0 of B, plus
//                 K-block 1 of A x K-block 1 of B with the instruction's negate-A bit;
//   D_im[i][j'] = sum_j Re x Im U + Im x Re U  : the same A against B's K-blocks swapped
//                 (descriptor start addresses only).
// Precision: operands are split into bf16 hi + lo parts; three products (hi.hi + hi.lo
// + lo.hi) accumulate in fp32 in tensor memory (~16 mantissa bits per product).
//
// One persistent, warp-specialised CTA per SM.  Shared memory holds U's image (32 KB,
// reloaded only when a per-row U changes with the batch row) and two A images (64 KB
// each).  Eight producer warps load a tile's amplitudes from global memory straight
// into registers (a warp's lanes are consecutive columns, so every load instruction
// covers contiguous runs), split them and write the A image; one thread of the MMA warp
// issues the tile's 48 MMAs into one of two tensor-memory accumulators; four epilogue
// warps drain the other accumulator (tcgen05.ld, lanes = consecutive columns) straight
// to global memory.  The roles meet only at mbarriers, so loads of tile t+2, MMAs of
// tile t+1 and stores of tile t overlap.  The adjoint step uses the same machinery on
// mixed tiles (64 columns of psi and the same 64 columns of lam) against U^H, and adds
// the cross term sum_columns lam~ psi~^T (MN-major reads of the same A image) in a
// third accumulator.  When the state the block was applied to is still in memory (the
// forward wrote each block's output to a new buffer), the adjoint step reads it as the
// psi half and stores only lam: three state transfers instead of four, and the cross
// term is then the block cotangent itself.
// Every mbarrier wait is bounded (clock-based); on a timeout the kernel records
// TQK_TIMEOUT in *status, stops issuing work, waits (bounded) for MMAs in flight,
// frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace tqk {
namespace tc {

constexpr int kImgBytes = 32768;        // one 128-row x 128-K bf16 A image
constexpr int kKBlockBytes = 16384;     // A: 128 rows x 128 B (64 bf16 of K)
constexpr int kBImgBytes = 32768;       // one 128-row x 128-K bf16 B image
constexpr int kBKBlockBytes = 16384;    // B: 128 rows x 128 B
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// byte offset of the 16-byte chunk holding K elements [8*chunk, 8*chunk+8) of row r in a
// SWIZZLE_128B K-major image with K = 128 (chunk 0..15) whose two 64-element K-blocks are
// kb_bytes apart
__device__ __forceinline__ uint32_t sw128_off(int r, int chunk, int kb_bytes) {
  const int kb = chunk >> 3, c = chunk & 7;
  return kb * kb_bytes + (r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4);
}

__device__ __forceinline__ uint32_t pack_bf2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

// 8 floats -> one 16-byte chunk of bf16 hi parts and one of lo parts
__device__ __forceinline__ void split8(const float (&v)[8], uint4& hi, uint4& lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    __nv_bfloat162 hv = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
    const float2 hf = __bfloat1622float2(hv);
    h[e] = *reinterpret_cast<uint32_t*>(&hv);
    l[e] = pack_bf2(v[2 * e] - hf.x, v[2 * e + 1] - hf.y);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Block product: 24 MMAs of 128x128x16 (three split-bf16 terms x 8 K-steps).
// Row-major orientation (tr = false): D[i][m] = sum_K A[i][K] B[m][K] -- TMEM lane =
// tile row i, column m = 2 j' + q.  Transposed (tr = true): the operands swap roles,
// D[m][i] -- TMEM lane m, column i.
__device__ __forceinline__ void issue_mma(uint32_t d_tmem, uint32_t a_s, uint32_t b_s, bool tr) {
  constexpr uint32_t idesc = idesc_bf16(128, 128);
  const uint32_t ao[3] = {0u, 0u, static_cast<uint32_t>(kImgBytes)};   // x: hi, hi, lo
  const uint32_t bo[3] = {0u, static_cast<uint32_t>(kBImgBytes), 0u};  // U: hi, lo, hi
#pragma unroll
  for (int prod = 0; prod < 3; ++prod) {
#pragma unroll
    for (int s = 0; s < 8; ++s) {
      const int kb = s >> 2;
      const uint32_t koff = (s & 3) * 32;
      const uint64_t xd = desc_sw128(a_s + ao[prod] + kb * kKBlockBytes + koff);
      const uint64_t ud = desc_sw128(b_s + bo[prod] + kb * kBKBlockBytes + koff);
      mma_bf16(d_tmem, tr ? ud : xd, tr ? xd : ud, idesc, (prod > 0 || s > 0) ? 1u : 0u);
    }
  }
}

// MN-major SWIZZLE_128B descriptor over a [column][128 (p,j)] tile image: the two
// 64-element halves (p = 0, 1) are 16 KB apart (LBO), 8-column groups 1024 B apart (SBO).
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
// lam~[m] psi~[n] (m, n = 64p + j); lam rows are tile rows 64..127, psi rows 0..63.
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

// insert zeros at the 6 target bits (ascending)
__device__ __forceinline__ uint64_t insert6(uint64_t g, const BitInsert& bi) {
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const int q = bi.pos[i];
    g = ((g >> q) << (q + 1)) | (g & ((1ull << q) - 1ull));
  }
  return g;
}

// U image (2 x 32 KB, contiguous and 1024-byte aligned in shared memory, 16-byte aligned
// in global memory) moved by the bulk-copy engine, completing on `bar`.
__device__ __forceinline__ void load_u_image(uint64_t* bar, uint8_t* dst, const uint8_t* src) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(2 * kBImgBytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(2 * kBImgBytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait of a whole warp on the U image; warp-uniform result.
__device__ __forceinline__ bool wait_u_image(uint64_t* bar, uint32_t parity) {
  return __all_sync(0xffffffffu, mbar_wait(bar, parity));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Pattern orders.  The natural index of a target pattern has wires[0] as its most
// significant bit.  Inside the kernels two other orders are used, both fixed by the
// target bits' positions alone: the output order o (bit b = the b-th lowest target bit)
// indexes output rows, and the K order jk (bit b = the b-th highest target bit) indexes
// the K dimension of the operand images, so that a 16-byte image chunk (K bits 0-2)
// always spans the three highest target bits.  tqk_fused_prepare builds U's image in
// these orders.
//
// A tile is a sub-cube of 13 free dimensions: the 6 target bits, the lowest 7 other
// bits (tile row = column i; ADJ: the lowest 6, plus a psi/lam dimension that selects
// the state and adds 64 to the row).  Producer thread (warp w, lane l) holds 32
// amplitudes r = e + 8c: e = K bits 0-2 (one chunk), c = two more dimensions; its lanes
// run over the 5 lowest-address remaining dimensions, so every load instruction is
// coalesced whatever the target bits are.
struct TcParams {
  float2* psi;               // state read (APPLY) / psi (ADJ)
  float2* psi_out;           // APPLY: product destination (psi: in place); ADJ: U^H psi
                             // destination (psi), or null when psi is the block's stored
                             // input state, which is only read
  float2* lam;               // ADJ only
  int n;
  BitInsert ins;             // the 6 target bits
  const uint8_t* uimg;       // [u_batch][2 images][32 KB] (U for APPLY, U^H for ADJ)
  int64_t u_batch;
  int64_t tiles_per_row;     // a power of two
  int tpr_log2;
  int64_t tiles;
  double* mr_out;            // ADJ: [u_batch][128][128] cross term, or null
  int* status;
  int transposed;            // output orientation (fewer store sectors per warp)
  uint64_t off[64];          // amplitude offset of output pattern j'
  uint64_t col_off[128];     // amplitude offset of tile row i (ADJ: i & 63)
  uint64_t lane_off[32];     // producer mapping: offsets, tile rows and chunk indices
  uint64_t warp_off[8];
  uint64_t reg_off[32];
  uint8_t lane_row[32], lane_g[32];
  uint8_t warp_row[8], warp_g[8], warp_lam[8];
  uint8_t c_row[4], c_g[4];
  uint8_t nat_of_k[64];      // natural pattern index of K-order index jk (cross term)
};

// Warp roles (416 threads): warps 0-7 produce A images, warps 8-11 drain the tensor-
// memory accumulators (warp w reads TMEM lanes 32*(w%4)...), warp 12 owns the tensor
// memory and lane 0 of it issues the MMAs.
constexpr int kProdThreads = 256;
constexpr int kEpiThreads = 128;
constexpr int kThreadsWS = kProdThreads + kEpiThreads + 32;
constexpr int kMmaWarp = (kProdThreads + kEpiThreads) / 32;
constexpr int kABufs = 2;

struct Sync {
  uint64_t a_full[kABufs], a_empty[kABufs], d_full[2], d_empty[2], x_full, x_empty;
  uint64_t u_full;        // bulk-copy (TMA) load of the U image, one use per batch row
  int nat_of_k[128];      // natural row/column of cross-term index 64p + jk
  uint32_t tmem_base;
  int abort;
};

// Bounded wait that also gives up when another role has aborted; warp-uniform result.
__device__ __forceinline__ bool wait_or_abort(uint64_t* bar, uint32_t parity, Sync* sy) {
  bool ok = true;
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (*reinterpret_cast<volatile int*>(&sy->abort)) {
      ok = false;
      break;
    }
    if (clock64() - t0 > kWaitCycles) {
      atomicExch(&sy->abort, 1);
      ok = false;
      break;
    }
  }
  return __all_sync(0xffffffffu, ok);
}

// amplitude offset of tile t within its state (batch row + fixed column bits)
__device__ __forceinline__ int64_t tile_base(const TcParams& p, int64_t t, bool adj) {
  const int cols = adj ? 64 : 128;
  const int64_t b = t >> p.tpr_log2;
  const int64_t c0 = (t & (p.tiles_per_row - 1)) * cols;
  return (b << p.n) + static_cast<int64_t>(insert6(static_cast<uint64_t>(c0), p.ins));
}

// Tiles ahead of the one being loaded whose lines the producers prefetch into L2, so that
// DRAM stays busy while a tile is split and written to shared memory.
#ifndef TQK_TC_PREFETCH
#define TQK_TC_PREFETCH 1
#endif
constexpr int kPrefetchTiles = TQK_TC_PREFETCH;
#ifndef TQK_TC_EARLY_LOAD
#define TQK_TC_EARLY_LOAD 1
#endif

// Registers r whose amplitude starts a 128-byte line (16 amplitudes).  Address bits 0-3
// are always tile dimensions (target bits or among the lowest non-target bits) and are
// clear in a tile's base, so every line of a tile is whole and owned by exactly one
// (thread, register).
__device__ __forceinline__ uint32_t line_owner_mask(const TcParams& p, int64_t toff) {
  uint32_t m = 0;
#pragma unroll
  for (int r = 0; r < 32; ++r)
    if (((static_cast<uint64_t>(toff) + p.reg_off[r]) & 15ull) == 0) m |= 1u << r;
  return m;
}

__device__ __forceinline__ void prefetch_lines(const TcParams& p, const float2* src, uint32_t mask) {
#pragma unroll
  for (int r = 0; r < 32; ++r)
    if ((mask >> r) & 1u) asm volatile("prefetch.global.L2 [%0];" ::"l"(src + p.reg_off[r]));
}

// Producer: the thread's 32 amplitudes of a tile (load_tile), split into bf16 hi/lo and
// stored as its four 16-byte chunks (K = 64p + 8g + e) of the A image (store_tile).
// The loads take the read-only (non-coherent) path: every 128-byte line belongs to one tile
// (see line_owner_mask), is read once by that tile's producers, and is written (by the
// epilogue, in place or lam) only after the tile's MMAs consumed it, so no line is read
// again after a write within the launch.
__device__ __forceinline__ void load_tile(const TcParams& p, const float2* src, float2 (&a)[32]) {
#pragma unroll
  for (int r = 0; r < 32; ++r) a[r] = __ldg(src + p.reg_off[r]);
}

__device__ __forceinline__ void store_tile(const float2 (&a)[32], const TcParams& p, uint8_t* abuf, int row0,
                                           int g0) {
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int row = row0 + p.c_row[c], g = g0 + p.c_g[c];
    float re[8], im[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      re[e] = a[8 * c + e].x;
      im[e] = a[8 * c + e].y;
    }
    uint4 hi, lo;
    split8(re, hi, lo);
    uint32_t o = sw128_off(row, g, kKBlockBytes);
    *reinterpret_cast<uint4*>(abuf + o) = hi;
    *reinterpret_cast<uint4*>(abuf + kImgBytes + o) = lo;
    split8(im, hi, lo);
    o = sw128_off(row, 8 + g, kKBlockBytes);
    *reinterpret_cast<uint4*>(abuf + o) = hi;
    *reinterpret_cast<uint4*>(abuf + kImgBytes + o) = lo;
  }
}

// Row-major drain: TMEM lane = tile row; columns 2j' + q hold part q of output j'.
template <bool ADJ>
__device__ __forceinline__ void drain_rows(const TcParams& p, int64_t tb, uint32_t d_tmem, int sub, int lane) {
  const int row = sub * 32 + lane;
  float2* dbase = (ADJ && row >= 64) ? p.lam : p.psi_out;
  if (ADJ && dbase == nullptr) return;  // psi rows of a stored-input step: warp-uniform (sub 0, 1)
  float2* dst = dbase + tb + p.col_off[row];
  const uint32_t lanes = static_cast<uint32_t>(sub * 32) << 16;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t v[32];
    tmem_ld16(d_tmem + lanes + q * 32, *reinterpret_cast<uint32_t(*)[16]>(&v[0]));
    tmem_ld16(d_tmem + lanes + q * 32 + 16, *reinterpret_cast<uint32_t(*)[16]>(&v[16]));
    tmem_wait_ld();
#pragma unroll
    for (int h = 0; h < 16; ++h)
      __stcs(dst + p.off[q * 16 + h], make_float2(__uint_as_float(v[2 * h]), __uint_as_float(v[2 * h + 1])));
  }
}

// Transposed drain: TMEM lane m = 2j' + q, columns = tile rows; lanes of a warp write 16
// consecutive outputs' real and imaginary parts.
template <bool ADJ>
__device__ __forceinline__ void drain_cols(const TcParams& p, int64_t tb, uint32_t d_tmem, int sub, int lane) {
  const int m = sub * 32 + lane;
  const uint32_t lanes = static_cast<uint32_t>(sub * 32) << 16;
  const int64_t o = tb + static_cast<int64_t>(p.off[m >> 1]);
  float* dpsi = p.psi_out ? reinterpret_cast<float*>(p.psi_out + o) + (m & 1) : nullptr;
  float* dlam = ADJ ? reinterpret_cast<float*>(p.lam + o) + (m & 1) : nullptr;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (ADJ && q < 4 && dpsi == nullptr) continue;  // psi columns of a stored-input step
    uint32_t v[16];
    tmem_ld16(d_tmem + lanes + q * 16, v);
    tmem_wait_ld();
    float* d = (ADJ && q >= 4) ? dlam : dpsi;
#pragma unroll
    for (int h = 0; h < 16; ++h) __stcs(d + 2 * p.col_off[q * 16 + h], __uint_as_float(v[h]));
  }
}

// Cross term (K-order rows and columns 64p + jk) added into dst in natural order.
__device__ __forceinline__ void flush_cross(const Sync* sy, double* dst, uint32_t d_tmem, int sub, int lane) {
  const int m = sub * 32 + lane;
  const uint32_t lanes = static_cast<uint32_t>(sub * 32) << 16;
  double* drow = dst + sy->nat_of_k[m] * 128;
#pragma unroll 1
  for (int part = 0; part < 8; ++part) {
    uint32_t r[16];
    tmem_ld16(d_tmem + lanes + part * 16, r);
    tmem_wait_ld();
#pragma unroll
    for (int v = 0; v < 16; ++v)
      atomicAdd(drow + sy->nat_of_k[part * 16 + v], static_cast<double>(__uint_as_float(r[v])));
  }
}

// Warp-specialised kernel for the forward block application (ADJ = false) and the
// adjoint step (ADJ = true).  Shared memory: U (U^H) image 64 KB + two A images of
// 64 KB.  Hand-offs: a_full/a_empty (producers <-> MMA), d_full/d_empty (MMA <->
// epilogue, two accumulators), x_full/x_empty (adjoint cross term of a finished row).
template <bool ADJ>
__global__ void __launch_bounds__(kThreadsWS, 1) k_tc(const TcParams p) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  uint8_t* bimg = smem;                    // 64 KB
  uint8_t* abufs = smem + 2 * kBImgBytes;  // kABufs x 64 KB
  Sync* sy = reinterpret_cast<Sync*>(abufs + kABufs * 2 * kImgBytes);

  const int64_t per = (p.tiles + gridDim.x - 1) / gridDim.x;
  const int64_t t_begin = blockIdx.x * per;
  const int64_t t_end = min(p.tiles, t_begin + per);
  if (t_begin >= t_end) return;  // uniform for the block
  const int64_t ntiles = t_end - t_begin;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ncols_tmem = ADJ ? 512u : 256u;
  const bool want_cross = ADJ && p.mr_out != nullptr;
  const bool flush_per_row = want_cross && p.u_batch > 1;
  const bool tr = p.transposed != 0;

  if (threadIdx.x < 128) sy->nat_of_k[threadIdx.x] = (threadIdx.x & 64) + p.nat_of_k[threadIdx.x & 63];
  if (threadIdx.x == 0) {
    for (int i = 0; i < kABufs; ++i) {
      mbar_init(&sy->a_full[i], kProdThreads);
      mbar_init(&sy->a_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&sy->d_full[i], 1);
      mbar_init(&sy->d_empty[i], kEpiThreads);
    }
    mbar_init(&sy->x_full, 1);
    mbar_init(&sy->x_empty, kEpiThreads);
    sy->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sy->tmem_base)),
                 "r"(ncols_tmem)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    // U (or U^H) image of the first row: one bulk-copy (TMA) load of 64 KB on u_full,
    // initialised here by the warp that uses it
    if (lane == 0) {
      mbar_init(&sy->u_full, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      load_u_image(&sy->u_full, bimg, p.uimg + (p.u_batch > 1 ? (t_begin >> p.tpr_log2) : 0) * 2 * kBImgBytes);
    }
    __syncwarp();
    if (!wait_u_image(&sy->u_full, 0u) && lane == 0) atomicExch(&sy->abort, 1);
    tc_fence_before();
  }
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sy->tmem_base;

  if (threadIdx.x < kProdThreads) {
    // ------------------------------------------------------------ producers
    const int64_t toff = static_cast<int64_t>(p.lane_off[lane] + p.warp_off[warp]);
    const int row0 = p.lane_row[lane] + p.warp_row[warp];
    const int g0 = p.lane_g[lane] + p.warp_g[warp];
    const float2* base = (ADJ && p.warp_lam[warp]) ? p.lam : p.psi;
    const uint32_t pf_mask = kPrefetchTiles > 0 ? line_owner_mask(p, toff) : 0u;
    for (int64_t k = 1; k < kPrefetchTiles && k < ntiles; ++k)
      prefetch_lines(p, base + tile_base(p, t_begin + k, ADJ) + toff, pf_mask);
    for (int64_t k = 0; k < ntiles; ++k) {
      const int buf = static_cast<int>(k % kABufs);
      if (kPrefetchTiles > 0 && k + kPrefetchTiles < ntiles)
        prefetch_lines(p, base + tile_base(p, t_begin + k + kPrefetchTiles, ADJ) + toff, pf_mask);
      // the tile's loads are issued before the wait for its buffer, so their latency
      // overlaps the MMA that still reads the buffer (tiles are disjoint: nothing this
      // kernel writes is read here)
      float2 a[32];
#if TQK_TC_EARLY_LOAD
      load_tile(p, base + tile_base(p, t_begin + k, ADJ) + toff, a);
#endif
      if (k >= kABufs && !wait_or_abort(&sy->a_empty[buf], static_cast<uint32_t>((k / kABufs - 1) & 1), sy)) break;
#if !TQK_TC_EARLY_LOAD
      load_tile(p, base + tile_base(p, t_begin + k, ADJ) + toff, a);
#endif
      store_tile(a, p, abufs + buf * 2 * kImgBytes, row0, g0);
      fence_proxy_async();
      mbar_arrive(&sy->a_full[buf]);
    }
  } else if (warp < kMmaWarp) {
    // ------------------------------------------------------------ epilogue
    const int sub = warp & 3;
    int64_t cur_b = t_begin >> p.tpr_log2;
    uint32_t xphase = 0;
    bool ok = true;
    for (int64_t k = 0; k < ntiles; ++k) {
      const int64_t t = t_begin + k;
      const int64_t b = t >> p.tpr_log2;
      if (flush_per_row && b != cur_b) {
        if (!(ok = wait_or_abort(&sy->x_full, xphase, sy))) break;
        tc_fence_after();
        flush_cross(sy, p.mr_out + cur_b * 128 * 128, tmem + 256, sub, lane);
        tc_fence_before();
        mbar_arrive(&sy->x_empty);
        xphase ^= 1u;
      }
      cur_b = b;
      const int d = static_cast<int>(k & 1);
      if (!(ok = wait_or_abort(&sy->d_full[d], static_cast<uint32_t>((k >> 1) & 1), sy))) break;
      tc_fence_after();
      const uint32_t dt = tmem + static_cast<uint32_t>(d * 128);
      if (tr) drain_cols<ADJ>(p, tile_base(p, t, ADJ), dt, sub, lane);
      else drain_rows<ADJ>(p, tile_base(p, t, ADJ), dt, sub, lane);
      tc_fence_before();
      mbar_arrive(&sy->d_empty[d]);
    }
    if (ok && want_cross && wait_or_abort(&sy->x_full, xphase, sy)) {
      tc_fence_after();
      flush_cross(sy, p.mr_out + (p.u_batch > 1 ? cur_b : 0) * 128 * 128, tmem + 256, sub, lane);
      tc_fence_before();
    }
  } else {
    // ------------------------------------------------------------ MMA issuer
    uint32_t u_use = 1;  // uses of u_full so far (the first row's image is use 0)
    int64_t cur_b = t_begin >> p.tpr_log2;
    bool first_cross = true;
    uint32_t xphase = 0;
    int64_t issued = 0;
    for (int64_t k = 0; k < ntiles; ++k) {
      const int64_t t = t_begin + k;
      const int64_t b = t >> p.tpr_log2;
      if (b != cur_b) {
        if (flush_per_row) {  // hand the finished row's cross term to the epilogue warps
          if (lane == 0) mma_commit(&sy->x_full);
          __syncwarp();
          if (!wait_or_abort(&sy->x_empty, xphase, sy)) break;
          xphase ^= 1u;
          first_cross = true;
        }
        if (p.u_batch > 1) {  // reload U once every MMA of the previous row has completed
          if (!wait_or_abort(&sy->d_full[(k - 1) & 1], static_cast<uint32_t>(((k - 1) >> 1) & 1), sy)) break;
          if (lane == 0) load_u_image(&sy->u_full, bimg, p.uimg + b * 2 * kBImgBytes);
          __syncwarp();
          if (!wait_or_abort(&sy->u_full, u_use & 1u, sy)) break;
          ++u_use;
        }
        cur_b = b;
      }
      const int buf = static_cast<int>(k % kABufs);
      const int d = static_cast<int>(k & 1);
      if (!wait_or_abort(&sy->a_full[buf], static_cast<uint32_t>((k / kABufs) & 1), sy)) break;
      if (k >= 2 && !wait_or_abort(&sy->d_empty[d], static_cast<uint32_t>(((k >> 1) - 1) & 1), sy)) break;
      tc_fence_after();
      if (lane == 0) {
        const uint32_t a_s = smem_u32(abufs + buf * 2 * kImgBytes);
        issue_mma(tmem + static_cast<uint32_t>(d * 128), a_s, smem_u32(bimg), tr);
        if (want_cross) issue_cross(tmem + 256, a_s, first_cross);
        mma_commit(&sy->a_empty[buf]);
        mma_commit(&sy->d_full[d]);
      }
      __syncwarp();
      first_cross = false;
      issued = k + 1;
    }
    if (want_cross && lane == 0) mma_commit(&sy->x_full);
    __syncwarp();
    // Bounded wait (even after an abort) for the MMAs in flight before the tensor
    // memory is released: the last commit covers every earlier MMA of this thread.
    if (issued > 0) {
      const bool done = mbar_wait(&sy->d_full[(issued - 1) & 1], static_cast<uint32_t>(((issued - 1) >> 1) & 1));
      if (!__all_sync(0xffffffffu, done) && lane == 0) atomicExch(&sy->abort, 1);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && sy->abort) atomicExch(p.status, TQK_TIMEOUT);
  if (warp == kMmaWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols_tmem) : "memory");
  }
}

struct PatternOrders {
  uint8_t nat_of_out[64];  // natural index of output-order index o
  uint8_t nat_of_k[64];    // natural index of K-order index jk
};

// Output and K orders of a block from its wires: the wire with the largest number is the
// lowest target bit.  asc[b] = position jb in `wires` of the b-th lowest target bit.
__host__ __device__ inline void target_order(const int32_t* wires, int (&asc)[6]) {
  for (int i = 0; i < 6; ++i) asc[i] = i;
  for (int x = 1; x < 6; ++x)
    for (int y = x; y > 0 && wires[asc[y - 1]] < wires[asc[y]]; --y) {
      const int t = asc[y];
      asc[y] = asc[y - 1];
      asc[y - 1] = t;
    }
}

// Natural index of output-order index x (korder = false) or K-order index x (true).
__host__ __device__ inline int nat_of(int x, const int (&asc)[6], bool korder) {
  int r = 0;
  for (int b = 0; b < 6; ++b)
    if ((x >> b) & 1) r |= 1 << (5 - asc[korder ? 5 - b : b]);
  return r;
}

__host__ PatternOrders pattern_orders(const int32_t* wires) {
  int asc[6];
  target_order(wires, asc);
  PatternOrders o;
  for (int x = 0; x < 64; ++x) {
    o.nat_of_out[x] = static_cast<uint8_t>(nat_of(x, asc, false));
    o.nat_of_k[x] = static_cast<uint8_t>(nat_of(x, asc, true));
  }
  return o;
}

// U (complex128 [u_batch][64][64], row-major, natural order) -> hi/lo bf16 images of the
// U operand expected by k_tc (SWIZZLE_128B K-major, 128 rows, K = 64p + jk): row 2o holds
// [Re U[o][jk] | -Im U[o][jk]], row 2o+1 holds [Im U[o][jk] | Re U[o][jk]] (o, jk in
// the output and K orders), so one N = 128 product with a tile [Re x | Im x] gives the
// real and imaginary parts of (U x)[o] side by side.  One thread per (batch, row,
// 16-byte chunk).
// ADJ: the image of U^H, read from U (entry (o, k) of U^H is conj U[k][o]).
// One 16-byte chunk (8 K entries) of row `row` of the image, hi and lo parts; orow is the
// natural output index of the row, kcol(k) the natural index of K-order index k.
template <bool ADJ, typename KCol>
__device__ __forceinline__ void prep_chunk(const double2* ub, uint8_t* base, int row, int chunk, int orow,
                                           KCol kcol) {
  float hv[8], lv[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) {
    const int kk = chunk * 8 + e;
    const int kc = kcol(kk & 63);
    double2 z = ADJ ? ub[kc * 64 + orow] : ub[orow * 64 + kc];
    if (ADJ) z.y = -z.y;
    const double v = (row & 1) == 0 ? (kk < 64 ? z.x : -z.y) : (kk < 64 ? z.y : z.x);
    const __nv_bfloat16 h = __double2bfloat16(v);
    hv[e] = __bfloat162float(h);
    lv[e] = static_cast<float>(v - static_cast<double>(hv[e]));
  }
  uint4 hi = make_uint4(pack_bf2(hv[0], hv[1]), pack_bf2(hv[2], hv[3]), pack_bf2(hv[4], hv[5]), pack_bf2(hv[6], hv[7]));
  uint4 lo = make_uint4(pack_bf2(lv[0], lv[1]), pack_bf2(lv[2], lv[3]), pack_bf2(lv[4], lv[5]), pack_bf2(lv[6], lv[7]));
  const uint32_t o = sw128_off(row, chunk, kBKBlockBytes);
  *reinterpret_cast<uint4*>(base + o) = hi;
  *reinterpret_cast<uint4*>(base + kBImgBytes + o) = lo;
}

// U (complex128 [u_batch][64][64], row-major, natural order) -> hi/lo bf16 images of the
// U operand expected by k_tc (SWIZZLE_128B K-major, 128 rows, K = 64p + jk): row 2o holds
// [Re U[o][jk] | -Im U[o][jk]], row 2o+1 holds [Im U[o][jk] | Re U[o][jk]] (o, jk in
// the output and K orders), so one N = 128 product with a tile [Re x | Im x] gives the
// real and imaginary parts of (U x)[o] side by side.  One thread per (batch, row,
// 16-byte chunk).
// ADJ: the image of U^H, read from U (entry (o, k) of U^H is conj U[k][o]).
template <bool ADJ>
__global__ void k_tc_prep(const double2* u, int64_t u_batch, uint8_t* img, const __grid_constant__ PatternOrders ord) {
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= u_batch * 128 * 16) return;
  const int64_t b = idx / (128 * 16);
  const int row = static_cast<int>((idx / 16) % 128);
  const int chunk = static_cast<int>(idx % 16);
  prep_chunk<ADJ>(u + b * 64 * 64, img + b * 2 * kBImgBytes, row, chunk, ord.nat_of_out[row >> 1],
                  [&](int k) { return static_cast<int>(ord.nat_of_k[k]); });
}

// Many images in one launch: blockIdx.y = job, the orders computed from the job's wires.
__global__ void k_tc_prep_many(const tqk_image_job* jobs) {
  const tqk_image_job j = jobs[blockIdx.y];
  const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (idx >= j.u_batch * 128 * 16) return;
  int asc[6];
  target_order(j.wires, asc);
  const int64_t b = idx / (128 * 16);
  const int row = static_cast<int>((idx / 16) % 128);
  const int chunk = static_cast<int>(idx % 16);
  const double2* ub = static_cast<const double2*>(j.u) + b * 64 * 64;
  uint8_t* base = static_cast<uint8_t*>(j.image) + b * 2 * kBImgBytes;
  const int orow = nat_of(row >> 1, asc, false);
  auto kcol = [&](int k) { return nat_of(k, asc, true); };
  if (j.adjoint) prep_chunk<true>(ub, base, row, chunk, orow, kcol);
  else prep_chunk<false>(ub, base, row, chunk, orow, kcol);
}

}  // namespace tc
}  // namespace tqk

using namespace tqk;

static_assert(sizeof(tqk_image_job) == 56 && sizeof(tqk_cross_job) == 24, "job records are part of the C ABI");

extern "C" int64_t tqk_fused_image_bytes(int64_t u_batch) { return u_batch * 2 * tc::kBImgBytes; }

namespace {
int prepare_entry(const void* u, int64_t u_batch, const int32_t* wires, void* image, void* stream, bool adj,
                  const char* what) {
  if (!u || !image || !wires) return fail(TQK_BAD_POINTER, "%s: null pointer", what);
  if ((reinterpret_cast<uintptr_t>(image) & 15u) != 0) return fail(TQK_BAD_POINTER, "%s: image must be 16-byte aligned", what);
  if (u_batch < 1) return fail(TQK_BAD_SHAPE, "%s: u_batch must be >= 1", what);
  for (int i = 0; i < 6; ++i) {
    if (wires[i] < 0) return fail(TQK_BAD_WIRES, "%s: negative wire %d", what, wires[i]);
    for (int k = 0; k < i; ++k)
      if (wires[k] == wires[i]) return fail(TQK_BAD_WIRES, "%s: wire %d used twice", what, wires[i]);
  }
  const int64_t work = u_batch * 128 * 16;
  const unsigned grid = static_cast<unsigned>((work + 255) / 256);
  if (adj)
    tc::k_tc_prep<true><<<grid, 256, 0, as_stream(stream)>>>(static_cast<const double2*>(u), u_batch,
                                                           static_cast<uint8_t*>(image), tc::pattern_orders(wires));
  else
    tc::k_tc_prep<false><<<grid, 256, 0, as_stream(stream)>>>(static_cast<const double2*>(u), u_batch,
                                                            static_cast<uint8_t*>(image), tc::pattern_orders(wires));
  return launch_status(what);
}
}  // namespace

extern "C" int tqk_fused_prepare(const void* u, int64_t u_batch, const int32_t* wires, void* image, void* stream) {
  return prepare_entry(u, u_batch, wires, image, stream, false, "tqk_fused_prepare");
}

extern "C" int tqk_fused_prepare_adjoint(const void* u, int64_t u_batch, const int32_t* wires, void* image,
                                         void* stream) {
  return prepare_entry(u, u_batch, wires, image, stream, true, "tqk_fused_prepare_adjoint");
}

extern "C" int tqk_fused_prepare_many(const tqk_image_job* jobs, int njobs, int64_t max_u_batch, void* stream) {
  if (njobs <= 0) return TQK_OK;
  if (!jobs) return fail(TQK_BAD_POINTER, "tqk_fused_prepare_many: null job table");
  if (njobs > 65535 || max_u_batch < 1 || max_u_batch > (1ll << 40))
    return fail(TQK_BAD_SHAPE, "tqk_fused_prepare_many: %d jobs, max u_batch %lld", njobs, (long long)max_u_batch);
  const int64_t work = max_u_batch * 128 * 16;
  dim3 grid(static_cast<unsigned>((work + 255) / 256), static_cast<unsigned>(njobs), 1);
  tc::k_tc_prep_many<<<grid, 256, 0, as_stream(stream)>>>(jobs);
  return launch_status("tqk_fused_prepare_many");
}

// gu[b] += M_b U_b for the block cotangent: M_b (64 x 64 complex) from the adjoint step's
// real cross term mr[b] (rows / columns 64p + j, p = 0 real, 1 imaginary part:
// M[j][j'] = mr[j][j'] + mr[64+j][64+j'] + i (mr[64+j][j'] - mr[j][64+j'])), U_b the
// block unitary (complex128); the product in float32 (M carries fp32 accuracy),
// accumulated into gu (complex128).  One CTA per batch row.
namespace tqk {
namespace tc {
__global__ void __launch_bounds__(256) k_cross_grad(const double* mr, const double2* u, double2* gu) {
  extern __shared__ float2 cg_smem[];  // M [64][64] then U [64][64]: 64 KB
  float2(*M)[64] = reinterpret_cast<float2(*)[64]>(cg_smem);
  float2(*U)[64] = reinterpret_cast<float2(*)[64]>(cg_smem + 64 * 64);
  const int64_t b = blockIdx.x;
  const double* m = mr + b * 128 * 128;
  const double2* ub = u + b * 64 * 64;
  for (int e = threadIdx.x; e < 64 * 64; e += 256) {
    const int j = e >> 6, k = e & 63;
    const double re = m[j * 128 + k] + m[(64 + j) * 128 + 64 + k];
    const double im = m[(64 + j) * 128 + k] - m[j * 128 + 64 + k];
    M[j][k] = make_float2(static_cast<float>(re), static_cast<float>(im));
    const double2 z = ub[e];
    U[j][k] = make_float2(static_cast<float>(z.x), static_cast<float>(z.y));
  }
  __syncthreads();
  double2* g = gu + b * 64 * 64;
  for (int e = threadIdx.x; e < 64 * 64; e += 256) {
    const int j = e >> 6, k = e & 63;
    float ax = 0.f, ay = 0.f;
#pragma unroll 8
    for (int t = 0; t < 64; ++t) {
      const float2 a = M[j][t], c = U[t][k];
      ax = fmaf(a.x, c.x, fmaf(-a.y, c.y, ax));
      ay = fmaf(a.x, c.y, fmaf(a.y, c.x, ay));
    }
    g[e].x += static_cast<double>(ax);
    g[e].y += static_cast<double>(ay);
  }
}

// gu[b] += M_b: the cross term of a stored-input adjoint step is the cotangent itself
// (float64 throughout).  One thread per complex entry.
__device__ __forceinline__ void cross_add_entry(const double* mr, double2* gu, int64_t e) {
  const int64_t b = e >> 12;
  const int j = static_cast<int>((e >> 6) & 63), k = static_cast<int>(e & 63);
  const double* m = mr + b * 128 * 128;
  gu[e].x += m[j * 128 + k] + m[(64 + j) * 128 + 64 + k];
  gu[e].y += m[(64 + j) * 128 + k] - m[j * 128 + 64 + k];
}

__global__ void __launch_bounds__(256) k_cross_add(const double* mr, int64_t batch, double2* gu) {
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < batch * 64 * 64) cross_add_entry(mr, gu, e);
}

// Many blocks in one launch: blockIdx.y = job.
__global__ void __launch_bounds__(256) k_cross_add_many(const tqk_cross_job* jobs) {
  const tqk_cross_job j = jobs[blockIdx.y];
  const int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (e < j.batch * 64 * 64) cross_add_entry(j.mr, static_cast<double2*>(j.gu), e);
}
}  // namespace tc
}  // namespace tqk

extern "C" int tqk_fused_cross_grad(const double* mr, const void* u, int64_t batch, void* gu, void* stream) {
  if (!mr || !gu) return fail(TQK_BAD_POINTER, "tqk_fused_cross_grad: null pointer");
  if (batch < 1 || batch > 0x7fffffff) return fail(TQK_BAD_SHAPE, "tqk_fused_cross_grad: batch %lld", (long long)batch);
  if (u == nullptr) {
    const int64_t work = batch * 64 * 64;
    tc::k_cross_add<<<static_cast<unsigned>((work + 255) / 256), 256, 0, as_stream(stream)>>>(
        mr, batch, static_cast<double2*>(gu));
    return launch_status("tqk_fused_cross_grad");
  }
  constexpr int smem = 2 * 64 * 64 * static_cast<int>(sizeof(float2));
  static int attr_dev = -1;
  int dev = 0;
  cudaGetDevice(&dev);
  if (attr_dev != dev) {
    cudaFuncSetAttribute(tc::k_cross_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr_dev = dev;
  }
  tc::k_cross_grad<<<static_cast<unsigned>(batch), 256, smem, as_stream(stream)>>>(
      mr, static_cast<const double2*>(u), static_cast<double2*>(gu));
  return launch_status("tqk_fused_cross_grad");
}

extern "C" int tqk_fused_cross_add_many(const tqk_cross_job* jobs, int njobs, int64_t max_batch, void* stream) {
  if (njobs <= 0) return TQK_OK;
  if (!jobs) return fail(TQK_BAD_POINTER, "tqk_fused_cross_add_many: null job table");
  if (njobs > 65535 || max_batch < 1 || max_batch > (1ll << 40))
    return fail(TQK_BAD_SHAPE, "tqk_fused_cross_add_many: %d jobs, max batch %lld", njobs, (long long)max_batch);
  const int64_t work = max_batch * 64 * 64;
  dim3 grid(static_cast<unsigned>((work + 255) / 256), static_cast<unsigned>(njobs), 1);
  tc::k_cross_add_many<<<grid, 256, 0, as_stream(stream)>>>(jobs);
  return launch_status("tqk_fused_cross_add_many");
}

namespace tqk {
namespace tc {

// Amplitude offsets of a 6-wire block's 64 patterns with every other bit clear.
struct PatternOffsets {
  uint64_t off[64];
};

// A block applied to |0...0>: row b's amplitude at pattern j becomes U_b[j][0] (the rest of
// the row is zero already).  One thread per pattern, one CTA per row.
__global__ void __launch_bounds__(64) k_zero_input(float2* state, int n, const double2* u, int64_t u_batch,
                                                   const __grid_constant__ PatternOffsets po) {
  const int64_t b = blockIdx.x;
  const int j = threadIdx.x;
  const double2 v = u[((u_batch > 1 ? b : 0) * 64 + j) * 64];
  state[(b << n) + po.off[j]] = make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
}

}  // namespace tc
}  // namespace tqk

extern "C" int tqk_fused_zero_input(void* state, int64_t bsz, int n, const int32_t* wires, const void* u,
                                    int64_t u_batch, void* stream) {
  using namespace tqk;
  const char* what = "tqk_fused_zero_input";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_batch(u_batch, bsz, what))) return rc;
  if (u == nullptr) return fail(TQK_BAD_POINTER, "%s: null block unitary", what);
  if (bsz > 2147483647ll) return fail(TQK_BAD_SHAPE, "%s: bsz %lld", what, (long long)bsz);
  int bits[6];
  uint64_t used = 0;
  if ((rc = wires_to_bits(n, wires, 6, bits, &used, what))) return rc;
  tc::PatternOffsets po;
  for (int j = 0; j < 64; ++j) {
    uint64_t o = 0;
    for (int i = 0; i < 6; ++i)
      if ((j >> (5 - i)) & 1) o |= 1ull << bits[i];
    po.off[j] = o;
  }
  tc::k_zero_input<<<static_cast<unsigned>(bsz), 64, 0, as_stream(stream)>>>(
      static_cast<float2*>(state), n, static_cast<const double2*>(u), u_batch, po);
  return launch_status(what);
}

namespace {

// One free dimension of a tile and what it adds to an amplitude offset, the tile row
// (i, plus 64 for lam), the image chunk index g (pattern bits 3-5) and the state choice.
struct TileDim {
  int addr;  // address bit (-1: the psi/lam dimension)
  uint64_t off;
  int row, g, lam;
};

int tc_setup(tqk::tc::TcParams& p, int64_t bsz, int n, const int32_t* wires, bool adj, const char* what) {
  using namespace tqk;
  uint64_t used = 0;
  int rc = wires_to_bits(n, wires, 6, nullptr, &used, what);
  if (rc) return rc;
  p.n = n;
  p.ins = make_insert(used);
  int tasc[6];  // target bits ascending
  for (int i = 0, q = 0; q < n; ++q)
    if ((used >> q) & 1ull) tasc[i++] = q;
  for (int o = 0; o < 64; ++o) {  // output order: bit b = b-th lowest target bit
    uint64_t x = 0;
    for (int b = 0; b < 6; ++b)
      if ((o >> b) & 1) x |= 1ull << tasc[b];
    p.off[o] = x;
  }
  const tc::PatternOrders ord = tc::pattern_orders(wires);
  for (int x = 0; x < 64; ++x) p.nat_of_k[x] = ord.nat_of_k[x];
  auto koff = [&](int jk) {  // K order: bit b = b-th highest target bit
    uint64_t x = 0;
    for (int b = 0; b < 6; ++b)
      if ((jk >> b) & 1) x |= 1ull << tasc[5 - b];
    return x;
  };
  const int ncol = adj ? 6 : 7;
  int colbit[7], nc = 0;
  for (int q = 0; q < n && nc < ncol; ++q)
    if (!((used >> q) & 1ull)) colbit[nc++] = q;
  for (int i = 0; i < 128; ++i) {
    const int ii = adj ? (i & 63) : i;
    uint64_t o = 0;
    for (int c = 0; c < ncol; ++c)
      if ((ii >> c) & 1) o |= 1ull << colbit[c];
    p.col_off[i] = o;
  }
  // Producer mapping.  Register bits 0-2: K bits 0-2 (the three highest target bits);
  // the remaining address dimensions sorted by address bit: 5 lanes, 2 register bits,
  // the rest warp bits; ADJ adds the psi/lam dimension as the top warp bit.
  TileDim rest[10];
  int nr = 0;
  for (int b = 3; b < 6; ++b) rest[nr++] = {tasc[5 - b], 1ull << tasc[5 - b], 0, 1 << (b - 3), 0};
  for (int c = 0; c < ncol; ++c) rest[nr++] = {colbit[c], 1ull << colbit[c], 1 << c, 0, 0};
  for (int x = 1; x < nr; ++x)  // insertion sort by address bit
    for (int y = x; y > 0 && rest[y - 1].addr > rest[y].addr; --y) {
      const TileDim t = rest[y];
      rest[y] = rest[y - 1];
      rest[y - 1] = t;
    }
  TileDim wdim[3];
  int nw = 0;
  for (int x = 7; x < nr; ++x) wdim[nw++] = rest[x];
  if (adj) wdim[nw++] = {-1, 0, 64, 0, 1};
  for (int l = 0; l < 32; ++l) {
    uint64_t o = 0;
    int row = 0, g = 0;
    for (int bb = 0; bb < 5; ++bb)
      if ((l >> bb) & 1) {
        o += rest[bb].off;
        row += rest[bb].row;
        g += rest[bb].g;
      }
    p.lane_off[l] = o;
    p.lane_row[l] = static_cast<uint8_t>(row);
    p.lane_g[l] = static_cast<uint8_t>(g);
  }
  for (int w = 0; w < 8; ++w) {
    uint64_t o = 0;
    int row = 0, g = 0, lam = 0;
    for (int bb = 0; bb < 3; ++bb)
      if ((w >> bb) & 1) {
        o += wdim[bb].off;
        row += wdim[bb].row;
        g += wdim[bb].g;
        lam |= wdim[bb].lam;
      }
    p.warp_off[w] = o;
    p.warp_row[w] = static_cast<uint8_t>(row);
    p.warp_g[w] = static_cast<uint8_t>(g);
    p.warp_lam[w] = static_cast<uint8_t>(lam);
  }
  for (int c = 0; c < 4; ++c) {
    p.c_row[c] = static_cast<uint8_t>(((c & 1) ? rest[5].row : 0) + ((c & 2) ? rest[6].row : 0));
    p.c_g[c] = static_cast<uint8_t>(((c & 1) ? rest[5].g : 0) + ((c & 2) ? rest[6].g : 0));
  }
  for (int r = 0; r < 32; ++r) {
    uint64_t o = koff(r & 7);  // K bits 0-2
    if (r & 8) o += rest[5].off;
    if (r & 16) o += rest[6].off;
    p.reg_off[r] = o;
  }
  // Output orientation: 32-byte sectors one warp store touches -- row-major: 32
  // consecutive tile rows of one output; transposed: both parts of 16 consecutive outputs.
  auto distinct_sectors = [](const uint64_t* o, int m) {
    int cnt = 0;
    for (int x = 0; x < m; ++x) {
      bool seen = false;
      for (int y = 0; y < x && !seen; ++y) seen = (o[y] >> 2) == (o[x] >> 2);
      cnt += !seen;
    }
    return cnt;
  };
  p.transposed = distinct_sectors(p.off, 16) < distinct_sectors(p.col_off, 32) ? 1 : 0;
  p.tiles_per_row = (1ll << (n - 6)) / (adj ? 64 : 128);
  p.tpr_log2 = n - 6 - (adj ? 6 : 7);
  p.tiles = p.tiles_per_row * bsz;
  return TQK_OK;
}

int tc_launch(const tqk::tc::TcParams& p, bool adj, void* stream, const char* what) {
  using namespace tqk;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = 1024 + 2 * tc::kBImgBytes + tc::kABufs * 2 * tc::kImgBytes + sizeof(tc::Sync);
  static int attr_dev[2] = {-1, -1};
  if (attr_dev[adj] != dev) {
    if (adj) cudaFuncSetAttribute(tc::k_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    else cudaFuncSetAttribute(tc::k_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    attr_dev[adj] = dev;
  }
  const int64_t grid = p.tiles < sms ? p.tiles : sms;
  if (adj) tc::k_tc<true><<<static_cast<unsigned>(grid), tc::kThreadsWS, smem, as_stream(stream)>>>(p);
  else tc::k_tc<false><<<static_cast<unsigned>(grid), tc::kThreadsWS, smem, as_stream(stream)>>>(p);
  return launch_status(what);
}

}  // namespace

namespace {

// Stored state buffers must not overlap a buffer the same launch writes (other than
// being that buffer).
bool overlaps(const void* a, const void* b, int64_t bytes) {
  const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
  return x != y && x < y + static_cast<uintptr_t>(bytes) && y < x + static_cast<uintptr_t>(bytes);
}

int adjoint_entry(const void* psi, float2* psi_out, void* lam, int64_t bsz, int n, const int32_t* wires,
                  const void* image_h, int64_t u_batch, double* mr_out, int* status, void* stream, const char* what) {
  int rc = check_state(psi, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(lam, bsz, n, what))) return rc;
  if ((rc = check_batch(u_batch, bsz, what))) return rc;
  if (!image_h || !status) return fail(TQK_BAD_POINTER, "%s: null image/status", what);
  if (n < 13) return fail(TQK_UNSUPPORTED, "%s: needs n_wires >= 13 (got %d)", what, n);
  const int64_t bytes = bsz * (int64_t(8) << n);
  if (psi == lam || overlaps(psi, lam, bytes)) return fail(TQK_BAD_POINTER, "%s: psi and lam overlap", what);
  tc::TcParams p;
  p.psi = const_cast<float2*>(static_cast<const float2*>(psi));
  p.psi_out = psi_out;
  p.lam = static_cast<float2*>(lam);
  p.uimg = static_cast<const uint8_t*>(image_h);
  p.u_batch = u_batch;
  p.mr_out = mr_out;
  p.status = status;
  if ((rc = tc_setup(p, bsz, n, wires, true, what))) return rc;
  return tc_launch(p, true, stream, what);
}

int apply_entry(const void* in, void* out, int64_t bsz, int n, const int32_t* wires, const void* image,
                int64_t u_batch, int* status, void* stream, const char* what) {
  int rc = check_state(in, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(out, bsz, n, what))) return rc;
  if ((rc = check_batch(u_batch, bsz, what))) return rc;
  if (!image || !status) return fail(TQK_BAD_POINTER, "%s: null image/status", what);
  if ((reinterpret_cast<uintptr_t>(image) & 15u) != 0) return fail(TQK_BAD_POINTER, "%s: image alignment", what);
  if (n < 13) return fail(TQK_UNSUPPORTED, "%s: needs n_wires >= 13 (got %d)", what, n);
  if (overlaps(in, out, bsz * (int64_t(8) << n)))
    return fail(TQK_BAD_POINTER, "%s: input and output states overlap without being the same buffer", what);
  tc::TcParams p;
  p.psi = const_cast<float2*>(static_cast<const float2*>(in));
  p.psi_out = static_cast<float2*>(out);
  p.lam = nullptr;
  p.uimg = static_cast<const uint8_t*>(image);
  p.u_batch = u_batch;
  p.mr_out = nullptr;
  p.status = status;
  if ((rc = tc_setup(p, bsz, n, wires, false, what))) return rc;
  return tc_launch(p, false, stream, what);
}

}  // namespace

extern "C" int tqk_fused_adjoint(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires,
                                 const void* image_h, int64_t u_batch, double* mr_out, int* status, void* stream) {
  return adjoint_entry(psi, static_cast<float2*>(psi), lam, bsz, n, wires, image_h, u_batch, mr_out, status, stream,
                       "tqk_fused_adjoint");
}

extern "C" int tqk_fused_adjoint_stored(const void* psi_in, void* lam, int64_t bsz, int n, const int32_t* wires,
                                        const void* image_h, int64_t u_batch, double* mr_out, int* status,
                                        void* stream) {
  return adjoint_entry(psi_in, nullptr, lam, bsz, n, wires, image_h, u_batch, mr_out, status, stream,
                       "tqk_fused_adjoint_stored");
}

extern "C" int tqk_fused_apply(void* state, int64_t bsz, int n, const int32_t* wires, const void* image,
                               int64_t u_batch, int* status, void* stream) {
  return apply_entry(state, state, bsz, n, wires, image, u_batch, status, stream, "tqk_fused_apply");
}

extern "C" int tqk_fused_apply_to(const void* state_in, void* state_out, int64_t bsz, int n, const int32_t* wires,
                                  const void* image, int64_t u_batch, int* status, void* stream) {
  return apply_entry(state_in, state_out, bsz, n, wires, image, u_batch, status, stream, "tqk_fused_apply_to");
}
