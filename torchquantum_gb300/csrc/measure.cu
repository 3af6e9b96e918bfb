// measure.cu -- probabilities and Pauli-string expectation values.
//
// <psi|P|psi> for P = (x) sigma_w is evaluated from two bit masks over the in-row
// index: xmask (X or Y on the wire) and zmask (Z or Y), with
//   (P psi)_i = i^{#Y} (-1)^{popcount((i ^ x) & z)} psi_{i ^ x}.
// Strings with several xmasks on rows of up to 2^24 amplitudes are evaluated 8 at a
// time in one sweep of the rows through L2 (k_expval_rows: each amplitude's partners
// for all 8 strings, the rows in order so that DRAM reads the state once); otherwise
// strings that share an xmask are evaluated in one pass over the state (each amplitude
// pair (i, i^x) is read once for all of them).  Each thread accumulates in float32,
// blocks reduce in float64 and write one partial per (row, block, string) to scratch;
// a second kernel adds the partials in a fixed order, so results are bitwise
// reproducible run to run.  The backward seed sum_s c_s P_s psi (k_pauli_apply_sum)
// reads each output's partners for up to 64 strings in one pass.
#include <atomic>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace tqk {

constexpr int kMaxStringsPerPass = 8;
constexpr int kMaxApplyStrings = 64;
constexpr int kApplyChunk = 8;  // apply_sum partner loads issued together

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

// Strings with different X-masks in one launch, the rows swept one after another by the
// whole grid.  While a row of up to kRowsMaxAmps amplitudes is being swept it stays in L2,
// so the partner reads psi[i ^ x_s] of every string are served from L2 and each row is
// read from DRAM about once -- one pass per X-mask reads it once per mask.  Each thread
// takes the two amplitudes i, i + 1 and adds Re(conj(psi_j) (P_s psi)_j) for both:
//   (P psi)_j = i^ny (-1)^popcount((j ^ x) & z) psi_{j ^ x},
// with the sign of j = i + 1 that of j = i times (-1)^(z & 1), and Re(i^ny u) = u_r, -u_i,
// -u_r, u_i for ny = 0..3 (one popcount per string per thread).
constexpr int kRowsBlocks = 152 * 4;             // CTAs of the row sweep (partials per row)
constexpr int64_t kRowsMaxAmps = 1ll << 24;       // rows of up to 128 MB (about the L2)

struct RowsParams {
  const float2* state;
  int n;
  int ns;
  int64_t bsz;
  uint64_t x[kMaxStringsPerPass], z[kMaxStringsPerPass];
  int ny[kMaxStringsPerPass];
  double* partial;  // [bsz][gridDim.x][kMaxStringsPerPass]
};

template <int NS, typename I>
__global__ void __launch_bounds__(256) k_expval_rows(const RowsParams p) {
  I xs[NS], zs[NS];
  float z0[NS];
  uint32_t ny[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    xs[s] = s < p.ns ? static_cast<I>(p.x[s]) : I(0);
    zs[s] = s < p.ns ? static_cast<I>(p.z[s]) : I(0);
    z0[s] = (zs[s] & I(1)) ? -1.f : 1.f;
    ny[s] = s < p.ns ? static_cast<uint32_t>(p.ny[s]) : 0u;
  }
  const I half = static_cast<I>((1ll << p.n) >> 1);
  const I stride = static_cast<I>(gridDim.x * blockDim.x);
  for (int64_t b = 0; b < p.bsz; ++b) {
    const float2* row = p.state + (b << p.n);
    float acc[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) acc[s] = 0.f;
    for (I t = static_cast<I>(blockIdx.x * blockDim.x + threadIdx.x); t < half; t += stride) {
      const I i = t * 2;
      const float4 v = ld4(row + i);
      float4 w[NS];
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s < p.ns) w[s] = ld4(row + ((i ^ xs[s]) & ~I(1)));
      const float2 a0 = lo2(v), a1 = hi2(v);
#pragma unroll
      for (int s = 0; s < NS; ++s)
        if (s < p.ns) {
          const bool sw = (xs[s] & I(1)) != 0;
          const float2 b0 = sw ? hi2(w[s]) : lo2(w[s]), b1 = sw ? lo2(w[s]) : hi2(w[s]);
          const float ur = fmaf(z0[s], a1.x * b1.x + a1.y * b1.y, a0.x * b0.x + a0.y * b0.y);
          const float ui = fmaf(z0[s], a1.x * b1.y - a1.y * b1.x, a0.x * b0.y - a0.y * b0.x);
          const uint32_t neg = ((ny[s] + 1u) >> 1) & 1u;  // ny = 1, 2
          acc[s] += flip_if_odd((ny[s] & 1u) ? ui : ur, popc_t<I>((i ^ xs[s]) & zs[s]) + neg);
        }
    }
    block_reduce_store<NS>(acc, p.partial + (b * gridDim.x + blockIdx.x) * kMaxStringsPerPass, p.ns);
    __syncthreads();  // the reduction's shared buffer is reused for the next row
  }
}

// CTAs of the row sweep for rows of 2^n amplitudes (0: rows too long to stay in L2).
static int64_t rows_blocks(int n) {
  const int64_t amps = 1ll << n;
  if (amps > kRowsMaxAmps) return 0;
  const int64_t cap = (amps / 2 + 255) / 256;
  return cap < kRowsBlocks ? cap : kRowsBlocks;
}

// Launch with every CTA resident at once (a CTA of a second wave would start the first
// row after the others finished the last one); returns the grid size (partials per row).
template <int NS, typename I>
unsigned launch_rows_ns(const RowsParams& p, int64_t max_blocks, cudaStream_t st) {
  int dev = 0, sms = 0, fit = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k_expval_rows<NS, I>, 256, 0) != cudaSuccess || fit < 1)
    fit = 1;
  int64_t grid = static_cast<int64_t>(sms) * fit;
  if (grid > max_blocks) grid = max_blocks;
  k_expval_rows<NS, I><<<static_cast<unsigned>(grid), 256, 0, st>>>(p);
  return static_cast<unsigned>(grid);
}

template <typename I>
unsigned launch_rows(const RowsParams& p, int64_t max_blocks, cudaStream_t st) {
  if (p.ns <= 1) return launch_rows_ns<1, I>(p, max_blocks, st);
  if (p.ns <= 2) return launch_rows_ns<2, I>(p, max_blocks, st);
  if (p.ns <= 4) return launch_rows_ns<4, I>(p, max_blocks, st);
  return launch_rows_ns<8, I>(p, max_blocks, st);
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

struct ApplySumParams {
  const float2* state;
  float2* out;
  int n;
  int ns;
  uint64_t x[kMaxApplyStrings], z[kMaxApplyStrings];
  int ny[kMaxApplyStrings];
  const float* coef;  // [bsz][m] + col0
  int m, col0;
  int accumulate;
};

// out[i] (+)= sum_s c_s (P_s psi)[i], (P_s psi)[i] = i^ny (-1)^popcount((i ^ x) & z) psi[i ^ x]
// (the sign algebra above: one popcount per string for the two outputs of a thread).
template <typename I>
__global__ void __launch_bounds__(256) k_pauli_apply_sum(const ApplySumParams p) {
  const int64_t b = blockIdx.y;
  const I half = static_cast<I>((1ll << p.n) >> 1);
  const I t = static_cast<I>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= half) return;
  const float2* row = p.state + (b << p.n);
  float2* orow = p.out + (b << p.n);
  const I i = t * 2;
  float2 o0 = make_float2(0.f, 0.f), o1 = make_float2(0.f, 0.f);
  if (p.accumulate) {
    const float4 v = ld4(orow + i);
    o0 = lo2(v);
    o1 = hi2(v);
  }
  // partner loads of up to kApplyChunk strings issued together, then the arithmetic
  for (int s0 = 0; s0 < p.ns; s0 += kApplyChunk) {
    float4 w[kApplyChunk];
#pragma unroll
    for (int u = 0; u < kApplyChunk; ++u)
      if (s0 + u < p.ns) w[u] = ld4(row + ((i ^ static_cast<I>(p.x[s0 + u])) & ~I(1)));
#pragma unroll
    for (int u = 0; u < kApplyChunk; ++u) {
      const int s = s0 + u;
      if (s >= p.ns) break;
      const I x = static_cast<I>(p.x[s]), z = static_cast<I>(p.z[s]);
      const int ny = p.ny[s];
      const bool sw = (x & I(1)) != 0;
      const float2 src0 = sw ? hi2(w[u]) : lo2(w[u]), src1 = sw ? lo2(w[u]) : hi2(w[u]);
      // i^ny: a quarter turn for odd ny, a sign for ny >= 2 (folded into the parity)
      const float c0 = flip_if_odd(__ldg(p.coef + b * p.m + p.col0 + s),
                                   popc_t<I>((i ^ x) & z) + static_cast<uint32_t>(ny >> 1));
      const float c1 = (z & I(1)) ? -c0 : c0;
      if (ny & 1) {
        o0.x = fmaf(-c0, src0.y, o0.x);
        o0.y = fmaf(c0, src0.x, o0.y);
        o1.x = fmaf(-c1, src1.y, o1.x);
        o1.y = fmaf(c1, src1.x, o1.y);
      } else {
        o0.x = fmaf(c0, src0.x, o0.x);
        o0.y = fmaf(c0, src0.y, o0.y);
        o1.x = fmaf(c1, src1.x, o1.x);
        o1.y = fmaf(c1, src1.y, o1.y);
      }
    }
  }
  st4(orow + i, pack4(o0, o1));
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
  // partials [bsz][nblk][kMaxStringsPerPass] per pass (passes reuse the region; the
  // stream orders them)
  int64_t nblk = reduce_blocks_per_row(bsz, n);
  const int64_t rb = rows_blocks(n);  // the row sweep's partials, when it may be used
  if (rb > nblk) nblk = rb;
  (void)m;
  return bsz * nblk * kMaxStringsPerPass * (int64_t)sizeof(double);
}

extern "C" int tqk_pauli_expval(const void* state, int64_t bsz, int n, const uint64_t* xmask, const uint64_t* zmask,
                                int m, double* out, void* scratch, int64_t scratch_bytes, void* stream) {
  const char* what = "tqk_pauli_expval";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (m <= 0) return TQK_OK;
  if (!xmask || !zmask || !out) return fail(TQK_BAD_POINTER, "%s: null mask/output pointer", what);
  if (scratch == nullptr || scratch_bytes < tqk_pauli_expval_scratch_bytes(bsz, n, m))
    return fail(TQK_SCRATCH_TOO_SMALL, "%s: scratch of %lld bytes needed", what,
                (long long)tqk_pauli_expval_scratch_bytes(bsz, n, m));
  const uint64_t lim = n >= 64 ? ~0ull : ((1ull << n) - 1ull);
  for (int j = 0; j < m; ++j)
    if ((xmask[j] | zmask[j]) & ~lim) return fail(TQK_BAD_WIRES, "%s: string %d has bits beyond n_wires=%d", what, j, n);
  cudaStream_t st = as_stream(stream);
  const int64_t nblk = reduce_blocks_per_row(bsz, n);
  double* partial = static_cast<double*>(scratch);
  // several X-masks and rows that stay in L2: sweep the rows once per 8 strings
  const int64_t rb = rows_blocks(n);
  bool several = false;
  for (int j = 1; j < m && !several; ++j) several = xmask[j] != xmask[0];
  if (rb > 0 && several) {
    for (int j0 = 0; j0 < m; j0 += kMaxStringsPerPass) {
      RowsParams p;
      p.state = static_cast<const float2*>(state);
      p.n = n;
      p.bsz = bsz;
      p.partial = partial;
      p.ns = (m - j0) < kMaxStringsPerPass ? (m - j0) : kMaxStringsPerPass;
      FinishCols cols;
      for (int s = 0; s < kMaxStringsPerPass; ++s) {
        const bool on = s < p.ns;
        p.x[s] = on ? xmask[j0 + s] : 0;
        p.z[s] = on ? zmask[j0 + s] : 0;
        p.ny[s] = on ? __builtin_popcountll(xmask[j0 + s] & zmask[j0 + s]) & 3 : 0;
        cols.c[s] = on ? j0 + s : 0;
      }
      const unsigned grid = n <= 31 ? launch_rows<uint32_t>(p, rb, st) : launch_rows<uint64_t>(p, rb, st);
      if ((rc = launch_status(what))) return rc;
      k_expval_finish<<<(unsigned)bsz, kFinishThreads, 0, st>>>(partial, grid, p.ns, kMaxStringsPerPass,
                                                                        cols, m, out, bsz);
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
                                   const uint64_t* zmask, int m, const float* coef, void* out, void* stream) {
  const char* what = "tqk_pauli_apply_sum";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if ((rc = check_state(out, bsz, n, what))) return rc;
  if (m <= 0) return fail(TQK_BAD_SHAPE, "%s: need at least one string", what);
  if (!xmask || !zmask || !coef) return fail(TQK_BAD_POINTER, "%s: null pointer", what);
  cudaStream_t st = as_stream(stream);
  const int64_t half = (1ll << n) >> 1;
  for (int j0 = 0; j0 < m; j0 += kMaxApplyStrings) {
    ApplySumParams p;
    p.state = static_cast<const float2*>(state);
    p.out = static_cast<float2*>(out);
    p.n = n;
    p.ns = (m - j0) < kMaxApplyStrings ? (m - j0) : kMaxApplyStrings;
    for (int s = 0; s < p.ns; ++s) {
      p.x[s] = xmask[j0 + s];
      p.z[s] = zmask[j0 + s];
      p.ny[s] = __builtin_popcountll(xmask[j0 + s] & zmask[j0 + s]) & 3;
    }
    p.coef = coef;
    p.m = m;
    p.col0 = j0;
    p.accumulate = j0 > 0;
    const int threads = threads_for(half);
    dim3 grid((unsigned)((half + threads - 1) / threads), (unsigned)bsz, 1);
    if (n <= 31) k_pauli_apply_sum<uint32_t><<<grid, threads, 0, st>>>(p);
    else k_pauli_apply_sum<uint64_t><<<grid, threads, 0, st>>>(p);
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
