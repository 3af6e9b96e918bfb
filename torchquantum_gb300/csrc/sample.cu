// sample.cu -- computational-basis sampling of a statevector on the GPU.
//
// Upstream's tq.measure copies |psi|^2 to the host and draws shots with
// random.choices (measurement/measurements.py:37-74).  Here each shot is an inverse-CDF
// draw on the device: given a uniform u in [0, 1), the outcome is the first index i
// whose running sum of |psi_j|^2 (j <= i) exceeds u * sum_j |psi_j|^2.  Three kernels:
//   k_tile_sums  one warp per tile of 2^tb amplitudes: the tile's probability (float64);
//   k_tile_scan  one block per row: inclusive prefix sums of the tile probabilities;
//   k_draw       one thread per (row, shot): binary search over the tile prefixes, then
//                a running sum over the chosen tile's amplitudes.
// Uniforms come from the caller (a seeded torch generator), so draws are reproducible.
#include <stdint.h>

#include "common.cuh"

namespace tqk {
namespace sample {

constexpr int kTileBits = 8;

__device__ __forceinline__ double prob(float2 a) { return (double)a.x * a.x + (double)a.y * a.y; }

// grid (ceil(ntiles / 8), bsz), 256 threads: warp w of the block sums tile 8 * blockIdx.x + w
__global__ void __launch_bounds__(256) k_tile_sums(const float2* state, int n, int tb, int64_t ntiles,
                                                   double* tile_sum) {
  const int64_t b = blockIdx.y;
  const int64_t tile = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (tile >= ntiles) return;
  const float2* src = state + (b << n) + (tile << tb);
  double s = 0.0;
  for (int j = lane; j < (1 << tb); j += 32) s += prob(src[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) tile_sum[b * ntiles + tile] = s;
}

// one block (1024 threads) per row: in-place inclusive scan in chunks of 1024
__global__ void __launch_bounds__(1024) k_tile_scan(double* tile_sum, int64_t ntiles) {
  __shared__ double buf[1024];
  __shared__ double carry;
  double* row = tile_sum + (int64_t)blockIdx.x * ntiles;
  if (threadIdx.x == 0) carry = 0.0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += 1024) {
    const int64_t i = base + threadIdx.x;
    buf[threadIdx.x] = i < ntiles ? row[i] : 0.0;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {  // Hillis-Steele scan
      const double v = threadIdx.x >= off ? buf[threadIdx.x - off] : 0.0;
      __syncthreads();
      buf[threadIdx.x] += v;
      __syncthreads();
    }
    if (i < ntiles) row[i] = buf[threadIdx.x] + carry;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_draw(const float2* state, int n, int tb, int64_t ntiles,
                                              const double* prefix, const double* uniforms, int64_t shots,
                                              int64_t* out) {
  const int64_t b = blockIdx.y;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= shots) return;
  const double* pre = prefix + b * ntiles;
  const double total = pre[ntiles - 1];
  const double target = uniforms[b * shots + s] * total;
  // first tile whose inclusive prefix exceeds target
  int64_t lo = 0, hi = ntiles - 1;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (pre[mid] > target) hi = mid;
    else lo = mid + 1;
  }
  const double before = lo > 0 ? pre[lo - 1] : 0.0;
  const float2* src = state + (b << n) + (lo << tb);
  double acc = before;
  int64_t pick = -1, last_nonzero = 0;
  for (int j = 0; j < (1 << tb); ++j) {
    const double p = prob(src[j]);
    if (p > 0.0) last_nonzero = j;
    acc += p;
    if (acc > target) {
      pick = j;
      break;
    }
  }
  if (pick < 0) pick = last_nonzero;  // rounding left target at the tile's end
  out[b * shots + s] = (lo << tb) + pick;
}

}  // namespace sample
}  // namespace tqk

using namespace tqk;

extern "C" int64_t tqk_sample_scratch_bytes(int64_t bsz, int n) {
  if (bsz < 1 || n < 1 || n > TQK_MAX_QUBITS) return 0;
  const int tb = n < sample::kTileBits ? n : sample::kTileBits;
  return bsz * (1ll << (n - tb)) * (int64_t)sizeof(double);
}

extern "C" int tqk_sample(const void* state, int64_t bsz, int n, const double* uniforms, int64_t shots,
                          int64_t* out, void* scratch, int64_t scratch_bytes, void* stream) {
  const char* what = "tqk_sample";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (shots < 0) return fail(TQK_BAD_SHAPE, "%s: shots %lld", what, (long long)shots);
  if (shots == 0) return TQK_OK;
  if (!uniforms || !out || !scratch) return fail(TQK_BAD_POINTER, "%s: null pointer", what);
  if (bsz > 65535) return fail(TQK_BAD_SHAPE, "%s: bsz %lld > 65535", what, (long long)bsz);
  if (shots > (1ll << 31) * 256) return fail(TQK_BAD_SHAPE, "%s: too many shots", what);
  if (scratch_bytes < tqk_sample_scratch_bytes(bsz, n))
    return fail(TQK_SCRATCH_TOO_SMALL, "%s: scratch %lld < %lld bytes", what, (long long)scratch_bytes,
                (long long)tqk_sample_scratch_bytes(bsz, n));
  const int tb = n < sample::kTileBits ? n : sample::kTileBits;
  const int64_t ntiles = 1ll << (n - tb);
  auto* st = static_cast<const float2*>(state);
  auto* pre = static_cast<double*>(scratch);
  cudaStream_t s = as_stream(stream);
  sample::k_tile_sums<<<dim3((unsigned)((ntiles + 7) / 8), (unsigned)bsz), 256, 0, s>>>(st, n, tb, ntiles, pre);
  sample::k_tile_scan<<<(unsigned)bsz, 1024, 0, s>>>(pre, ntiles);
  sample::k_draw<<<dim3((unsigned)((shots + 255) / 256), (unsigned)bsz), 256, 0, s>>>(st, n, tb, ntiles, pre,
                                                                                      uniforms, shots, out);
  return launch_status(what);
}
