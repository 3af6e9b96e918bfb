// common.cuh -- shared device/host helpers of the statevector engine (sm_103a).
//
// Index scheme: a statevector row holds 2^n complex64 amplitudes; wire w is bit
// (n-1-w) of the in-row index (wire 0 = most significant).  A gate touching a set of
// m bit positions is applied over "groups": the group index g in [0, 2^(n-m)) is
// expanded to an amplitude base index by inserting a 0 at each touched position
// (ascending), then control bits are OR-ed in; the 2^k amplitudes of the group are
// base | (target-bit pattern).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/tqk.h"

namespace tqk {

constexpr int kMaxInsert = 16;  // touched bit positions per gate (targets + controls)

struct BitInsert {
  int m;                 // number of inserted zero bits
  int pos[kMaxInsert];   // ascending bit positions
};

__device__ __forceinline__ uint64_t insert_zero_bits(uint64_t g, const BitInsert& bi) {
#pragma unroll
  for (int i = 0; i < kMaxInsert; ++i) {
    if (i < bi.m) {
      const int q = bi.pos[i];
      const uint64_t lo = g & ((1ull << q) - 1ull);
      g = ((g >> q) << (q + 1)) | lo;
    }
  }
  return g;
}

// ------------------------------------------------------------------ complex helpers
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * b + c
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
// conj(a) * b + c
__device__ __forceinline__ float2 cfma_conj(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, c.y)));
}
// a * conj(b) + c
__device__ __forceinline__ float2 cfma_bconj(float2 a, float2 b, float2 c) {
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.y, b.x, fmaf(-a.x, b.y, c.y)));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }

// Default caching on purpose: states that fit in L2 stay resident across gates.
__device__ __forceinline__ float4 ld4(const float2* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float2* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 pack4(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }

// ------------------------------------------------------------------ block reductions
// Sum NV float accumulators of every thread of the block into NV doubles, then
// atomically add them to dst[0..NV) (one atomic per value per block).  Warp level in
// float32, block level in float64.  Block size must be a multiple of 32 and <= 1024.
template <int NV>
__device__ __forceinline__ void block_reduce_add(float (&v)[NV], double* dst) {
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
  if (warp == 0) {
    for (int j = lane; j < NV; j += 32) {
      double s = 0.0;
      for (int w = 0; w < nwarps; ++w) s += red[w][j];
      atomicAdd(dst + j, s);
    }
  }
}

// ------------------------------------------------------------------ host helpers
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int launch_status(const char* what);

// Validate wire indices: in range [0,n), no duplicates among the union of lists.
// Converts to bit positions (n-1-w).  Returns TQK_OK or an error (message set).
int wires_to_bits(int n, const int32_t* wires, int k, int* bits_out, uint64_t* used_mask,
                  const char* what);
int check_state(const void* state, int64_t bsz, int n, const char* what);
int check_batch(int64_t batch, int64_t bsz, const char* what);

// Sorted insertion table from a bit mask.
BitInsert make_insert(uint64_t mask);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Threads per block for a row of `work` items (multiple of 32, <= 256).
inline int threads_for(int64_t work) {
  int64_t t = work < 256 ? work : 256;
  t = (t + 31) / 32 * 32;
  return (int)(t < 32 ? 32 : t);
}

}  // namespace tqk
