// apply.cu -- plain (gate-by-gate) statevector kernels and their adjoint steps.
//
// Every kernel streams the amplitudes a gate touches exactly once (read + write),
// with 128-bit accesses wherever the index layout allows:
//   MODE_VEC  bit 0 is not touched by the gate: groups g and g+1 are adjacent in
//             memory, so each float4 carries the same offset of two groups;
//   MODE_LOW  bit 0 is a target: each float4 is the (bit0=0, bit0=1) amplitude pair
//             of one group;
//   MODE_SCL  bit 0 is a control: scalar float2 accesses (the touched amplitudes are
//             every other one, so sectors are fully used anyway).
// Grids are 2-D: blockIdx.y = batch row (the per-row operand is read once per block),
// blockIdx.x tiles the row's groups.
#include <stdio.h>

#include "common.cuh"

namespace tqk {

enum { MODE_SCL = 0, MODE_VEC = 1, MODE_LOW = 2 };

// ------------------------------------------------------------------ dense 1/2-target
template <int D>
struct DenseParams {
  float2* state;
  float2* lam;            // adjoint only
  int n;
  int64_t groups;         // groups per row
  BitInsert ins;          // all touched bits (targets + controls)
  uint64_t setmask;       // control bits forced to 1
  uint64_t off[D];        // target-bit pattern of matrix index r (wires[0] = MSB)
  int pair[D];            // MODE_LOW: index r' with off[r'] = off[r] | 1, or -1
  const float2* mat;      // [batch][D][D]
  int64_t mat_stride;     // D*D if per row else 0
  const float2* uinv;     // adjoint: exact inverse used to uncompute psi (non-unitary gates), or null
  double* grad;           // adjoint: [batch][D][D] complex128, or null
  int64_t grad_stride;    // 2*D*D if per row else 0
};

template <int D>
__device__ __forceinline__ void load_mat(const float2* m, float2 (&M)[D][D]) {
#pragma unroll
  for (int r = 0; r < D; ++r)
#pragma unroll
    for (int c = 0; c < D; ++c) M[r][c] = __ldg(m + r * D + c);
}

// y = M x
template <int D>
__device__ __forceinline__ void matvec(const float2 (&M)[D][D], const float2 (&x)[D], float2 (&y)[D]) {
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < D; ++c) acc = cfma(M[r][c], x[c], acc);
    y[r] = acc;
  }
}
// y = M^H x
template <int D>
__device__ __forceinline__ void matvec_h(const float2 (&M)[D][D], const float2 (&x)[D], float2 (&y)[D]) {
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
    for (int c = 0; c < D; ++c) acc = cfma_conj(M[c][r], x[c], acc);
    y[r] = acc;
  }
}

// Load / store the D amplitudes of NG groups starting at group g0 (NG = 2 for VEC/LOW
// pairs of groups, handled by the caller's loop).  a[j][r]: group j, matrix index r.
template <int D, int MODE>
__device__ __forceinline__ void load_groups(const float2* row, const DenseParams<D>& p, int64_t g0, bool two,
                                            float2 (&a)[2][D]) {
  if (MODE == MODE_VEC) {
    const uint64_t base = insert_zero_bits((uint64_t)g0, p.ins) | p.setmask;
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float4 v = ld4(row + (base + p.off[r]));
      a[0][r] = lo2(v);
      a[1][r] = hi2(v);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      if (j == 1 && !two) break;
      const uint64_t base = insert_zero_bits((uint64_t)(g0 + j), p.ins) | p.setmask;
      if (MODE == MODE_LOW) {
#pragma unroll
        for (int r = 0; r < D; ++r) {
          if (p.pair[r] >= 0) {
            float4 v = ld4(row + (base + p.off[r]));
            a[j][r] = lo2(v);
            a[j][p.pair[r]] = hi2(v);
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < D; ++r) a[j][r] = row[base + p.off[r]];
      }
    }
  }
}

template <int D, int MODE>
__device__ __forceinline__ void store_groups(float2* row, const DenseParams<D>& p, int64_t g0, bool two,
                                             const float2 (&a)[2][D]) {
  if (MODE == MODE_VEC) {
    const uint64_t base = insert_zero_bits((uint64_t)g0, p.ins) | p.setmask;
#pragma unroll
    for (int r = 0; r < D; ++r) st4(row + (base + p.off[r]), pack4(a[0][r], a[1][r]));
  } else {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      if (j == 1 && !two) break;
      const uint64_t base = insert_zero_bits((uint64_t)(g0 + j), p.ins) | p.setmask;
      if (MODE == MODE_LOW) {
#pragma unroll
        for (int r = 0; r < D; ++r)
          if (p.pair[r] >= 0) st4(row + (base + p.off[r]), pack4(a[j][r], a[j][p.pair[r]]));
      } else {
#pragma unroll
        for (int r = 0; r < D; ++r) row[base + p.off[r]] = a[j][r];
      }
    }
  }
}

template <int D, int MODE>
__global__ void __launch_bounds__(256) k_dense(const DenseParams<D> p) {
  const int64_t b = blockIdx.y;
  const int64_t pairs = (p.groups + 1) >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= pairs) return;
  float2 M[D][D];
  load_mat<D>(p.mat + b * p.mat_stride, M);
  float2* row = p.state + (b << p.n);
  const int64_t g0 = t * 2;
  const bool two = g0 + 1 < p.groups;
  float2 a[2][D], y[2][D];
  load_groups<D, MODE>(row, p, g0, two, a);
#pragma unroll
  for (int j = 0; j < 2; ++j) matvec<D>(M, a[j], y[j]);
  store_groups<D, MODE>(row, p, g0, two, y);
}

// Adjoint step: psi <- U^H psi (or U^-1 psi when INV), lam <- U^H lam,
// grad += lam_after (x) conj(psi_before).
template <int D, int MODE, bool GRAD, bool INV>
__global__ void __launch_bounds__(256) k_dense_adj(const DenseParams<D> p) {
  const int64_t b = blockIdx.y;
  const int64_t pairs = (p.groups + 1) >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float acc[GRAD ? 2 * D * D : 1];
#pragma unroll
  for (int i = 0; i < (GRAD ? 2 * D * D : 1); ++i) acc[i] = 0.f;
  if (t < pairs) {
    float2 M[D][D];
    load_mat<D>(p.mat + b * p.mat_stride, M);
    float2* prow = p.state + (b << p.n);
    float2* lrow = p.lam + (b << p.n);
    const int64_t g0 = t * 2;
    const bool two = g0 + 1 < p.groups;
    float2 a[2][D], l[2][D], y[2][D], z[2][D];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int r = 0; r < D; ++r) a[j][r] = l[j][r] = make_float2(0.f, 0.f);
    load_groups<D, MODE>(prow, p, g0, two, a);
    load_groups<D, MODE>(lrow, p, g0, two, l);
    if (INV) {
      float2 Mi[D][D];
      load_mat<D>(p.uinv + b * p.mat_stride, Mi);
#pragma unroll
      for (int j = 0; j < 2; ++j) matvec<D>(Mi, a[j], y[j]);
    } else {
#pragma unroll
      for (int j = 0; j < 2; ++j) matvec_h<D>(M, a[j], y[j]);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) matvec_h<D>(M, l[j], z[j]);
    if (GRAD) {
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int r = 0; r < D; ++r)
#pragma unroll
          for (int c = 0; c < D; ++c) {
            float2 v = cfma_bconj(l[j][r], y[j][c], make_float2(acc[2 * (r * D + c)], acc[2 * (r * D + c) + 1]));
            acc[2 * (r * D + c)] = v.x;
            acc[2 * (r * D + c) + 1] = v.y;
          }
    }
    store_groups<D, MODE>(prow, p, g0, two, y);
    store_groups<D, MODE>(lrow, p, g0, two, z);
  }
  if (GRAD) block_reduce_add<GRAD ? 2 * D * D : 1>(acc, p.grad + b * p.grad_stride);
}

// ------------------------------------------------------------------ generic dense k
// One block stages gpb groups (2^k amplitudes each) in shared memory, applies the
// matrix (staged in shared memory too when 2^k <= 64) and writes back.  Thread idx
// maps to (group gi = idx % gpb, row r = idx / gpb), so a warp shares its matrix row.
struct DenseKParams {
  float2* state;
  float2* lam;                      // adjoint only
  int n, k;
  int64_t groups;
  BitInsert ins;
  int tbits[TQK_MAX_DENSE_WIRES];   // bit of matrix-index bit j (j=0 is the MSB of r)
  const float2* mat;
  const float2* uinv;               // adjoint: exact inverse for psi, or null (use U^H)
  int64_t mat_stride;
  double* grad;                     // adjoint: [batch][D][D] complex128 or null
  int64_t grad_stride;
  int gpb;                          // groups per block
  int mat_in_smem;
};

__device__ __forceinline__ uint64_t dk_offset(const DenseKParams& p, int r) {
  uint64_t off = 0;
  for (int j = 0; j < p.k; ++j)
    if ((r >> (p.k - 1 - j)) & 1) off |= 1ull << p.tbits[j];
  return off;
}

constexpr int kDkMaxOut = 16;

// smem: [mat D*D if staged][tile gpb*(D+1)] (tile rows padded by one amplitude)
__global__ void __launch_bounds__(256) k_dense_k(const DenseKParams p) {
  extern __shared__ float2 sm[];
  const int D = 1 << p.k;
  const int ld = D + 1;
  const int64_t b = blockIdx.y;
  const int64_t gbase = (int64_t)blockIdx.x * p.gpb;
  float2* row = p.state + (b << p.n);
  const float2* Mg = p.mat + b * p.mat_stride;
  float2* Ms = sm;
  float2* tile = sm + (p.mat_in_smem ? D * D : 0);
  if (p.mat_in_smem)
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) Ms[i] = Mg[i];
  const float2* M = p.mat_in_smem ? Ms : Mg;
  const int total = p.gpb * D;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int gi = idx % p.gpb, r = idx / p.gpb;
    const int64_t g = gbase + gi;
    if (g < p.groups) tile[gi * ld + r] = row[insert_zero_bits((uint64_t)g, p.ins) + dk_offset(p, r)];
  }
  __syncthreads();
  float2 out[kDkMaxOut];
  int cnt = 0;
  for (int idx = threadIdx.x; idx < total && cnt < kDkMaxOut; idx += blockDim.x, ++cnt) {
    const int gi = idx % p.gpb, r = idx / p.gpb;
    float2 acc = make_float2(0.f, 0.f);
    const float2* mr = M + (int64_t)r * D;
    const float2* s = tile + gi * ld;
    for (int c = 0; c < D; ++c) acc = cfma(mr[c], s[c], acc);
    out[cnt] = acc;
  }
  __syncthreads();
  cnt = 0;
  for (int idx = threadIdx.x; idx < total && cnt < kDkMaxOut; idx += blockDim.x, ++cnt) {
    const int gi = idx % p.gpb, r = idx / p.gpb;
    const int64_t g = gbase + gi;
    if (g < p.groups) row[insert_zero_bits((uint64_t)g, p.ins) + dk_offset(p, r)] = out[cnt];
  }
}

// Adjoint of a dense k-wire gate: psi <- U^H psi (or U^-1 psi), lam <- U^H lam,
// grad[r][c] += sum over groups of lam_after[r] * conj(psi_before[c]).
// smem: [psi tile gpb*(D+1)][lam tile gpb*(D+1)]
__global__ void __launch_bounds__(256) k_dense_k_adj(const DenseKParams p) {
  extern __shared__ float2 sm[];
  const int D = 1 << p.k;
  const int ld = D + 1;
  const int64_t b = blockIdx.y;
  const int64_t gbase = (int64_t)blockIdx.x * p.gpb;
  float2* prow = p.state + (b << p.n);
  float2* lrow = p.lam + (b << p.n);
  const float2* M = p.mat + b * p.mat_stride;
  const float2* Mi = p.uinv ? p.uinv + b * p.mat_stride : nullptr;
  float2* ps = sm;
  float2* ls = sm + p.gpb * ld;
  const int total = p.gpb * D;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int gi = idx % p.gpb, r = idx / p.gpb;
    const int64_t g = gbase + gi;
    float2 a = make_float2(0.f, 0.f), l = make_float2(0.f, 0.f);
    if (g < p.groups) {
      const uint64_t ad = insert_zero_bits((uint64_t)g, p.ins) + dk_offset(p, r);
      a = prow[ad];
      l = lrow[ad];
    }
    ps[gi * ld + r] = a;
    ls[gi * ld + r] = l;
  }
  __syncthreads();
  float2 po[kDkMaxOut], lo[kDkMaxOut];
  int cnt = 0;
  for (int idx = threadIdx.x; idx < total && cnt < kDkMaxOut; idx += blockDim.x, ++cnt) {
    const int gi = idx % p.gpb, r = idx / p.gpb;
    float2 ap = make_float2(0.f, 0.f), al = make_float2(0.f, 0.f);
    const float2* s = ps + gi * ld;
    const float2* t = ls + gi * ld;
    for (int c = 0; c < D; ++c) {
      const float2 m = __ldg(M + (int64_t)c * D + r);  // (U^H)[r][c] = conj(U[c][r])
      al = cfma_conj(m, t[c], al);
      if (Mi) ap = cfma(__ldg(Mi + (int64_t)r * D + c), s[c], ap);
      else ap = cfma_conj(m, s[c], ap);
    }
    po[cnt] = ap;
    lo[cnt] = al;
  }
  __syncthreads();
  // psi_before into the psi tile (lam tile keeps lam_after for the gradient)
  cnt = 0;
  for (int idx = threadIdx.x; idx < total && cnt < kDkMaxOut; idx += blockDim.x, ++cnt) {
    const int gi = idx % p.gpb, r = idx / p.gpb;
    ps[gi * ld + r] = po[cnt];
    const int64_t g = gbase + gi;
    if (g < p.groups) {
      const uint64_t ad = insert_zero_bits((uint64_t)g, p.ins) + dk_offset(p, r);
      prow[ad] = po[cnt];
      lrow[ad] = lo[cnt];
    }
  }
  if (p.grad == nullptr) return;
  __syncthreads();
  double* gd = p.grad + b * p.grad_stride;
  for (int e = threadIdx.x; e < D * D; e += blockDim.x) {
    const int r = e / D, c = e % D;
    float2 acc = make_float2(0.f, 0.f);
    for (int gi = 0; gi < p.gpb; ++gi) acc = cfma_bconj(ls[gi * ld + r], ps[gi * ld + c], acc);
    atomicAdd(gd + 2 * e, (double)acc.x);
    atomicAdd(gd + 2 * e + 1, (double)acc.y);
  }
}

// ------------------------------------------------------------------ controlled X
struct XParams {
  float2* state;
  int n;
  int64_t groups;
  BitInsert ins;
  uint64_t setmask, tbit;
};

// Touched-subset kernels (controlled X, swap, phase) move few bytes per unit, so each
// thread takes kUnits units (block-strided, so every unit index stays coalesced) and
// issues all its loads before its stores: more bytes in flight per SM.
constexpr int kUnits = 4;

template <int MODE>
__global__ void __launch_bounds__(256) k_mcx(const XParams p) {
  const int64_t b = blockIdx.y;
  float2* row = p.state + (b << p.n);
  const int64_t units = MODE == MODE_VEC ? (p.groups + 1) >> 1 : p.groups;
  int64_t u[kUnits];
#pragma unroll
  for (int r = 0; r < kUnits; ++r) u[r] = ((int64_t)blockIdx.x * kUnits + r) * blockDim.x + threadIdx.x;
  if (MODE == MODE_VEC) {  // two adjacent groups per unit
    float4 a[kUnits], c[kUnits];
    uint64_t i0[kUnits];
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      i0[r] = insert_zero_bits((uint64_t)(u[r] * 2), p.ins) | p.setmask;
      a[r] = ld4(row + i0[r]);
      c[r] = ld4(row + (i0[r] | p.tbit));
    }
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      st4(row + i0[r], c[r]);
      st4(row + (i0[r] | p.tbit), a[r]);
    }
  } else if (MODE == MODE_LOW) {  // target is bit 0: swap the lanes of one float4
    float4 a[kUnits];
    uint64_t i0[kUnits];
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      i0[r] = insert_zero_bits((uint64_t)u[r], p.ins) | p.setmask;
      a[r] = ld4(row + i0[r]);
    }
#pragma unroll
    for (int r = 0; r < kUnits; ++r)
      if (u[r] < units) st4(row + i0[r], make_float4(a[r].z, a[r].w, a[r].x, a[r].y));
  } else {
    float2 a[kUnits], c[kUnits];
    uint64_t i0[kUnits];
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      i0[r] = insert_zero_bits((uint64_t)u[r], p.ins) | p.setmask;
      a[r] = row[i0[r]];
      c[r] = row[i0[r] | p.tbit];
    }
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      row[i0[r]] = c[r];
      row[i0[r] | p.tbit] = a[r];
    }
  }
}

// ------------------------------------------------------------------ swap
struct SwapParams {
  float2* state;
  int n;
  int64_t groups;
  BitInsert ins;
  uint64_t setmask, b0, b1;  // exchange base|b1 <-> base|b0
};

template <bool VEC>
__global__ void __launch_bounds__(256) k_swap(const SwapParams p) {
  const int64_t b = blockIdx.y;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float2* row = p.state + (b << p.n);
  if (VEC) {
    if (t * 2 >= p.groups) return;
    const uint64_t base = insert_zero_bits((uint64_t)(t * 2), p.ins) | p.setmask;
    float4 x = ld4(row + (base | p.b1)), y = ld4(row + (base | p.b0));
    st4(row + (base | p.b1), y);
    st4(row + (base | p.b0), x);
  } else {
    if (t >= p.groups) return;
    const uint64_t base = insert_zero_bits((uint64_t)t, p.ins) | p.setmask;
    float2 x = row[base | p.b1], y = row[base | p.b0];
    row[base | p.b1] = y;
    row[base | p.b0] = x;
  }
}

// ------------------------------------------------------------------ phase
struct PhaseParams {
  float2* state;
  float2* lam;
  int n;
  int64_t groups;
  BitInsert ins;
  uint64_t setmask;
  const float2* phase;
  int64_t phase_stride;  // 1 if per row else 0
  double* grad;
  int64_t grad_stride;   // 2 if per row else 0
};

template <bool VEC>
__global__ void __launch_bounds__(256) k_phase(const PhaseParams p) {
  const int64_t b = blockIdx.y;
  const float2 ph = __ldg(p.phase + b * p.phase_stride);
  float2* row = p.state + (b << p.n);
  const int64_t units = VEC ? (p.groups + 1) >> 1 : p.groups;
  int64_t u[kUnits];
#pragma unroll
  for (int r = 0; r < kUnits; ++r) u[r] = ((int64_t)blockIdx.x * kUnits + r) * blockDim.x + threadIdx.x;
  if (VEC) {
    float4 a[kUnits];
    uint64_t i0[kUnits];
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      i0[r] = insert_zero_bits((uint64_t)(u[r] * 2), p.ins) | p.setmask;
      a[r] = ld4(row + i0[r]);
    }
#pragma unroll
    for (int r = 0; r < kUnits; ++r)
      if (u[r] < units) st4(row + i0[r], pack4(cmul(ph, lo2(a[r])), cmul(ph, hi2(a[r]))));
  } else {
    float2 a[kUnits];
    uint64_t i0[kUnits];
#pragma unroll
    for (int r = 0; r < kUnits; ++r) {
      if (u[r] >= units) continue;
      i0[r] = insert_zero_bits((uint64_t)u[r], p.ins) | p.setmask;
      a[r] = row[i0[r]];
    }
#pragma unroll
    for (int r = 0; r < kUnits; ++r)
      if (u[r] < units) row[i0[r]] = cmul(ph, a[r]);
  }
}

template <bool VEC, bool GRAD>
__global__ void __launch_bounds__(256) k_phase_adj(const PhaseParams p) {
  const int64_t b = blockIdx.y;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float2 phc = cconj(__ldg(p.phase + b * p.phase_stride));
  float2* prow = p.state + (b << p.n);
  float2* lrow = p.lam + (b << p.n);
  float acc[2] = {0.f, 0.f};
  if (VEC) {
    if (t * 2 < p.groups) {
      const uint64_t i0 = insert_zero_bits((uint64_t)(t * 2), p.ins) | p.setmask;
      float4 a = ld4(prow + i0), l = ld4(lrow + i0);
      float2 y0 = cmul(phc, lo2(a)), y1 = cmul(phc, hi2(a));
      if (GRAD) {
        float2 g = cfma_bconj(lo2(l), y0, make_float2(0.f, 0.f));
        g = cfma_bconj(hi2(l), y1, g);
        acc[0] = g.x;
        acc[1] = g.y;
      }
      st4(prow + i0, pack4(y0, y1));
      st4(lrow + i0, pack4(cmul(phc, lo2(l)), cmul(phc, hi2(l))));
    }
  } else {
    if (t < p.groups) {
      const uint64_t i0 = insert_zero_bits((uint64_t)t, p.ins) | p.setmask;
      float2 y = cmul(phc, prow[i0]), l = lrow[i0];
      if (GRAD) {
        float2 g = cfma_bconj(l, y, make_float2(0.f, 0.f));
        acc[0] = g.x;
        acc[1] = g.y;
      }
      prow[i0] = y;
      lrow[i0] = cmul(phc, l);
    }
  }
  if (GRAD) block_reduce_add<2>(acc, p.grad + b * p.grad_stride);
}

// ------------------------------------------------------------------ diagonal
template <int K>
struct DiagParams {
  float2* state;
  float2* lam;
  int n;
  int64_t half;          // amplitudes per row / 2
  int bits[K];           // bit of diag-index bit j (j=0 is the MSB)
  const float2* diag;    // [batch][2^K]
  int64_t diag_stride;
  double* grad;
  int64_t grad_stride;   // 2*2^K if per row else 0
};

template <int K>
__device__ __forceinline__ int diag_index(const DiagParams<K>& p, uint64_t i) {
  int d = 0;
#pragma unroll
  for (int j = 0; j < K; ++j) d = (d << 1) | (int)((i >> p.bits[j]) & 1ull);
  return d;
}

template <int K>
__global__ void __launch_bounds__(256) k_diag(const DiagParams<K> p) {
  const int64_t b = blockIdx.y;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.half) return;
  constexpr int DD = 1 << K;
  float2 dv[DD];
#pragma unroll
  for (int j = 0; j < DD; ++j) dv[j] = __ldg(p.diag + b * p.diag_stride + j);
  float2* row = p.state + (b << p.n);
  const uint64_t i0 = (uint64_t)t * 2;
  float4 a = ld4(row + i0);
  st4(row + i0, pack4(cmul(dv[diag_index<K>(p, i0)], lo2(a)), cmul(dv[diag_index<K>(p, i0 + 1)], hi2(a))));
}

template <int K, bool GRAD>
__global__ void __launch_bounds__(256) k_diag_adj(const DiagParams<K> p) {
  constexpr int DD = 1 << K;
  const int64_t b = blockIdx.y;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float acc[GRAD ? 2 * DD : 1];
#pragma unroll
  for (int j = 0; j < (GRAD ? 2 * DD : 1); ++j) acc[j] = 0.f;
  if (t < p.half) {
    float2 dv[DD];
#pragma unroll
    for (int j = 0; j < DD; ++j) dv[j] = cconj(__ldg(p.diag + b * p.diag_stride + j));
    float2* prow = p.state + (b << p.n);
    float2* lrow = p.lam + (b << p.n);
    const uint64_t i0 = (uint64_t)t * 2;
    const int d0 = diag_index<K>(p, i0), d1 = diag_index<K>(p, i0 + 1);
    float4 a = ld4(prow + i0), l = ld4(lrow + i0);
    float2 y0 = cmul(dv[d0], lo2(a)), y1 = cmul(dv[d1], hi2(a));
    if (GRAD) {
#pragma unroll
      for (int j = 0; j < DD; ++j) {
        float2 g = make_float2(acc[2 * j], acc[2 * j + 1]);
        if (j == d0) g = cfma_bconj(lo2(l), y0, g);
        if (j == d1) g = cfma_bconj(hi2(l), y1, g);
        acc[2 * j] = g.x;
        acc[2 * j + 1] = g.y;
      }
    }
    st4(prow + i0, pack4(y0, y1));
    st4(lrow + i0, pack4(cmul(dv[d0], lo2(l)), cmul(dv[d1], hi2(l))));
  }
  if (GRAD) block_reduce_add<GRAD ? 2 * DD : 1>(acc, p.grad + b * p.grad_stride);
}

// ------------------------------------------------------------------ reset
__global__ void k_reset_zero(float2* state, int n, uint64_t mask, double* norm2) {
  const int64_t b = blockIdx.y;
  const int64_t half = (1ll << n) >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float acc[1] = {0.f};
  if (t < half) {
    float2* row = state + (b << n);
    const uint64_t i0 = (uint64_t)t * 2;
    float4 a = ld4(row + i0);
    if ((i0 & mask) != 0) a.x = a.y = 0.f;
    if (((i0 + 1) & mask) != 0) a.z = a.w = 0.f;
    acc[0] = a.x * a.x + a.y * a.y + a.z * a.z + a.w * a.w;
    st4(row + i0, a);
  }
  block_reduce_add<1>(acc, norm2 + b);
}

__global__ void k_reset_scale(float2* state, int n, const double* norm2) {
  const int64_t b = blockIdx.y;
  const int64_t half = (1ll << n) >> 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= half) return;
  float2* row = state + (b << n);
  const double nn = norm2[b];
  const uint64_t i0 = (uint64_t)t * 2;
  if (nn == 0.0) {  // functional/reset.py via normalize_statevector: an all-zero row becomes |0..0>
    if (i0 == 0) row[0] = make_float2(1.f, 0.f);
    return;
  }
  const float s = (float)(1.0 / sqrt(nn));
  float4 a = ld4(row + i0);
  st4(row + i0, make_float4(a.x * s, a.y * s, a.z * s, a.w * s));
}

// ================================================================== host side
namespace {

struct GateSetup {
  int n;
  int64_t bsz;
  uint64_t touched = 0;  // all bits touched
  uint64_t ctrl = 0;     // control bits
  int tb[TQK_MAX_DENSE_WIRES];
  int kt = 0;
};

inline dim3 grid_for(int64_t work, int threads, int64_t bsz) {
  return dim3((unsigned)((work + threads - 1) / threads), (unsigned)bsz, 1);
}

template <int D>
int fill_dense(DenseParams<D>& p, const GateSetup& s, int& mode) {
  p.n = s.n;
  const int m = __builtin_popcountll(s.touched);
  p.groups = 1ll << (s.n - m);
  p.ins = make_insert(s.touched);
  p.setmask = s.ctrl;
  for (int r = 0; r < D; ++r) {
    uint64_t off = 0;
    for (int j = 0; j < s.kt; ++j)
      if ((r >> (s.kt - 1 - j)) & 1) off |= 1ull << s.tb[j];
    p.off[r] = off;
  }
  const bool bit0_target = (s.touched & 1ull) && !(s.ctrl & 1ull);
  const bool bit0_ctrl = (s.ctrl & 1ull) != 0;
  mode = bit0_ctrl ? MODE_SCL : (bit0_target ? MODE_LOW : MODE_VEC);
  for (int r = 0; r < D; ++r) {
    p.pair[r] = -1;
    if (mode == MODE_LOW && (p.off[r] & 1ull) == 0)
      for (int r2 = 0; r2 < D; ++r2)
        if (p.off[r2] == (p.off[r] | 1ull)) p.pair[r] = r2;
  }
  return TQK_OK;
}

template <int D, bool INV>
void launch_dense_adj(const DenseParams<D>& p, int mode, bool grad, dim3 grid, int threads, cudaStream_t st) {
  if (grad) {
    if (mode == MODE_VEC) k_dense_adj<D, MODE_VEC, true, INV><<<grid, threads, 0, st>>>(p);
    else if (mode == MODE_LOW) k_dense_adj<D, MODE_LOW, true, INV><<<grid, threads, 0, st>>>(p);
    else k_dense_adj<D, MODE_SCL, true, INV><<<grid, threads, 0, st>>>(p);
  } else {
    if (mode == MODE_VEC) k_dense_adj<D, MODE_VEC, false, INV><<<grid, threads, 0, st>>>(p);
    else if (mode == MODE_LOW) k_dense_adj<D, MODE_LOW, false, INV><<<grid, threads, 0, st>>>(p);
    else k_dense_adj<D, MODE_SCL, false, INV><<<grid, threads, 0, st>>>(p);
  }
}

template <int D>
int launch_dense(const GateSetup& s, float2* state, float2* lam, const float2* mat, int64_t mat_batch,
                 const float2* uinv, double* grad, bool adjoint, cudaStream_t st) {
  DenseParams<D> p;
  int mode;
  fill_dense<D>(p, s, mode);
  p.state = state;
  p.lam = lam;
  p.mat = mat;
  p.mat_stride = mat_batch > 1 ? D * D : 0;
  p.uinv = uinv;
  p.grad = grad;
  p.grad_stride = mat_batch > 1 ? 2 * D * D : 0;
  const int64_t work = (p.groups + 1) >> 1;
  const int threads = threads_for(work);
  dim3 grid = grid_for(work, threads, s.bsz);
  if (!adjoint) {
    if (mode == MODE_VEC) k_dense<D, MODE_VEC><<<grid, threads, 0, st>>>(p);
    else if (mode == MODE_LOW) k_dense<D, MODE_LOW><<<grid, threads, 0, st>>>(p);
    else k_dense<D, MODE_SCL><<<grid, threads, 0, st>>>(p);
  } else if (uinv) {
    launch_dense_adj<D, true>(p, mode, grad != nullptr, grid, threads, st);
  } else {
    launch_dense_adj<D, false>(p, mode, grad != nullptr, grid, threads, st);
  }
  return launch_status(adjoint ? "adjoint dense gate" : "dense gate");
}

int launch_dense_k(const GateSetup& s, float2* state, float2* lam, const float2* mat, const float2* uinv,
                   int64_t mat_batch, double* grad, bool adjoint, cudaStream_t st) {
  DenseKParams p;
  p.state = state;
  p.lam = lam;
  p.n = s.n;
  p.k = s.kt;
  const int m = __builtin_popcountll(s.touched);
  p.groups = 1ll << (s.n - m);
  p.ins = make_insert(s.touched);
  for (int j = 0; j < s.kt; ++j) p.tbits[j] = s.tb[j];
  const int D = 1 << s.kt;
  p.mat = mat;
  p.uinv = uinv;
  p.mat_stride = mat_batch > 1 ? (int64_t)D * D : 0;
  p.grad = grad;
  p.grad_stride = mat_batch > 1 ? 2ll * D * D : 0;
  const int threads = 256;
  // groups per block: up to 32 for narrow gates, bounded by 16 outputs per thread
  int gpb = 32;
  while (gpb > 1 && (int64_t)gpb * D > kDkMaxOut * threads) gpb >>= 1;
  if (gpb > p.groups) gpb = (int)p.groups;
  p.gpb = gpb;
  p.mat_in_smem = (!adjoint && D <= 64) ? 1 : 0;
  const size_t tile = (size_t)gpb * (D + 1) * sizeof(float2);
  const size_t smem = adjoint ? 2 * tile : tile + (p.mat_in_smem ? (size_t)D * D * sizeof(float2) : 0);
  if (smem > 200 * 1024) return fail(TQK_TOO_MANY_QUBITS, "dense gate: k=%d too wide", s.kt);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_dense_k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_dense_k_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr_set = true;
  }
  dim3 grid((unsigned)((p.groups + gpb - 1) / gpb), (unsigned)s.bsz, 1);
  if (adjoint) k_dense_k_adj<<<grid, threads, smem, st>>>(p);
  else k_dense_k<<<grid, threads, smem, st>>>(p);
  return launch_status(adjoint ? "adjoint dense k-wire gate" : "dense k-wire gate");
}

int setup_targets(GateSetup& s, int n, int64_t bsz, const int32_t* targets, int kt, const int32_t* controls,
                  int nc, const char* what) {
  s.n = n;
  s.bsz = bsz;
  s.kt = kt;
  if (nc < 0 || kt < 0 || nc + kt > kMaxInsert || nc + kt > n)
    return fail(TQK_BAD_WIRES, "%s: %d targets + %d controls invalid for n_wires=%d", what, kt, nc, n);
  int rc = wires_to_bits(n, targets, kt, s.tb, &s.touched, what);
  if (rc) return rc;
  int cb[kMaxInsert];
  rc = wires_to_bits(n, controls, nc, cb, &s.touched, what);
  if (rc) return rc;
  for (int i = 0; i < nc; ++i) s.ctrl |= 1ull << cb[i];
  return TQK_OK;
}

int dense_entry(void* state, void* lam, int64_t bsz, int n, const int32_t* controls, int nc,
                const int32_t* targets, int kt, const void* mat, int64_t mat_batch, const void* uinv,
                double* grad, bool adjoint, void* stream, const char* what) {
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (adjoint && (rc = check_state(lam, bsz, n, what))) return rc;
  if ((rc = check_batch(mat_batch, bsz, what))) return rc;
  if (mat == nullptr) return fail(TQK_BAD_POINTER, "%s: null matrix", what);
  if (kt < 1 || kt > TQK_MAX_DENSE_WIRES) return fail(TQK_TOO_MANY_QUBITS, "%s: k=%d unsupported", what, kt);
  GateSetup s;
  if ((rc = setup_targets(s, n, bsz, targets, kt, controls, nc, what))) return rc;
  cudaStream_t st = as_stream(stream);
  auto* ps = static_cast<float2*>(state);
  auto* pl = static_cast<float2*>(lam);
  auto* pm = static_cast<const float2*>(mat);
  auto* pi = static_cast<const float2*>(uinv);
  if (kt == 1) return launch_dense<2>(s, ps, pl, pm, mat_batch, pi, grad, adjoint, st);
  if (kt == 2) return launch_dense<4>(s, ps, pl, pm, mat_batch, pi, grad, adjoint, st);
  if (nc > 0) return fail(TQK_UNSUPPORTED, "%s: controlled gates take 1 or 2 targets", what);
  return launch_dense_k(s, ps, pl, pm, pi, mat_batch, grad, adjoint, st);
}

int phase_entry(void* state, void* lam, int64_t bsz, int n, const int32_t* wires, int k, const void* phase,
                int64_t phase_batch, double* grad, bool adjoint, void* stream, const char* what) {
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (adjoint && (rc = check_state(lam, bsz, n, what))) return rc;
  if ((rc = check_batch(phase_batch, bsz, what))) return rc;
  if (phase == nullptr) return fail(TQK_BAD_POINTER, "%s: null phase", what);
  GateSetup s;
  if ((rc = setup_targets(s, n, bsz, nullptr, 0, wires, k, what))) return rc;
  PhaseParams p;
  p.state = static_cast<float2*>(state);
  p.lam = static_cast<float2*>(lam);
  p.n = n;
  p.groups = 1ll << (n - k);
  p.ins = make_insert(s.touched);
  p.setmask = s.touched;
  p.phase = static_cast<const float2*>(phase);
  p.phase_stride = phase_batch > 1 ? 1 : 0;
  p.grad = grad;
  p.grad_stride = phase_batch > 1 ? 2 : 0;
  const bool vec = (s.touched & 1ull) == 0;
  const int64_t work = vec ? p.groups / 2 : p.groups;
  const int threads = threads_for(work);
  dim3 grid = grid_for(work, threads, bsz);
  cudaStream_t st = as_stream(stream);
  if (!adjoint) {
    const dim3 gridu = grid_for(work, threads * kUnits, bsz);  // kUnits units per thread
    if (vec) k_phase<true><<<gridu, threads, 0, st>>>(p);
    else k_phase<false><<<gridu, threads, 0, st>>>(p);
  } else if (grad) {
    if (vec) k_phase_adj<true, true><<<grid, threads, 0, st>>>(p);
    else k_phase_adj<false, true><<<grid, threads, 0, st>>>(p);
  } else {
    if (vec) k_phase_adj<true, false><<<grid, threads, 0, st>>>(p);
    else k_phase_adj<false, false><<<grid, threads, 0, st>>>(p);
  }
  return launch_status(what);
}

template <int K>
int launch_diag(int64_t bsz, int n, const int* bits, float2* state, float2* lam, const float2* diag,
                int64_t diag_batch, double* grad, bool adjoint, cudaStream_t st) {
  DiagParams<K> p;
  p.state = state;
  p.lam = lam;
  p.n = n;
  p.half = (1ll << n) >> 1;
  for (int j = 0; j < K; ++j) p.bits[j] = bits[j];
  p.diag = diag;
  p.diag_stride = diag_batch > 1 ? (1 << K) : 0;
  p.grad = grad;
  p.grad_stride = diag_batch > 1 ? 2 * (1 << K) : 0;
  const int threads = threads_for(p.half);
  dim3 grid = grid_for(p.half, threads, bsz);
  if (!adjoint) k_diag<K><<<grid, threads, 0, st>>>(p);
  else if (grad) k_diag_adj<K, true><<<grid, threads, 0, st>>>(p);
  else k_diag_adj<K, false><<<grid, threads, 0, st>>>(p);
  return launch_status("diagonal gate");
}

int diag_entry(void* state, void* lam, int64_t bsz, int n, const int32_t* wires, int k, const void* diag,
               int64_t diag_batch, double* grad, bool adjoint, void* stream, const char* what) {
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (adjoint && (rc = check_state(lam, bsz, n, what))) return rc;
  if ((rc = check_batch(diag_batch, bsz, what))) return rc;
  if (diag == nullptr) return fail(TQK_BAD_POINTER, "%s: null diagonal", what);
  if (k < 1 || k > 4) return fail(TQK_UNSUPPORTED, "%s: k=%d (1..4 supported; wider diagonals go dense)", what, k);
  GateSetup s;
  if ((rc = setup_targets(s, n, bsz, wires, k, nullptr, 0, what))) return rc;
  auto* ps = static_cast<float2*>(state);
  auto* pl = static_cast<float2*>(lam);
  auto* pd = static_cast<const float2*>(diag);
  cudaStream_t st = as_stream(stream);
  switch (k) {
    case 1: return launch_diag<1>(bsz, n, s.tb, ps, pl, pd, diag_batch, grad, adjoint, st);
    case 2: return launch_diag<2>(bsz, n, s.tb, ps, pl, pd, diag_batch, grad, adjoint, st);
    case 3: return launch_diag<3>(bsz, n, s.tb, ps, pl, pd, diag_batch, grad, adjoint, st);
    default: return launch_diag<4>(bsz, n, s.tb, ps, pl, pd, diag_batch, grad, adjoint, st);
  }
}

}  // namespace
}  // namespace tqk

using namespace tqk;

extern "C" int tqk_apply_matrix(void* state, int64_t bsz, int n, const int32_t* wires, int k, const void* mat,
                                int64_t mat_batch, void* stream) {
  return dense_entry(state, nullptr, bsz, n, nullptr, 0, wires, k, mat, mat_batch, nullptr, nullptr, false, stream,
                     "tqk_apply_matrix");
}

extern "C" int tqk_apply_controlled(void* state, int64_t bsz, int n, const int32_t* controls, int nc,
                                    const int32_t* targets, int kt, const void* mat, int64_t mat_batch,
                                    void* stream) {
  if (kt != 1 && kt != 2) return fail(TQK_UNSUPPORTED, "tqk_apply_controlled: kt=%d must be 1 or 2", kt);
  return dense_entry(state, nullptr, bsz, n, controls, nc, targets, kt, mat, mat_batch, nullptr, nullptr, false,
                     stream, "tqk_apply_controlled");
}

extern "C" int tqk_adjoint_matrix(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires, int k,
                                  const void* mat, int64_t mat_batch, const void* uncompute, double* grad,
                                  void* stream) {
  return dense_entry(psi, lam, bsz, n, nullptr, 0, wires, k, mat, mat_batch, uncompute, grad, true, stream,
                     "tqk_adjoint_matrix");
}

extern "C" int tqk_adjoint_controlled(void* psi, void* lam, int64_t bsz, int n, const int32_t* controls, int nc,
                                      const int32_t* targets, int kt, const void* mat, int64_t mat_batch,
                                      const void* uncompute, double* grad, void* stream) {
  if (kt != 1 && kt != 2) return fail(TQK_UNSUPPORTED, "tqk_adjoint_controlled: kt=%d must be 1 or 2", kt);
  return dense_entry(psi, lam, bsz, n, controls, nc, targets, kt, mat, mat_batch, uncompute, grad, true, stream,
                     "tqk_adjoint_controlled");
}

extern "C" int tqk_apply_mcx(void* state, int64_t bsz, int n, const int32_t* controls, int nc, int ctrl_val,
                             int target, void* stream) {
  const char* what = "tqk_apply_mcx";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  GateSetup s;
  int32_t t = target;
  if ((rc = setup_targets(s, n, bsz, &t, 1, controls, nc, what))) return rc;
  XParams p;
  p.state = static_cast<float2*>(state);
  p.n = n;
  p.groups = 1ll << (n - nc - 1);
  p.ins = make_insert(s.touched);
  p.setmask = ctrl_val ? s.ctrl : 0ull;
  p.tbit = 1ull << s.tb[0];
  const bool bit0_ctrl = (s.ctrl & 1ull) != 0;
  const bool bit0_tgt = (p.tbit & 1ull) != 0;
  const int mode = bit0_ctrl ? MODE_SCL : (bit0_tgt ? MODE_LOW : MODE_VEC);
  const int64_t work = mode == MODE_VEC ? p.groups / 2 : p.groups;
  const int threads = threads_for(work);
  dim3 grid = grid_for(work, threads * kUnits, bsz);  // kUnits units per thread
  cudaStream_t st = as_stream(stream);
  if (mode == MODE_VEC) k_mcx<MODE_VEC><<<grid, threads, 0, st>>>(p);
  else if (mode == MODE_LOW) k_mcx<MODE_LOW><<<grid, threads, 0, st>>>(p);
  else k_mcx<MODE_SCL><<<grid, threads, 0, st>>>(p);
  return launch_status(what);
}

extern "C" int tqk_apply_swap(void* state, int64_t bsz, int n, const int32_t* controls, int nc, int w0, int w1,
                              void* stream) {
  const char* what = "tqk_apply_swap";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  GateSetup s;
  int32_t tw[2] = {w0, w1};
  if ((rc = setup_targets(s, n, bsz, tw, 2, controls, nc, what))) return rc;
  SwapParams p;
  p.state = static_cast<float2*>(state);
  p.n = n;
  p.groups = 1ll << (n - nc - 2);
  p.ins = make_insert(s.touched);
  p.setmask = s.ctrl;
  p.b0 = 1ull << s.tb[0];
  p.b1 = 1ull << s.tb[1];
  const bool vec = (s.touched & 1ull) == 0;
  const int64_t work = vec ? p.groups / 2 : p.groups;
  const int threads = threads_for(work);
  dim3 grid = grid_for(work, threads, bsz);
  cudaStream_t st = as_stream(stream);
  if (vec) k_swap<true><<<grid, threads, 0, st>>>(p);
  else k_swap<false><<<grid, threads, 0, st>>>(p);
  return launch_status(what);
}

extern "C" int tqk_apply_phase(void* state, int64_t bsz, int n, const int32_t* wires, int k, const void* phase,
                               int64_t phase_batch, void* stream) {
  return phase_entry(state, nullptr, bsz, n, wires, k, phase, phase_batch, nullptr, false, stream,
                     "tqk_apply_phase");
}

extern "C" int tqk_adjoint_phase(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires, int k,
                                 const void* phase, int64_t phase_batch, double* grad, void* stream) {
  return phase_entry(psi, lam, bsz, n, wires, k, phase, phase_batch, grad, true, stream, "tqk_adjoint_phase");
}

extern "C" int tqk_apply_diagonal(void* state, int64_t bsz, int n, const int32_t* wires, int k, const void* diag,
                                  int64_t diag_batch, void* stream) {
  return diag_entry(state, nullptr, bsz, n, wires, k, diag, diag_batch, nullptr, false, stream,
                    "tqk_apply_diagonal");
}

extern "C" int tqk_adjoint_diagonal(void* psi, void* lam, int64_t bsz, int n, const int32_t* wires, int k,
                                    const void* diag, int64_t diag_batch, double* grad, void* stream) {
  return diag_entry(psi, lam, bsz, n, wires, k, diag, diag_batch, grad, true, stream, "tqk_adjoint_diagonal");
}

extern "C" int64_t tqk_reset_scratch_bytes(int64_t bsz, int n) {
  (void)n;
  return bsz * (int64_t)sizeof(double);
}

extern "C" int tqk_reset(void* state, int64_t bsz, int n, const int32_t* wires, int k, void* scratch,
                         int64_t scratch_bytes, void* stream) {
  const char* what = "tqk_reset";
  int rc = check_state(state, bsz, n, what);
  if (rc) return rc;
  if (scratch == nullptr || scratch_bytes < tqk_reset_scratch_bytes(bsz, n))
    return fail(TQK_SCRATCH_TOO_SMALL, "%s: scratch of %lld bytes needed", what,
                (long long)tqk_reset_scratch_bytes(bsz, n));
  uint64_t mask = 0;
  if ((rc = wires_to_bits(n, wires, k, nullptr, &mask, what))) return rc;
  cudaStream_t st = as_stream(stream);
  double* norm2 = static_cast<double*>(scratch);
  if (cudaMemsetAsync(norm2, 0, bsz * sizeof(double), st) != cudaSuccess)
    return fail(TQK_CUDA_ERROR, "%s: memset failed", what);
  const int64_t half = (1ll << n) >> 1;
  const int threads = threads_for(half);
  dim3 grid = grid_for(half, threads, bsz);
  k_reset_zero<<<grid, threads, 0, st>>>(static_cast<float2*>(state), n, mask, norm2);
  if ((rc = launch_status(what))) return rc;
  k_reset_scale<<<grid, threads, 0, st>>>(static_cast<float2*>(state), n, norm2);
  return launch_status(what);
}
