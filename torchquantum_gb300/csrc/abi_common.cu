// abi_common.cu -- error reporting and argument validation shared by the C ABI.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "common.cuh"

namespace tqk {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int launch_status(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(TQK_CUDA_ERROR, "%s: CUDA error %s", what, cudaGetErrorString(e));
  return TQK_OK;
}

int check_state(const void* state, int64_t bsz, int n, const char* what) {
  if (state == nullptr) return fail(TQK_BAD_POINTER, "%s: null state pointer", what);
  if ((reinterpret_cast<uintptr_t>(state) & 15u) != 0)
    return fail(TQK_BAD_POINTER, "%s: state pointer must be 16-byte aligned", what);
  if (bsz <= 0 || bsz > 65535) return fail(TQK_BAD_SHAPE, "%s: bsz=%lld out of range [1,65535]", what, (long long)bsz);
  if (n < 1 || n > TQK_MAX_QUBITS) return fail(TQK_TOO_MANY_QUBITS, "%s: n_wires=%d out of range [1,%d]", what, n, TQK_MAX_QUBITS);
  return TQK_OK;
}

int check_batch(int64_t batch, int64_t bsz, const char* what) {
  if (batch != 1 && batch != bsz)
    return fail(TQK_BAD_SHAPE, "%s: operand batch %lld must be 1 or bsz=%lld", what, (long long)batch, (long long)bsz);
  return TQK_OK;
}

int wires_to_bits(int n, const int32_t* wires, int k, int* bits_out, uint64_t* used_mask, const char* what) {
  if (k > 0 && wires == nullptr) return fail(TQK_BAD_WIRES, "%s: null wires", what);
  for (int i = 0; i < k; ++i) {
    const int w = wires[i];
    if (w < 0 || w >= n) return fail(TQK_BAD_WIRES, "%s: wire %d out of range for n_wires=%d", what, w, n);
    const uint64_t bit = 1ull << (n - 1 - w);
    if (*used_mask & bit) return fail(TQK_BAD_WIRES, "%s: wire %d used twice", what, w);
    *used_mask |= bit;
    if (bits_out) bits_out[i] = n - 1 - w;
  }
  return TQK_OK;
}

BitInsert make_insert(uint64_t mask) {
  BitInsert bi;
  bi.m = 0;
  for (int q = 0; q < 64 && bi.m < kMaxInsert; ++q)
    if (mask & (1ull << q)) bi.pos[bi.m++] = q;
  for (int i = bi.m; i < kMaxInsert; ++i) bi.pos[i] = 0;
  return bi;
}

}  // namespace tqk

extern "C" const char* tqk_last_error(void) { return tqk::g_err; }
extern "C" int tqk_version(void) { return 1; }
