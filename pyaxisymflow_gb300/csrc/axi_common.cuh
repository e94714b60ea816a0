// Shared helpers of the sm_103a kernels behind the C ABI in include/axisym_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <initializer_list>
#include <string>

#include "../../include/axisym_gb300.h"

namespace axi {

// Per-thread message of the last failing entry point (read by axi_last_error).
void set_error(const char* fmt, ...);
void clear_error();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

// Turns a launch error into AXI_ERR_CUDA with a message naming the kernel.
inline int launch_status(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: CUDA launch failed: %s", what, cudaGetErrorString(e));
    return AXI_ERR_CUDA;
  }
  return AXI_OK;
}

inline int check_grid(const char* what, int nr, int nz, int min_nr = 3, int min_nz = 3) {
  if (nr < min_nr || nz < min_nz) {
    set_error("%s: grid %d x %d is smaller than %d x %d", what, nr, nz, min_nr, min_nz);
    return AXI_ERR_INVALID;
  }
  return AXI_OK;
}

inline int check_ptr(const char* what, const void* p, const char* name) {
  if (p == nullptr) {
    set_error("%s: %s is null", what, name);
    return AXI_ERR_INVALID;
  }
  return AXI_OK;
}

// Every pointer in `ptrs` non-null; `names` names them in the same order.
inline int check_ptrs(const char* what, std::initializer_list<const void*> ptrs,
                      std::initializer_list<const char*> names) {
  const char* const* n = names.begin();
  for (const void* p : ptrs) {
    const char* name = n != names.end() ? *n++ : "pointer";
    if (p == nullptr) {
      set_error("%s: %s is null", what, name);
      return AXI_ERR_INVALID;
    }
  }
  return AXI_OK;
}

// Number of SMs on the current device (cached per device).
int sm_count();

}  // namespace axi

#define AXI_TRY(expr)            \
  do {                           \
    int _st = (expr);            \
    if (_st != AXI_OK) return _st; \
  } while (0)

// Rounded arithmetic that the compiler may not contract into FMA: used where
// results must match the reference's numpy evaluation bit for bit.
template <typename T> __device__ __forceinline__ T rn_mul(T a, T b);
template <typename T> __device__ __forceinline__ T rn_add(T a, T b);
template <typename T> __device__ __forceinline__ T rn_sub(T a, T b);
template <typename T> __device__ __forceinline__ T rn_div(T a, T b);
template <> __device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
template <> __device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }

// Host-side product of two scalars (kept separate so no contraction applies).
template <typename T> inline T rn_host_mul(T a, T b) { return a * b; }

template <typename T> __device__ __forceinline__ T dev_sin(T x);
template <> __device__ __forceinline__ double dev_sin(double x) { return sin(x); }
template <> __device__ __forceinline__ float dev_sin(float x) { return sinf(x); }

template <typename T> struct Pi;
template <> struct Pi<double> { static constexpr double v = 3.141592653589793; };
template <> struct Pi<float> { static constexpr float v = 3.14159265f; };

// Error-free float transformations (Knuth's two-sum; the FMA form of the
// exact product): a + b = s + e and a * b = p + e exactly. Used where float
// values are carried as unevaluated pairs (hi + lo) to keep more than float
// precision in float storage and arithmetic.
namespace axi_eft {
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = fmaf(a, b, -p);
}
// (hi, lo) + v as a renormalised pair: hi' is the rounded sum, lo' the
// remainder; hi' + lo' = hi + lo + v up to the rounding of the low part.
__device__ __forceinline__ void pair_add(float& hi, float& lo, float v) {
  float s, e, h2, l2;
  two_sum(hi, v, s, e);
  two_sum(s, __fadd_rn(lo, e), h2, l2);
  hi = h2;
  lo = l2;
}
}  // namespace axi_eft
