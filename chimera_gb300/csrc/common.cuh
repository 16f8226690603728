// Shared helpers for the chimera_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/chimera_gb300.h"

typedef int64_t i64;

namespace chm {

// Last error text for chm_last_error(); set by the entry points.
void set_error(const char *fmt, ...);
// Host-side counters read by chm_launch_count() / chm_gemm_flops().
void count_launch();
void count_gemm_flops(double flops);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Complex FP64 helpers on double2 {re, im}.
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) {
  return make_double2(a.x * s, a.y * s);
}
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// i * a
__host__ __device__ __forceinline__ double2 cmuli(double2 a) { return make_double2(-a.y, a.x); }

__host__ __device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// SMs of the current device (read once)
inline int sm_count() {
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 152;
  }
  return nsm;
}

// Grid size helper: enough blocks to cover n, capped to keep every SM busy
// with several resident blocks.
inline unsigned grid_for(i64 n, int threads, int cap_per_sm = 32) {
  i64 b = (n + threads - 1) / threads;
  i64 cap = (i64)sm_count() * cap_per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

}  // namespace chm

// Launch-status check used by every entry point: returns CHM_ERR_CUDA with
// the CUDA error text recorded.
#define CHM_CHECK_LAUNCH()                                                   \
  do {                                                                       \
    cudaError_t _e = cudaGetLastError();                                     \
    if (_e != cudaSuccess) {                                                 \
      chm::set_error("%s: %s", __func__, cudaGetErrorString(_e));            \
      return CHM_ERR_CUDA;                                                   \
    }                                                                        \
  } while (0)

#define CHM_REQUIRE(cond, ...)                                               \
  do {                                                                       \
    if (!(cond)) {                                                           \
      chm::set_error(__VA_ARGS__);                                           \
      return CHM_ERR_ARG;                                                    \
    }                                                                        \
  } while (0)
