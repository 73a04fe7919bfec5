// Shared definitions for the brisc_gb300 sparse-PCA kernels (sm_103a).
//
// Conventions used throughout the library:
//  * every C-ABI entry point returns an `int` status (0 = ok) and records a
//    human-readable message retrievable with bgpu_last_error();
//  * dense bases (U, V and their rotated copies) are column-major with a padded
//    leading dimension so every column starts on a 256-byte boundary;
//  * every reduction runs over fixed blocks in a fixed order, so results are
//    bit-identical from run to run (no floating-point atomics anywhere).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <set>
#include <string>
#include <utility>

#include "../../include/briscgpu.h"

namespace bgpu {

// ---------------------------------------------------------------------------
// error plumbing
void set_error(const std::string& msg);
const char* get_error();

struct Status {
  int code = BGPU_OK;
  bool ok() const { return code == BGPU_OK; }
};

#define BGPU_CUDA(call)                                                        \
  do {                                                                         \
    cudaError_t e__ = (call);                                                  \
    if (e__ != cudaSuccess) {                                                  \
      ::bgpu::set_error(std::string(#call) + " failed: " +                     \
                        cudaGetErrorString(e__) + " (" __FILE__ ":" +          \
                        std::to_string(__LINE__) + ")");                       \
      return BGPU_ERR_CUDA;                                                    \
    }                                                                          \
  } while (0)

#define BGPU_CHECK_LAUNCH() BGPU_CUDA(cudaGetLastError())

#define BGPU_REQUIRE(cond, code, msg)                                          \
  do {                                                                         \
    if (!(cond)) {                                                             \
      ::bgpu::set_error(msg);                                                  \
      return (code);                                                           \
    }                                                                          \
  } while (0)

#define BGPU_TRY(expr)                                                         \
  do {                                                                         \
    int s__ = (expr);                                                          \
    if (s__ != BGPU_OK) return s__;                                            \
  } while (0)

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs; refreshed at runtime
int num_sms();                 // queried once per device

// Lets `fn` use up to the device's opt-in shared memory per block. The limit
// is a per-function setting shared by every host thread: setting it to one
// fixed value (rather than each launch's own size) means concurrent launches
// from several threads never meet a limit another thread has just lowered.
int device_smem_optin();
// Set once per function and device (a launch path then pays no driver calls).
template <typename F>
inline cudaError_t allow_max_smem(F* fn) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const auto key = std::make_pair((const void*)fn, dev);
  std::lock_guard<std::mutex> lk(mu);
  if (done.count(key)) return cudaSuccess;
  cudaFuncAttributes a;
  e = cudaFuncGetAttributes(&a, fn);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           device_smem_optin() - (int)a.sharedSizeBytes);
  if (e == cudaSuccess) done.insert(key);
  return e;
}

__host__ __device__ inline uint64_t round_up(uint64_t x, uint64_t m) {
  return (x + m - 1) / m * m;
}
__host__ __device__ inline uint64_t ceil_div(uint64_t x, uint64_t m) {
  return (x + m - 1) / m;
}
__device__ inline uint64_t ceil_div_dev(uint64_t x, uint64_t m) {
  return (x + m - 1) / m;
}
__host__ __device__ inline uint64_t min_u64(uint64_t a, uint64_t b) {
  return a < b ? a : b;
}

// Leading dimension for an n-row column-major basis: columns start 256-byte
// aligned (64 floats), which keeps every float4 / bulk copy aligned.
inline uint64_t basis_ld(uint64_t n) { return round_up(n, 64); }

// ---------------------------------------------------------------------------
// device helpers
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// Sum over aligned groups of G lanes (G power of two, <= 32); fixed xor tree.
template <int G>
__device__ __forceinline__ float group_sum(float v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Streaming 128-bit load that bypasses L1 (the matrix is read once per pass).
__device__ __forceinline__ uint4 ld_stream_u4(const void* p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ uint2 ld_stream_u2(const void* p) {
  uint2 r;
  asm volatile("ld.global.nc.L1::no_allocate.v2.u32 {%0,%1}, [%2];"
               : "=r"(r.x), "=r"(r.y)
               : "l"(p));
  return r;
}

// Normalised value of one raw count in the fused layout: the reference's
// `log1p(data[j] * inverse_size_factor)` (brisc/normalize.pyx:81), evaluated
// in float exactly as written there (the product rounded before the log, in
// every kernel that inlines this).
__device__ __forceinline__ float norm_count(uint32_t count, float isf) {
  return log1pf(__fmul_rn((float)count, isf));
}

}  // namespace bgpu
