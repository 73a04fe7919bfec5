// bgpu_small_svd_noalloc: the small SVD of bgpu_small_svd with its scratch
// in a fixed device array instead of per-call allocations.
//
// Who needs it: a caller whose process hands all device memory to its own
// pool (a framework's caching allocator, a serving engine that reserves HBM
// at start-up) cannot let a library call cudaMalloc behind its back without
// running out of memory or fragmenting the pool; and a caller in a
// latency-critical loop cannot afford cudaMalloc/cudaFree, which may
// synchronise the whole device. This entry point allocates nothing.
//
// Scratch: one file-scope device array, sized for subspaces up to
// kNoAllocSvdMaxM (3 * m * (m + 1) doubles: the FP64 copy of B, then the
// Jacobi workspace used when the matrices do not fit in shared memory). Every
// GPU that loads the library holds it (about 1.6 MB) until the process exits.
// Its address is looked up once per device with cudaGetSymbolAddress, on the
// first call made with that device current; make that first call before any
// stream capture. Nothing in the array has to start at zero (every word that
// is read was written earlier in the same call), and all calls share it, so
// calls whose work overlaps on the GPU (different streams, or different host
// threads on one device) race and must be serialised by the caller.
#include <mutex>

#include "svd.cuh"

namespace bgpu {
namespace {

constexpr uint32_t kNoAllocSvdMaxM = 256;
constexpr size_t kNoAllocSvdDoubles =
    3ull * kNoAllocSvdMaxM * (kNoAllocSvdMaxM + 1);

static __device__ __align__(256) double g_svd_scratch[kNoAllocSvdDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_svd_scratch on the current device (looked up once).
int scratch_for_current_device(double** out) {
  int dev = -1;
  BGPU_CUDA(cudaGetDevice(&dev));
  BGPU_REQUIRE(dev >= 0 && dev < kMaxDevices, BGPU_ERR_UNSUPPORTED,
               "bgpu_small_svd_noalloc: device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    BGPU_CUDA(cudaGetSymbolAddress(&p, g_svd_scratch));
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return BGPU_OK;
}

}  // namespace
}  // namespace bgpu

using namespace bgpu;

extern "C" BGPU_API int bgpu_small_svd_noalloc(const float* B, uint32_t m,
                                               float* Ub, float* Sb, float* Vbt,
                                               void* stream) {
  BGPU_REQUIRE(B && Ub && Sb && Vbt && m >= 1, BGPU_ERR_INVALID,
               "bad small-SVD arguments");
  BGPU_REQUIRE(m <= kNoAllocSvdMaxM, BGPU_ERR_INVALID,
               "m = " + std::to_string(m) +
                   " exceeds the fixed scratch limit of " +
                   std::to_string(kNoAllocSvdMaxM) +
                   " (use bgpu_small_svd, which allocates)");
  cudaStream_t s = (cudaStream_t)stream;
  double* scratch = nullptr;
  BGPU_TRY(scratch_for_current_device(&scratch));
  const size_t cnt = (size_t)m * (m + 1);
  double* Bd = scratch;          // FP64 copy of B, m * (m + 1)
  double* gwork = scratch + cnt;  // Jacobi workspace, 2 * m * (m + 1)
  static_assert(3ull * kNoAllocSvdMaxM * (kNoAllocSvdMaxM + 1) ==
                    kNoAllocSvdDoubles, "scratch layout");
  const bool need_work = jacobi_smem_bytes(m, true) > 220 * 1024;
  BGPU_REQUIRE(!need_work || jacobi_global_bytes(m, true) <= 2 * cnt * sizeof(double),
               BGPU_ERR_UNSUPPORTED, "small-SVD workspace layout mismatch");
  BGPU_TRY(launch_float_to_double(B, cnt, Bd, s));
  BGPU_TRY(launch_jacobi_svd(nullptr, Bd, m, Ub, Sb, Vbt, nullptr, nullptr,
                             need_work ? gwork : nullptr, nullptr, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  return BGPU_OK;
}
