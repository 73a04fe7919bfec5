// Small SVD of the IRLBA projection matrix B (m x (m+1)), replacing the
// reference's LAPACK sgesdd call (brisc/pca.pyx:514-545, 1178), and the
// convergence test + restart bookkeeping of brisc/pca.pyx:1180-1231.
//
// Method: one-sided (Hestenes) Jacobi on A = B^T, one CTA. Columns of A are
// rotated pairwise until mutually orthogonal; the accumulated rotations J
// give Ub = J, the column norms give Sb and the normalised columns give the
// rows of Vbt. Pairs are visited in a fixed round-robin (circle) schedule,
// m/2 disjoint pairs per round, one warp per pair, so the result does not
// depend on timing. Arithmetic is FP32: GB300's FP64 rate is a small fraction
// of its FP32 rate, and an O(m^3) FP64 Jacobi on one SM would cost more than
// the Lanczos steps it serves; the reference itself uses FP32 (sgesdd).
#include <algorithm>
#include <cmath>

#include "svd.cuh"

namespace bgpu {

namespace {

__device__ __forceinline__ void pair_of(int round, int idx, int M2, int* p,
                                        int* q) {
  const int L = M2 - 1;
  int a, b;
  if (idx == 0) {
    a = round;
    b = L;
  } else {
    a = (round + idx) % L;
    b = (round - idx + L) % L;
  }
  *p = min(a, b);
  *q = max(a, b);
}

__global__ void __launch_bounds__(1024)
k_jacobi(const float* __restrict__ Bf, uint32_t m, float* __restrict__ Ub,
         float* __restrict__ Sb, float* __restrict__ Vbt,
         float* __restrict__ gwork, int use_smem, int max_sweeps, float thresh,
         int* __restrict__ info) {
  extern __shared__ float sm[];
  __shared__ int rotated;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int la = (int)m + 1;  // column length of A = B^T
  float* A = use_smem ? sm : gwork;
  float* J = A + (uint64_t)m * la;
  for (uint32_t t = threadIdx.x; t < m * (uint32_t)la; t += blockDim.x) {
    const uint32_t i = t / la, r = t % la;   // A[r, i] = B[i, r]
    A[(uint64_t)i * la + r] = Bf[i + (uint64_t)r * m];
  }
  for (uint32_t t = threadIdx.x; t < m * m; t += blockDim.x)
    J[t] = (t / m == t % m) ? 1.f : 0.f;
  __syncthreads();

  const int M2 = (int)m + ((int)m & 1);
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int round = 0; round < M2 - 1; ++round) {
      for (int idx = wid; idx < M2 / 2; idx += nw) {
        int p, q;
        pair_of(round, idx, M2, &p, &q);
        if (q >= (int)m) continue;
        float* ap = A + (uint64_t)p * la;
        float* aq = A + (uint64_t)q * la;
        float al = 0.f, be = 0.f, ga = 0.f;
        for (int r = lane; r < la; r += 32) {
          const float x = ap[r], y = aq[r];
          al += x * x;
          be += y * y;
          ga += x * y;
        }
        al = warp_sum(al);
        be = warp_sum(be);
        ga = warp_sum(ga);
        if (al > 0.f && be > 0.f && fabsf(ga) > thresh * sqrtf(al * be)) {
          const float zeta = (be - al) / (2.f * ga);
          const float t = copysignf(1.f, zeta) /
                          (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
          const float c = 1.f / sqrtf(1.f + t * t);
          const float s = c * t;
          for (int r = lane; r < la; r += 32) {
            const float x = ap[r], y = aq[r];
            ap[r] = c * x - s * y;
            aq[r] = s * x + c * y;
          }
          float* jp = J + (uint64_t)p * m;
          float* jq = J + (uint64_t)q * m;
          for (int r = lane; r < (int)m; r += 32) {
            const float x = jp[r], y = jq[r];
            jp[r] = c * x - s * y;
            jq[r] = s * x + c * y;
          }
          if (lane == 0) rotated = 1;
        }
      }
      __syncthreads();
    }
    const int any = rotated;
    __syncthreads();
    if (!any) break;
  }

  // singular values, descending order (ties by index), vectors
  float* sig = use_smem ? (J + (uint64_t)m * m) : (J + (uint64_t)m * m);
  for (uint32_t i = wid; i < m; i += nw) {
    const float* ai = A + (uint64_t)i * la;
    float t = 0.f;
    for (int r = lane; r < la; r += 32) t += ai[r] * ai[r];
    t = warp_sum(t);
    if (lane == 0) sig[i] = sqrtf(t);
  }
  __syncthreads();
  for (uint32_t i = wid; i < m; i += nw) {
    const float si = sig[i];
    int rank = 0;
    for (uint32_t jj = lane; jj < m; jj += 32) {
      const float sj = sig[jj];
      rank += (sj > si || (sj == si && jj < i)) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rank += __shfl_xor_sync(0xffffffffu, rank, o);
    if (lane == 0) Sb[rank] = si;
    const float* ji = J + (uint64_t)i * m;
    for (uint32_t r = lane; r < m; r += 32) Ub[r + (uint64_t)rank * m] = ji[r];
    const float* ai = A + (uint64_t)i * la;
    const float inv = si > 0.f ? 1.f / si : 0.f;
    for (int r = lane; r < la; r += 32) Vbt[rank + (uint64_t)r * m] = ai[r] * inv;
  }
  if (threadIdx.x == 0 && info) {
    info[0] = sweep;
    info[1] = sweep < max_sweeps ? 1 : 0;
  }
}

__global__ void __launch_bounds__(256)
k_restart_check(const float* __restrict__ Ub, const float* __restrict__ Sb,
                uint32_t m, uint32_t k, float* __restrict__ rem, uint32_t g,
                float tol, float* __restrict__ smax, uint32_t kc,
                double* __restrict__ B, RestartStatus* __restrict__ st) {
  __shared__ double red[8];
  __shared__ float rn_s;
  __shared__ int conv_s, kc_s;
  double t = 0.0;
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) t += (double)rem[c] * rem[c];
  t = warp_sum(t);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w];
    const float rn = (float)sqrt(s);  // remainder_norm, pca.pyx:1181
    const float S = fmaxf(Sb[0], *smax);  // pca.pyx:1187
    *smax = S;
    uint32_t nconv = 0;
    for (uint32_t i = 0; i < k; ++i) {
      const float residual = rn * Ub[(m - 1) + (uint64_t)i * m];  // pca.pyx:1192
      nconv += fabsf(residual) < tol * S ? 1u : 0u;
    }
    const int conv = nconv == k;
    uint32_t kc_new = max(kc, k + nconv);
    kc_new = min(kc_new, m - 1);  // pca.pyx:1201-1202
    st->converged = conv;
    st->num_converged = (int)nconv;
    st->k_current = (int)kc_new;
    st->remainder_norm = rn;
    st->smax = S;
    rn_s = rn;
    conv_s = conv;
    kc_s = (int)kc_new;
  }
  __syncthreads();
  const float rn = rn_s;
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) rem[c] /= rn;  // :1182-1183
  if (!conv_s) {
    const uint32_t kcn = (uint32_t)kc_s;
    const uint64_t total = (uint64_t)m * (m + 1);
    for (uint64_t t2 = threadIdx.x; t2 < total; t2 += blockDim.x) B[t2] = 0.0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kcn; i += blockDim.x) {  // :1227-1231
      B[i + (uint64_t)i * m] = (double)Sb[i];
      B[i + (uint64_t)kcn * m] = (double)(rn * Ub[(m - 1) + (uint64_t)i * m]);
    }
  }
}

}  // namespace

size_t jacobi_smem_bytes(uint32_t m) {
  return ((size_t)m * (m + 1) + (size_t)m * m + m) * sizeof(float);
}

size_t jacobi_global_floats(uint32_t m) {
  return (size_t)m * (m + 1) + (size_t)m * m + m;
}

float jacobi_threshold(uint32_t m) {
  return std::max(1e-6f, 2.4e-7f * std::sqrt((float)(m + 1)));
}

int launch_jacobi_svd(const float* Bf, uint32_t m, float* Ub, float* Sb,
                      float* Vbt, float* gwork, int* info, cudaStream_t s) {
  const size_t smem = jacobi_smem_bytes(m);
  const bool use_smem = smem <= 220 * 1024;
  BGPU_REQUIRE(use_smem || gwork, BGPU_ERR_INVALID,
               "small SVD of this size needs a global workspace");
  if (use_smem && smem > 48 * 1024)
    BGPU_CUDA(cudaFuncSetAttribute(k_jacobi,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  k_jacobi<<<1, 1024, use_smem ? smem : 0, s>>>(Bf, m, Ub, Sb, Vbt, gwork,
                                                use_smem ? 1 : 0, 40,
                                                jacobi_threshold(m), info);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_restart_check(const float* Ub, const float* Sb, uint32_t m,
                         uint32_t k, float* rem, uint32_t g, float tol,
                         float* smax, uint32_t kc, double* B,
                         RestartStatus* st, cudaStream_t s) {
  k_restart_check<<<1, 256, 0, s>>>(Ub, Sb, m, k, rem, g, tol, smax, kc, B, st);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu

using namespace bgpu;

extern "C" int bgpu_small_svd(const float* B, uint32_t m, float* Ub, float* Sb,
                              float* Vbt, void* stream) {
  BGPU_REQUIRE(B && Ub && Sb && Vbt && m >= 1, BGPU_ERR_INVALID,
               "bad small-SVD arguments");
  cudaStream_t s = (cudaStream_t)stream;
  float* gwork = nullptr;
  if (jacobi_smem_bytes(m) > 220 * 1024)
    BGPU_CUDA(cudaMallocAsync((void**)&gwork, jacobi_global_floats(m) * 4, s));
  int rc = launch_jacobi_svd(B, m, Ub, Sb, Vbt, gwork, nullptr, s);
  if (gwork) cudaFreeAsync(gwork, s);
  return rc;
}
