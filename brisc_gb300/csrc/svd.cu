// Small SVD of the IRLBA projection matrix B (m x (m+1)), replacing the
// reference's LAPACK sgesdd call (brisc/pca.pyx:514-545, 1178), and the
// convergence test + restart bookkeeping of brisc/pca.pyx:1180-1231.
//
// Method: one-sided (Hestenes) Jacobi on A = B^T, one CTA. Columns of A are
// rotated pairwise until mutually orthogonal; the accumulated rotations J
// give Ub = J, the column norms give Sb and the normalised columns give the
// rows of Vbt. Pairs are visited in a fixed round-robin (circle) schedule,
// m/2 disjoint pairs per round, one 8-lane group per pair, so the result
// does not depend on timing. Arithmetic is FP32: GB300's FP64 rate is a small fraction
// of its FP32 rate, and an O(m^3) FP64 Jacobi on one SM would cost more than
// the Lanczos steps it serves; the reference itself uses FP32 (sgesdd).
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "svd.cuh"

namespace bgpu {

namespace {

__device__ __forceinline__ void pair_of(int round, int idx, int M2, int* p,
                                        int* q) {
  const int L = M2 - 1;  // round, idx < L: one conditional subtraction is the modulo
  int a, b;
  if (idx == 0) {
    a = round;
    b = L;
  } else {
    a = round + idx;
    a -= a >= L ? L : 0;
    b = round - idx + L;
    b -= b >= L ? L : 0;
  }
  *p = min(a, b);
  *q = max(a, b);
}

// Jacobi rotation (c, s) zeroing the off-diagonal ga of the Gram block
// [al ga; ga be]: with x = be - al, y = 2 ga, t = tan(theta) =
// sign(x y) |y| / (|x| + sqrt(x^2 + y^2)) (the smaller root, no cancellation),
// c = 1 / sqrt(1 + t^2), s = c t. Every operation is correctly rounded.
__device__ __forceinline__ void rotation_of(float al, float be, float ga, float* c,
                                            float* s, float* tan_out) {
  const float x = be - al, y = 2.f * ga;
  const float r = sqrtf(fmaf(x, x, y * y));
  const float t = copysignf(fabsf(y), x * y) / (fabsf(x) + r);
  *c = __frsqrt_rn(fmaf(t, t, 1.f));
  *s = *c * t;
  *tan_out = t;
}
__device__ __forceinline__ void rotation_of(double al, double be, double ga, double* c,
                                            double* s, double* tan_out) {
  const double x = be - al, y = 2.0 * ga;
  const double r = sqrt(fma(x, x, y * y));
  const double t = copysign(fabs(y), x * y) / (fabs(x) + r);
  *c = 1.0 / sqrt(fma(t, t, 1.0));
  *s = *c * t;
  *tan_out = t;
}

// Column stride of A (len m + 1) and J (len m) in the workspace. The FP32
// kernel pads columns to a multiple of 32 floats so each lane of a pair's
// 8-lane group moves whole float4s (a group covers 128 contiguous bytes per
// access: no bank conflicts, a quarter of the shared-memory instructions);
// the padding is zero and stays zero under rotations.
template <typename T>
__host__ __device__ constexpr uint32_t col_stride(uint32_t len) {
  return std::is_same<T, float>::value ? (len + 31u) & ~31u : len;
}

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Rotates the float4 columns x, y (nv vectors each) of one pair: an 8-lane
// group, lane l8 taking vectors l8, l8 + 8, ...
__device__ __forceinline__ void rotate_cols4(float4* x, float4* y, uint32_t nv,
                                             int l8, float c, float sn) {
  for (uint32_t v = l8; v < nv; v += 8) {
    const float4 a = x[v], b = y[v];
    x[v] = make_float4(c * a.x - sn * b.x, c * a.y - sn * b.y, c * a.z - sn * b.z,
                       c * a.w - sn * b.w);
    y[v] = make_float4(sn * a.x + c * b.x, sn * a.y + c * b.y, sn * a.z + c * b.z,
                       sn * a.w + c * b.w);
  }
}

// T = float (FP32 Jacobi) or double (FP64 Jacobi). B is read in T; outputs are
// float (for the rotation GEMMs) plus, when non-null, the FP64 last row of Ub
// and FP64 singular values for the convergence test.
template <typename T>
__global__ void __launch_bounds__(1024)
k_jacobi(const T* __restrict__ Bin, uint32_t m, float* __restrict__ Ub,
         float* __restrict__ Sb, float* __restrict__ Vbt,
         double* __restrict__ ub_last, double* __restrict__ sb64,
         double* __restrict__ ub64, T* __restrict__ gwork, int use_smem,
         int max_sweeps, T thresh, int* __restrict__ info) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int rotated;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int la = (int)m + 1;  // column length of A = B^T
  const uint32_t lp = col_stride<T>(m + 1), jd = col_stride<T>(m);
  T* A = use_smem ? reinterpret_cast<T*>(smraw) : gwork;
  T* J = A + (uint64_t)m * lp;
  T* sig = J + (uint64_t)m * jd;
  for (uint32_t t = threadIdx.x; t < m * lp; t += blockDim.x) {
    const uint32_t i = t / lp, r = t % lp;   // A[r, i] = B[i, r]
    A[t] = r < (uint32_t)la ? Bin[i + (uint64_t)r * m] : T(0);
  }
  for (uint32_t t = threadIdx.x; t < m * jd; t += blockDim.x) {
    const uint32_t i = t / jd, r = t % jd;
    J[t] = r == i ? T(1) : T(0);
  }
  __syncthreads();

  // Pairs go to 8-lane groups (up to 128 disjoint pairs per round at once):
  // 8-lane reductions are 3 shuffle levels instead of 5.
  const int M2 = (int)m + ((int)m & 1);
  const int l8 = threadIdx.x & 7;
  const unsigned gm8 = 0xFFu << (lane & 24);
  const int grp = threadIdx.x >> 3, ngrp = blockDim.x >> 3;
  // Squared column norms live in `sig` during the sweeps: recomputed at each
  // sweep's start and carried through the rotations by the exact identities
  // |a_p'|^2 = |a_p|^2 - t ga, |a_q'|^2 = |a_q|^2 + t ga, so a pair needs only
  // its cross product.
  T* nrm = sig;
  int sweep = 0;
  for (; sweep < max_sweeps; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    for (uint32_t i = wid; i < m; i += nw) {
      const T* ai = A + (uint64_t)i * lp;
      T t2 = 0;
      for (int r = lane; r < la; r += 32) t2 += ai[r] * ai[r];
      t2 = warp_sum_t(t2);
      if (lane == 0) nrm[i] = t2;
    }
    __syncthreads();
    for (int round = 0; round < M2 - 1; ++round) {
      for (int idx = grp; idx < M2 / 2; idx += ngrp) {
        int p, q;
        pair_of(round, idx, M2, &p, &q);
        if (q >= (int)m) continue;
        T* ap = A + (uint64_t)p * lp;
        T* aq = A + (uint64_t)q * lp;
        T* jp = J + (uint64_t)p * jd;
        T* jq = J + (uint64_t)q * jd;
        const T al = nrm[p], be = nrm[q];
        T ga = 0;
        if constexpr (std::is_same<T, float>::value) {
          const float4* apv = reinterpret_cast<const float4*>(ap);
          const float4* aqv = reinterpret_cast<const float4*>(aq);
          for (uint32_t v = l8; v < lp / 4; v += 8) {
            const float4 x = apv[v], y = aqv[v];
            ga += x.x * y.x;
            ga += x.y * y.y;
            ga += x.z * y.z;
            ga += x.w * y.w;
          }
        } else {
          for (int r = l8; r < la; r += 8) ga += ap[r] * aq[r];
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) ga += __shfl_xor_sync(gm8, ga, o);
        if (al > T(0) && be > T(0) && ga * ga > thresh * thresh * (al * be)) {
          T c, sn, tn;
          rotation_of(al, be, ga, &c, &sn, &tn);
          if (l8 == 0) {
            nrm[p] = al - tn * ga;
            nrm[q] = be + tn * ga;
          }
          if constexpr (std::is_same<T, float>::value) {
            rotate_cols4(reinterpret_cast<float4*>(ap), reinterpret_cast<float4*>(aq),
                         lp / 4, l8, c, sn);
            rotate_cols4(reinterpret_cast<float4*>(jp), reinterpret_cast<float4*>(jq),
                         jd / 4, l8, c, sn);
          } else {
            for (int r = l8; r < la; r += 8) {
              const T x = ap[r], y = aq[r];
              ap[r] = c * x - sn * y;
              aq[r] = sn * x + c * y;
            }
            for (int r = l8; r < (int)m; r += 8) {
              const T x = jp[r], y = jq[r];
              jp[r] = c * x - sn * y;
              jq[r] = sn * x + c * y;
            }
          }
          if (l8 == 0) rotated = 1;
        }
      }
      __syncthreads();
    }
    const int any = rotated;
    __syncthreads();
    if (!any) break;
  }

  // singular values, descending order (ties by index), vectors
  for (uint32_t i = wid; i < m; i += nw) {
    const T* ai = A + (uint64_t)i * lp;
    T t = 0;
    for (int r = lane; r < la; r += 32) t += ai[r] * ai[r];
    t = warp_sum_t(t);
    if (lane == 0) sig[i] = sqrt(t);
  }
  __syncthreads();
  for (uint32_t i = wid; i < m; i += nw) {
    const T si = sig[i];
    int rank = 0;
    for (uint32_t jj = lane; jj < m; jj += 32) {
      const T sj = sig[jj];
      rank += (sj > si || (sj == si && jj < i)) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rank += __shfl_xor_sync(0xffffffffu, rank, o);
    const T* ji = J + (uint64_t)i * jd;
    if (lane == 0) {
      Sb[rank] = (float)si;
      if (sb64) sb64[rank] = (double)si;
      if (ub_last) ub_last[rank] = (double)ji[m - 1];
    }
    for (uint32_t r = lane; r < m; r += 32) {
      Ub[r + (uint64_t)rank * m] = (float)ji[r];
      if (ub64) ub64[r + (uint64_t)rank * m] = (double)ji[r];
    }
    const T* ai = A + (uint64_t)i * lp;
    const T inv = si > T(0) ? T(1) / si : T(0);
    for (int r = lane; r < la; r += 32)
      Vbt[rank + (uint64_t)r * m] = (float)(ai[r] * inv);
  }
  if (threadIdx.x == 0 && info) {
    info[0] = sweep;
    info[1] = sweep < max_sweeps ? 1 : 0;
  }
}

__global__ void __launch_bounds__(256)
k_restart_check(const float* __restrict__ Ub, const float* __restrict__ Sb,
                const double* __restrict__ ub_last, const double* __restrict__ sb64,
                uint32_t m, uint32_t k, float* __restrict__ rem, uint32_t g,
                float tol, float* __restrict__ smax, uint32_t kc,
                double* __restrict__ B, RestartStatus* __restrict__ st,
                float* __restrict__ ratios) {
  __shared__ double red[8];
  __shared__ double rn_s;
  __shared__ int conv_s, kc_s, nconv_w[8];
  __shared__ float smax_s;
  double t = 0.0;
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) t += (double)rem[c] * rem[c];
  t = warp_sum(t);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w];
    rn_s = sqrt(s);                          // remainder_norm, pca.pyx:1181
    smax_s = fmaxf(Sb[0], *smax);            // pca.pyx:1187
  }
  __syncthreads();
  // the residual test of every Ritz value at once (pca.pyx:1190-1193); the
  // count is an integer sum, so its order does not matter
  const double rn = rn_s;
  const float S = smax_s;
  uint32_t mine = 0;
  for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) {
    const double u = ub_last ? ub_last[i] : (double)Ub[(m - 1) + (uint64_t)i * m];
    const double residual = fabs(rn * u);
    const double bound = (double)tol * (double)S;
    mine += residual < bound ? 1u : 0u;
    if (ratios) ratios[i] = (float)(residual / bound);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0) nconv_w[threadIdx.x >> 5] = (int)mine;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t nconv = 0;
    for (int w = 0; w < 8; ++w) nconv += (uint32_t)nconv_w[w];
    *smax = S;
    const int conv = nconv == k;
    uint32_t kc_new = max(kc, k + nconv);
    kc_new = min(kc_new, m - 1);  // pca.pyx:1201-1202
    st->converged = conv;
    st->num_converged = (int)nconv;
    st->k_current = (int)kc_new;
    st->remainder_norm = (float)rn;
    st->smax = S;
    conv_s = conv;
    kc_s = (int)kc_new;
  }
  __syncthreads();
  const float rnf = (float)rn_s;
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) rem[c] /= rnf;  // :1182-1183
  if (!conv_s) {
    const uint32_t kcn = (uint32_t)kc_s;
    const uint64_t total = (uint64_t)m * (m + 1);
    for (uint64_t t2 = threadIdx.x; t2 < total; t2 += blockDim.x) B[t2] = 0.0;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < kcn; i += blockDim.x) {  // :1227-1231
      const double si = sb64 ? sb64[i] : (double)Sb[i];
      const double u = ub_last ? ub_last[i] : (double)Ub[(m - 1) + (uint64_t)i * m];
      B[i + (uint64_t)i * m] = si;
      B[i + (uint64_t)kcn * m] = rn_s * u;
    }
  }
}

__global__ void k_f2d(const float* __restrict__ a, uint64_t n, double* __restrict__ b) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

// ---------------------------------------------------------------------------
// FP64 Newton refinement of the FP32 SVD (Ogita & Aishima, "Iterative
// refinement for symmetric eigenvalue decomposition", 2018, Algorithm 1,
// applied to B B^T = U diag(sigma^2) U^T). The FP32 Jacobi stops rotating a
// pair once its columns are orthogonal to ~2.4e-6; for two singular values a
// relative 6e-5 apart that leaves their vectors mixed by ~2 %, and the
// convergence test reads exactly those vectors' last entries. Each step, in
// FP64 with every product spread over many CTAs:
//   W = B^T U, S = W^T W, R = I - U^T U, lam_i = S_ii / (1 - R_ii),
//   E_ij = (S_ij + lam_j R_ij) / (lam_j - lam_i)   (i != j, when the pair is
//          resolved: |numerator| < |lam_j - lam_i| / 4),
//   E_ij = R_ij / 2 otherwise and on the diagonal,   U <- U + U E,
// which converges quadratically; three steps take FP32-accurate factors to
// FP64 accuracy. Then sigma_i = sqrt(lam_i) and Vbt's rows are (B^T U)_i /
// sigma_i.
// Warp-per-output dot products: lanes stride the summed index (coalesced,
// contiguous columns), a fixed xor tree closes the sum.
__device__ __forceinline__ double warp_dot64(const double* __restrict__ a,
                                             const double* __restrict__ b,
                                             uint32_t len, int lane) {
  double acc = 0.0;
  for (uint32_t c = lane; c < len; c += 32) acc = fma(a[c], b[c], acc);
  return warp_sum_t(acc);
}

// W = B^T U: W[r, i] = column r of B . column i of U ((m+1) x m outputs).
__global__ void __launch_bounds__(256)
k_oa_w(const double* __restrict__ B, const double* __restrict__ U, uint32_t m,
       double* __restrict__ W) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= (uint64_t)(m + 1) * m) return;
  const uint32_t r = (uint32_t)(w % (m + 1)), i = (uint32_t)(w / (m + 1));
  const double v = warp_dot64(B + (uint64_t)r * m, U + (uint64_t)i * m, m, lane);
  if (lane == 0) W[r + (uint64_t)i * (m + 1)] = v;
}

// S = W^T W and R = I - U^T U (m x m outputs, one warp each).
__global__ void __launch_bounds__(256)
k_oa_sr(const double* __restrict__ W, const double* __restrict__ U, uint32_t m,
        double* __restrict__ S, double* __restrict__ R) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= (uint64_t)m * m) return;
  const uint32_t i = (uint32_t)(w % m), j = (uint32_t)(w / m);
  const double s = warp_dot64(W + (uint64_t)i * (m + 1), W + (uint64_t)j * (m + 1),
                              m + 1, lane);
  const double q = warp_dot64(U + (uint64_t)i * m, U + (uint64_t)j * m, m, lane);
  if (lane == 0) {
    S[w] = s;
    R[w] = (i == j ? 1.0 : 0.0) - q;
  }
}

// lam_i = S_ii / (1 - R_ii) and the Newton correction E (m x m outputs,
// one thread each; every thread recomputes the two lam it needs).
__global__ void __launch_bounds__(256)
k_oa_e(const double* __restrict__ S, const double* __restrict__ R, uint32_t m,
       double* __restrict__ lam, double* __restrict__ E) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t >= (uint64_t)m * m) return;
  const uint32_t i = (uint32_t)(t % m), j = (uint32_t)(t / m);
  const uint64_t di = (uint64_t)i * m + i, dj = (uint64_t)j * m + j;
  const double li = S[di] / (1.0 - R[di]);
  const double lj = S[dj] / (1.0 - R[dj]);
  if (i == j) lam[i] = li;
  double e = 0.5 * R[t];
  if (i != j) {
    const double num = S[t] + lj * R[t];
    const double den = lj - li;
    if (fabs(num) < 0.25 * fabs(den)) e = num / den;
  }
  E[t] = e;
}

__global__ void k_oa_u(const double* __restrict__ U, const double* __restrict__ E,
                       uint32_t m, double* __restrict__ Un) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t >= (uint64_t)m * m) return;
  const uint32_t r = (uint32_t)(t % m), i = (uint32_t)(t / m);
  const double* e = E + (uint64_t)i * m;
  double acc = U[t];
  for (uint32_t c = 0; c < m; ++c) acc = fma(U[r + (uint64_t)c * m], e[c], acc);
  Un[t] = acc;
}

// Outputs: Vbt[i, r] = (B^T U)[r, i] / sigma_i (one warp each), Ub, Sb and
// the FP64 last row of Ub and singular values.
__global__ void __launch_bounds__(256)
k_oa_out(const double* __restrict__ B, const double* __restrict__ U,
         const double* __restrict__ lam, uint32_t m, float* __restrict__ Ub,
         float* __restrict__ Sb, float* __restrict__ Vbt, double* __restrict__ ub_last,
         double* __restrict__ sb64) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (w >= (uint64_t)(m + 1) * m) return;
  const uint32_t i = (uint32_t)(w % m), r = (uint32_t)(w / m);
  const double sig = sqrt(fmax(lam[i], 0.0));
  const double v = warp_dot64(B + (uint64_t)r * m, U + (uint64_t)i * m, m, lane);
  if (lane == 0) {
    Vbt[w] = sig > 0.0 ? (float)(v / sig) : 0.f;
    if (r < m) Ub[(uint64_t)r + (uint64_t)i * m] = (float)U[(uint64_t)r + (uint64_t)i * m];
    if (r == 0) {
      Sb[i] = (float)sig;
      sb64[i] = sig;
      ub_last[i] = U[(uint64_t)(m - 1) + (uint64_t)i * m];
    }
  }
}

}  // namespace

size_t svd_refine_doubles(uint32_t m) {
  return 5ull * m * m + (uint64_t)(m + 1) * m + m;
}

int launch_svd_refine(const double* B, uint32_t m, float* Ub, float* Sb, float* Vbt,
                      double* ub_last, double* sb64, double* work, int steps,
                      cudaStream_t s, double* u64_out) {
  const uint64_t mm = (uint64_t)m * m;
  double* U = work;
  double* Un = U + mm;
  double* Sm = Un + mm;
  double* R = Sm + mm;
  double* E = R + mm;
  double* W = E + mm;
  double* lam = W + (uint64_t)(m + 1) * m;
  // warp-per-output kernels: 8 outputs per 256-thread block
  const unsigned gw = (unsigned)ceil_div((uint64_t)(m + 1) * m, 8);
  const unsigned gs = (unsigned)ceil_div(mm, 8);
  const unsigned ge = (unsigned)ceil_div(mm, 256);
  const unsigned gm = (unsigned)ceil_div(mm, 128);
  k_f2d<<<(unsigned)ceil_div(mm, 256), 256, 0, s>>>(Ub, mm, U);
  BGPU_CHECK_LAUNCH();
  for (int it = 0; it < steps; ++it) {
    k_oa_w<<<gw, 256, 0, s>>>(B, U, m, W);
    BGPU_CHECK_LAUNCH();
    k_oa_sr<<<gs, 256, 0, s>>>(W, U, m, Sm, R);
    BGPU_CHECK_LAUNCH();
    k_oa_e<<<ge, 256, 0, s>>>(Sm, R, m, lam, E);
    BGPU_CHECK_LAUNCH();
    k_oa_u<<<gm, 128, 0, s>>>(U, E, m, Un);
    BGPU_CHECK_LAUNCH();
    std::swap(U, Un);
  }
  // the eigenvalues of the refined U: one more S diagonal
  k_oa_w<<<gw, 256, 0, s>>>(B, U, m, W);
  BGPU_CHECK_LAUNCH();
  k_oa_sr<<<gs, 256, 0, s>>>(W, U, m, Sm, R);
  BGPU_CHECK_LAUNCH();
  k_oa_e<<<ge, 256, 0, s>>>(Sm, R, m, lam, E);
  BGPU_CHECK_LAUNCH();
  k_oa_out<<<gw, 256, 0, s>>>(B, U, lam, m, Ub, Sb, Vbt, ub_last, sb64);
  BGPU_CHECK_LAUNCH();
  if (u64_out) BGPU_CUDA(cudaMemcpyAsync(u64_out, U, mm * 8, cudaMemcpyDeviceToDevice, s));
  return BGPU_OK;
}

int launch_float_to_double(const float* a, uint64_t n, double* b, cudaStream_t s) {
  k_f2d<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(a, n, b);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

size_t jacobi_smem_bytes(uint32_t m, bool fp64) {
  if (fp64)
    return ((size_t)m * col_stride<double>(m + 1) + (size_t)m * col_stride<double>(m) + m) * 8;
  return ((size_t)m * col_stride<float>(m + 1) + (size_t)m * col_stride<float>(m) + m) * 4;
}

size_t jacobi_global_bytes(uint32_t m, bool fp64) {
  return jacobi_smem_bytes(m, fp64);
}

float jacobi_threshold(uint32_t m) {
  return std::max(1e-6f, 2.4e-7f * std::sqrt((float)(m + 1)));
}

int launch_jacobi_svd(const float* Bf, const double* Bd, uint32_t m, float* Ub,
                      float* Sb, float* Vbt, double* ub_last, double* sb64,
                      void* gwork, int* info, cudaStream_t s, double* ub64) {
  const bool fp64 = Bd != nullptr;
  const size_t smem = jacobi_smem_bytes(m, fp64);
  const bool use_smem = smem <= 220 * 1024;
  BGPU_REQUIRE(use_smem || gwork, BGPU_ERR_INVALID,
               "small SVD of this size needs a global workspace");
  // one 8-lane group per pair of a round, in whole warps: a small matrix
  // gets a small block and cheap barriers (each pair's arithmetic, and so
  // the result, does not depend on the block size)
  const unsigned threads = (unsigned)std::min<uint64_t>(
      1024, std::max<uint64_t>(64, round_up(8ull * ((m + 1) / 2), 32)));
  if (fp64) {
    if (use_smem && smem > 48 * 1024)
      BGPU_CUDA(allow_max_smem(k_jacobi<double>));
    k_jacobi<double><<<1, threads, use_smem ? smem : 0, s>>>(
        Bd, m, Ub, Sb, Vbt, ub_last, sb64, ub64, (double*)gwork, use_smem ? 1 : 0, 40,
        1e-13, info);
  } else {
    if (use_smem && smem > 48 * 1024)
      BGPU_CUDA(allow_max_smem(k_jacobi<float>));
    k_jacobi<float><<<1, threads, use_smem ? smem : 0, s>>>(
        Bf, m, Ub, Sb, Vbt, ub_last, sb64, ub64, (float*)gwork, use_smem ? 1 : 0, 40,
        jacobi_threshold(m), info);
  }
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_restart_check(const float* Ub, const float* Sb, const double* ub_last,
                         const double* sb64, uint32_t m, uint32_t k, float* rem,
                         uint32_t g, float tol, float* smax, uint32_t kc,
                         double* B, RestartStatus* st, float* ratios,
                         cudaStream_t s) {
  k_restart_check<<<1, 256, 0, s>>>(Ub, Sb, ub_last, sb64, m, k, rem, g, tol,
                                    smax, kc, B, st, ratios);
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
  // FP64 Jacobi on a double copy of B (the solver's own precision).
  const size_t cnt = (size_t)m * (m + 1);
  double* Bd = nullptr;
  void* gwork = nullptr;
  BGPU_CUDA(cudaMallocAsync((void**)&Bd, cnt * 8, s));
  if (jacobi_smem_bytes(m, true) > 220 * 1024)
    BGPU_CUDA(cudaMallocAsync(&gwork, jacobi_global_bytes(m, true), s));
  int rc = launch_float_to_double(B, cnt, Bd, s);
  if (rc == BGPU_OK)
    rc = launch_jacobi_svd(nullptr, Bd, m, Ub, Sb, Vbt, nullptr, nullptr, gwork,
                           nullptr, s);
  cudaFreeAsync(Bd, s);
  if (gwork) cudaFreeAsync(gwork, s);
  if (rc == BGPU_OK) BGPU_CUDA(cudaStreamSynchronize(s));
  return rc;
}
