// Restart SVD by a secular-equation merge. It replaces the reference's full
// LAPACK sgesdd of B (brisc/pca.pyx:514-545, 1178) at every restart after
// the first.
//
// After a restart the reference rebuilds B as diag(s) in its first kc
// columns plus the residual column kc (brisc/pca.pyx:1227-1231); the Lanczos
// steps of the next cycle then fill rows kc..m-1 with alpha on the diagonal
// and beta above it, and B[m-1, m] stays 0 (pca.pyx:1129-1162). So
//
//   B = [ diag(s) | w |  0 ]     w = column kc of B
//       [    0    |   |  L ]       = (a_0 .. a_{kc-1}, alpha_kc, 0 .. 0)
//
// with L (t x t, t = m - kc) the lower bidiagonal of the tail rows without
// column kc, and
//
//   B B^T = blockdiag(diag(s^2), L L^T) + w w^T.
//
// With L L^T = Q diag(mu) Q^T (the tail's own small SVD, size t), B B^T =
// blockdiag(I, Q) (diag(d) + z z^T) blockdiag(I, Q)^T, d = (s^2, mu), z =
// (a, alpha_kc Q[0, :]). The eigenpairs of diag(d) + z z^T follow the
// divide-and-conquer symmetric eigensolvers (Cuppen 1981; Bunch, Nielsen and
// Sorensen 1978; Gu and Eisenstat, "A stable and efficient algorithm for the
// rank-one modification of the symmetric eigenproblem", 1994):
//  - deflation: a component with |z_l| |z| <= 8 eps max(d_max, |z|^2) keeps
//    (d_l, e_l); of two poles whose coupling after a Givens rotation (which
//    moves z onto one of them) is below the same tolerance, one deflates.
//    Converged Ritz values have residual entries a_l of that size, so their
//    columns of Ub come out exactly e_l;
//  - roots: lambda_i in (d_i, d_{i+1}) solves 1 + sum_l z_l^2 / (d_l - lambda)
//    = 0. Each root is carried as an offset tau from its nearer pole, found by
//    a rational step (that pole exact, the rest linear) inside a bisection
//    bracket, so lambda - d_l is known to full relative accuracy;
//  - vectors: z is recomputed from the roots (Gu-Eisenstat), u_i[l] =
//    zhat_l / (d_l - lambda_i), normalised: orthogonal to working accuracy.
// Everything is FP64. Ub = blockdiag(I, Q) u, sigma = sqrt(lambda), and the
// rows of Vbt are (B^T Ub)_i / sigma_i from B's nonzeros.
//
// The work is O(m^2) plus the tail's SVD (t = m - kc, a few rows late in a
// solve), against the O(m^3) of a full SVD of B. Every reduction is in a
// fixed order, so the result does not depend on timing.
#include <algorithm>
#include <cmath>

#include "svd.cuh"

namespace bgpu {

namespace {

constexpr double kEps = 1.1102230246251565e-16;  // 2^-53

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_prod_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v *= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Tail matrix L_ext (t x (t+1), column-major, FP64 and optionally FP32):
// L[r, c] = B[kc + r, kc + 1 + c]; its column t is zero.
__global__ void k_build_tail(const double* __restrict__ B, uint32_t m, uint32_t kc,
                             double* __restrict__ L64, float* __restrict__ L32) {
  const uint32_t t = m - kc;
  const uint64_t total = (uint64_t)t * (t + 1);
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < total;
       e += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = (uint32_t)(e % t), c = (uint32_t)(e / t);
    const double v = c < t ? B[(kc + r) + (uint64_t)(kc + 1 + c) * m] : 0.0;
    L64[e] = v;
    if (L32) L32[e] = (float)v;
  }
}

// Tails of one or two rows in closed form. The tail's last column is B's
// column m, which stays zero (pca.pyx:1129-1162): t = 1 gives L = [0]; t = 2
// gives L = [[beta, 0], [alpha, 0]], so L L^T = v v^T with v = (beta, alpha).
__global__ void k_tail_small(const double* __restrict__ B, uint32_t m, uint32_t kc,
                             double* __restrict__ Q, double* __restrict__ sig) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const uint32_t t = m - kc;
  if (t == 1) {
    Q[0] = 1.0;
    sig[0] = 0.0;
    return;
  }
  const double beta = B[kc + (uint64_t)(kc + 1) * m];
  const double alpha = B[(kc + 1) + (uint64_t)(kc + 1) * m];
  const double r = hypot(beta, alpha);
  if (r > 0.0) {
    Q[0] = beta / r;   // column 0: v / |v|
    Q[1] = alpha / r;
    Q[2] = -alpha / r; // column 1: v rotated a quarter turn
    Q[3] = beta / r;
  } else {
    Q[0] = 1.0; Q[1] = 0.0; Q[2] = 0.0; Q[3] = 1.0;
  }
  sig[0] = r;
  sig[1] = 0.0;
}

// Poles, sorted ascending, and deflation. One block, in parallel: GB300's
// FP64 latency makes a thread walking the poles one by one the slowest part
// of the merge, so the sums, the single-component test, the close-pole test
// (against each pole's previous surviving pole) and the compaction run
// across the block. Only when some close pair needs a rotation (rare) does
// one thread redo the scan sequentially, as rotations can chain.
__global__ void __launch_bounds__(256)
k_merge_setup(const double* __restrict__ B, uint32_t m, uint32_t kc,
              const double* __restrict__ Q, const double* __restrict__ sig_t,
              MergeWork w) {
  extern __shared__ double sm[];
  double* d0 = sm;      // unsorted d
  double* z0 = d0 + m;  // unsorted z
  double* ds = z0 + m;  // sorted
  double* zs = ds + m;
  int* src = reinterpret_cast<int*>(zs + m);
  int* defl = src + m;
  __shared__ double red[2][8];
  __shared__ double tol_s, znrm_s;
  __shared__ int any_rot, cnt_w[2][8];
  const uint32_t t = m - kc;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const double alpha = B[kc + (uint64_t)kc * m];
  for (uint32_t l = tid; l < m; l += blockDim.x) {
    if (l < kc) {
      const double sv = B[l + (uint64_t)l * m];
      d0[l] = sv * sv;
      z0[l] = B[l + (uint64_t)kc * m];
    } else {
      const uint32_t j = l - kc;
      d0[l] = sig_t[j] * sig_t[j];
      z0[l] = alpha * Q[(uint64_t)j * t];  // row 0 of Q, column j
    }
  }
  if (tid == 0) any_rot = 0;
  __syncthreads();
  for (uint32_t l = tid; l < m; l += blockDim.x) {  // rank sort
    const double dl = d0[l];
    uint32_t rank = 0;
    for (uint32_t q = 0; q < m; ++q) {
      const double dq = d0[q];
      rank += (dq < dl || (dq == dl && q < l)) ? 1u : 0u;
    }
    ds[rank] = dl;
    zs[rank] = z0[l];
    src[rank] = (int)l;
  }
  __syncthreads();
  // |z|^2 and max |d|: per-thread runs, a fixed shuffle tree, warps in order
  {
    double a = 0.0, b = 0.0;
    for (uint32_t l = tid; l < m; l += blockDim.x) {
      a += zs[l] * zs[l];
      b = fmax(b, fabs(ds[l]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    if (lane == 0) { red[0][wid] = a; red[1][wid] = b; }
    __syncthreads();
    if (tid == 0) {
      double zn2 = 0.0, dmax = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
        zn2 += red[0][q];
        dmax = fmax(dmax, red[1][q]);
      }
      znrm_s = sqrt(zn2);
      tol_s = 8.0 * kEps * fmax(dmax, zn2);
    }
    __syncthreads();
  }
  const double tol = tol_s, znrm = znrm_s;
  for (uint32_t l = tid; l < m; l += blockDim.x) defl[l] = fabs(zs[l]) * znrm <= tol;
  __syncthreads();
  for (uint32_t l = tid; l < m; l += blockDim.x) {  // close poles
    if (defl[l]) continue;
    int p = (int)l - 1;
    while (p >= 0 && defl[p]) --p;
    if (p < 0) continue;
    const double zp = zs[p], zq = zs[l];
    const double r = hypot(zp, zq);
    if (fabs((ds[l] - ds[p]) * (zq / r) * (zp / r)) <= tol) any_rot = 1;
  }
  __syncthreads();
  int nrot = 0;
  if (any_rot) {
    if (tid == 0) {  // the sequential scan: rotations can chain
      int prev = -1;
      for (uint32_t l = 0; l < m; ++l) {
        if (defl[l]) continue;
        if (prev >= 0) {
          const double zp = zs[prev], zq = zs[l];
          const double r = hypot(zp, zq);
          const double c = zq / r, sn = zp / r;
          if (fabs((ds[l] - ds[prev]) * c * sn) <= tol) {
            const double dp = ds[prev], dq = ds[l];
            ds[prev] = dp * c * c + dq * sn * sn;
            ds[l] = dp * sn * sn + dq * c * c;
            zs[prev] = 0.0;
            zs[l] = r;
            defl[prev] = 1;
            w.rot_p[nrot] = prev;
            w.rot_q[nrot] = (int)l;
            w.rot_c[nrot] = c;
            w.rot_s[nrot] = sn;
            ++nrot;
          }
        }
        prev = (int)l;
      }
      cnt_w[0][0] = nrot;
    }
    __syncthreads();
    nrot = cnt_w[0][0];
    __syncthreads();
  }
  // compaction in ascending order: per-thread contiguous runs, then offsets
  {
    const uint32_t per = (m + blockDim.x - 1) / blockDim.x;
    const uint32_t a = min(m, tid * per), b2 = min(m, a + per);
    int cd = 0;
    for (uint32_t l = a; l < b2; ++l) cd += defl[l];
    const int cn = (int)(b2 - a) - cd;
    int incl_d = cd, incl_n = cn;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int vd = __shfl_up_sync(0xffffffffu, incl_d, o);
      const int vn = __shfl_up_sync(0xffffffffu, incl_n, o);
      if (lane >= o) { incl_d += vd; incl_n += vn; }
    }
    if (lane == 31) { cnt_w[0][wid] = incl_d; cnt_w[1][wid] = incl_n; }
    __syncthreads();
    int off_d = 0, off_n = 0;
    for (int q = 0; q < wid; ++q) { off_d += cnt_w[0][q]; off_n += cnt_w[1][q]; }
    int pd = off_d + incl_d - cd, pn = off_n + incl_n - cn;
    for (uint32_t l = a; l < b2; ++l) {
      if (defl[l]) {
        w.defpos[pd++] = (int)l;
      } else {
        w.ndpos[pn] = (int)l;
        w.dn[pn] = ds[l];
        w.zn[pn] = zs[l];
        ++pn;
      }
    }
    if (tid == (int)blockDim.x - 1) {
      w.state[0] = pn;
      w.state[1] = nrot;
      w.state[2] = pd;
    }
  }
  __syncthreads();
  {  // |z|^2 over the surviving poles (the last root's bracket)
    double a = 0.0;
    for (uint32_t l = tid; l < m; l += blockDim.x)
      if (!defl[l]) a += zs[l] * zs[l];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) red[0][wid] = a;
    __syncthreads();
    if (tid == 0) {
      double zz = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) zz += red[0][q];
      w.znorm2[0] = zz;
    }
  }
  for (uint32_t l = tid; l < m; l += blockDim.x) {  // for the later kernels
    w.ds[l] = ds[l];
    w.src[l] = src[l];
  }
}

// Secular roots, one warp per root (grid m; blocks past n' return).
__global__ void __launch_bounds__(32)
k_merge_roots(MergeWork w) {
  const int n = w.state[0];
  const int i = blockIdx.x;
  if (i >= n) return;
  const int lane = threadIdx.x;
  int K;
  double lo, hi;
  if (i < n - 1) {
    const double di = w.dn[i], dj = w.dn[i + 1];
    const double half = 0.5 * (dj - di);
    double f = 0.0;
    for (int l = lane; l < n; l += 32) {
      const double zl = w.zn[l];
      f += zl * zl / ((w.dn[l] - di) - half);
    }
    f = 1.0 + warp_sum_d(f);
    if (f >= 0.0) {  // root in (d_i, d_i + half]
      K = i;
      lo = 0.0;
      hi = half;
    } else {  // root in (d_i + half, d_{i+1})
      K = i + 1;
      lo = (di + half) - dj;
      hi = 0.0;
    }
  } else {
    K = n - 1;
    lo = 0.0;
    hi = w.znorm2[0];
  }
  const double dK = w.dn[K];
  const double zK2 = w.zn[K] * w.zn[K];
  const bool right = K > i;  // tau < 0
  double tau = 0.5 * (lo + hi);
  for (int it = 0; it < 300; ++it) {
    double phi = 0.0, dphi = 0.0, mag = 0.0;
    for (int l = lane; l < n; l += 32) {
      if (l == K) continue;
      const double zl = w.zn[l];
      const double q = (w.dn[l] - dK) - tau;
      const double term = zl * zl / q;
      phi += term;
      dphi += term / q;
      mag += fabs(term);
    }
    phi = warp_sum_d(phi);
    dphi = warp_sum_d(dphi);
    mag = warp_sum_d(mag);
    const double pole = -zK2 / tau;  // z_K^2 / (0 - tau)
    const double F = 1.0 + phi + pole;
    if (F == 0.0) break;
    if (F < 0.0) lo = tau; else hi = tau;
    // converged: |F| within the rounding of its terms, or the bracket down
    // to the last bits of tau
    if (fabs(F) <= 16.0 * kEps * (1.0 + mag + fabs(pole))) break;
    if (hi - lo <= 4.0 * kEps * fmax(fabs(lo), fabs(hi))) break;
    // model 1 + phi(tau) + phi'(tau) (x - tau) - z_K^2 / x = 0, i.e.
    // phi' x^2 + c0 x - z_K^2 = 0; the root on the side of the pole
    const double c0 = 1.0 + phi - dphi * tau;
    double x;
    if (dphi > 0.0) {
      const double disc = sqrt(c0 * c0 + 4.0 * dphi * zK2);
      if (!right)
        x = c0 > 0.0 ? 2.0 * zK2 / (c0 + disc) : (disc - c0) / (2.0 * dphi);
      else
        x = c0 < 0.0 ? -2.0 * zK2 / (disc - c0) : -(c0 + disc) / (2.0 * dphi);
    } else {
      x = c0 != 0.0 ? zK2 / c0 : 0.5 * (lo + hi);
    }
    if (!(x > lo && x < hi)) {  // outside the bracket (or NaN): bisect
      const double alo = fabs(lo), ahi = fabs(hi);
      const double mn = fmin(alo, ahi), mx = fmax(alo, ahi);
      if (mn > 0.0 && mx > 4.0 * mn)
        x = (right ? -1.0 : 1.0) * sqrt(mn * mx);  // geometric across scales
      else
        x = 0.5 * (lo + hi);
    }
    if (x == tau) break;
    tau = x;
  }
  if (lane == 0) {
    w.korig[i] = K;
    w.tau[i] = tau;
  }
}

// Gu-Eisenstat zhat, one warp per pole: zhat_l^2 = (lambda_{n-1} - d_l)
// prod_{i<l} (lambda_i - d_l)/(d_i - d_l) prod_{l<=i<n-1} (lambda_i - d_l)/
// (d_{i+1} - d_l), every factor positive by interlacing.
__global__ void __launch_bounds__(32)
k_merge_zhat(MergeWork w) {
  const int n = w.state[0];
  const int l = blockIdx.x;
  if (l >= n) return;
  const int lane = threadIdx.x;
  const double dl = w.dn[l];
  double p = 1.0;
  for (int i = lane; i < n; i += 32) {
    const double lam_dl = (w.dn[w.korig[i]] - dl) + w.tau[i];  // lambda_i - d_l
    double f;
    if (i == n - 1) f = lam_dl;
    else if (i < l) f = lam_dl / (w.dn[i] - dl);
    else f = lam_dl / (w.dn[i + 1] - dl);
    p *= f;
  }
  p = warp_prod_d(p);
  if (lane == 0) w.zhat[l] = copysign(sqrt(fabs(p)), w.zn[l]);
}

// Eigenvalue of every eigen id (roots first, then deflated poles) and the
// descending order (ties by id). One block.
__global__ void __launch_bounds__(256)
k_merge_order(uint32_t m, MergeWork w) {
  extern __shared__ double lam[];
  const int n = w.state[0];
  for (uint32_t id = threadIdx.x; id < m; id += blockDim.x)
    lam[id] = (int)id < n ? w.dn[w.korig[id]] + w.tau[id] : w.ds[w.defpos[id - n]];
  __syncthreads();
  for (uint32_t id = threadIdx.x; id < m; id += blockDim.x) {
    const double li = lam[id];
    uint32_t rank = 0;
    for (uint32_t q = 0; q < m; ++q) {
      const double lq = lam[q];
      rank += (lq > li || (lq == li && q < id)) ? 1u : 0u;
    }
    w.order[rank] = (int)id;
    w.lam[id] = li;
  }
}

// Output column r (descending order): Ub[:, r], Sb[r], Vbt[r, :] and the
// FP64 last-row entry and singular value the convergence test reads.
__global__ void __launch_bounds__(128)
k_merge_vectors(const double* __restrict__ B, uint32_t m, uint32_t kc,
                const double* __restrict__ Q, MergeWork w, float* __restrict__ Ub,
                float* __restrict__ Sb, float* __restrict__ Vbt,
                double* __restrict__ ub_last, double* __restrict__ sb64) {
  extern __shared__ double sm[];
  double* x = sm;     // sorted coordinates
  double* u = x + m;  // output column
  double* yt = u + m; // tail coordinates before Q
  __shared__ double red[4];
  __shared__ double scal;
  const uint32_t r = blockIdx.x;
  const uint32_t t = m - kc;
  const int n = w.state[0];
  const int nrot = w.state[1];
  const int id = w.order[r];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (uint32_t l = tid; l < m; l += blockDim.x) x[l] = 0.0;
  __syncthreads();
  double lam;
  if (id < n) {
    const int K = w.korig[id];
    const double tau = w.tau[id], dK = w.dn[K];
    double ss = 0.0;
    for (int a = tid; a < n; a += blockDim.x) {
      const double v = w.zhat[a] / ((w.dn[a] - dK) - tau);
      x[w.ndpos[a]] = v;
      ss += v * v;
    }
    ss = warp_sum_d(ss);
    if (lane == 0) red[wid] = ss;
    __syncthreads();
    if (tid == 0) scal = 1.0 / sqrt(((red[0] + red[1]) + red[2]) + red[3]);
    __syncthreads();
    for (int a = tid; a < n; a += blockDim.x) x[w.ndpos[a]] *= scal;
    lam = dK + tau;
  } else {
    const int pos = w.defpos[id - n];
    if (tid == 0) x[pos] = 1.0;
    lam = w.ds[pos];
  }
  __syncthreads();
  if (tid == 0) {  // undo the deflation rotations, last first
    for (int k = nrot - 1; k >= 0; --k) {
      const int p = w.rot_p[k], q = w.rot_q[k];
      const double c = w.rot_c[k], sn = w.rot_s[k];
      const double xp = x[p], xq = x[q];
      x[p] = c * xp + sn * xq;
      x[q] = -sn * xp + c * xq;
    }
  }
  __syncthreads();
  for (uint32_t a = tid; a < m; a += blockDim.x) {
    const uint32_t o = (uint32_t)w.src[a];
    if (o < kc) u[o] = x[a];
    else yt[o - kc] = x[a];
  }
  __syncthreads();
  for (uint32_t row = tid; row < t; row += blockDim.x) {
    double acc = 0.0;
    for (uint32_t j = 0; j < t; ++j) acc = fma(Q[row + (uint64_t)j * t], yt[j], acc);
    u[kc + row] = acc;
  }
  __syncthreads();
  const double sig = sqrt(fmax(lam, 0.0));
  const double inv = sig > 0.0 ? 1.0 / sig : 0.0;
  for (uint32_t row = tid; row < m; row += blockDim.x)
    Ub[row + (uint64_t)r * m] = (float)u[row];
  if (tid == 0) {
    Sb[r] = (float)sig;
    sb64[r] = sig;
    ub_last[r] = u[m - 1];
  }
  // Vbt[r, c] = (B^T u)[c] / sigma: column c of B holds B[c, c] (c < m),
  // B[c-1, c] (c > kc) and, for c = kc, the residual entries of rows < kc.
  for (uint32_t c = tid; c <= m; c += blockDim.x) {
    if (c == kc) continue;
    double v;
    if (c < kc) {
      v = B[c + (uint64_t)c * m] * u[c];
    } else {
      v = B[(c - 1) + (uint64_t)c * m] * u[c - 1];
      if (c < m) v = fma(B[c + (uint64_t)c * m], u[c], v);
    }
    Vbt[r + (uint64_t)c * m] = (float)(v * inv);
  }
  double acc = 0.0;
  for (uint32_t row = tid; row <= kc; row += blockDim.x)
    acc = fma(B[row + (uint64_t)kc * m], u[row], acc);
  acc = warp_sum_d(acc);
  if (lane == 0) red[wid] = acc;
  __syncthreads();
  if (tid == 0)
    Vbt[r + (uint64_t)kc * m] = (float)((((red[0] + red[1]) + red[2]) + red[3]) * inv);
}

}  // namespace

size_t merge_work_bytes(uint32_t m) {
  return (size_t)m * (10 * 8 + 9 * 4) + 256;  // 10 double and 9 int arrays
}

static MergeWork merge_work_carve(void* base, uint32_t m) {
  MergeWork w;
  double* d = reinterpret_cast<double*>(base);
  double** dp[] = {&w.ds, &w.zs, &w.dn, &w.zn, &w.tau, &w.zhat, &w.lam,
                   &w.rot_c, &w.rot_s, &w.znorm2};
  for (double** q : dp) { *q = d; d += m; }
  int* i = reinterpret_cast<int*>(d);
  int** ip[] = {&w.src, &w.defl, &w.ndpos, &w.defpos, &w.rot_p, &w.rot_q,
                &w.korig, &w.order, &w.state};
  for (int** q : ip) { *q = i; i += m; }
  return w;
}

size_t tail_work_bytes(uint32_t m) {
  const size_t mm1 = (size_t)m * (m + 1), mm = (size_t)m * m;
  // FP64 L_ext, Q, last row, singular values; FP32 L_ext, Ub, Vbt, Sb
  return mm1 * 8 + mm * 8 + 2 * (size_t)m * 8 + mm1 * 4 + mm * 4 + mm1 * 4 +
         (size_t)m * 4 + 256;
}

int launch_svd_merge(const double* B, uint32_t m, uint32_t kc, float* Ub, float* Sb,
                     float* Vbt, double* ub_last, double* sb64, void* tailw,
                     void* mergew, double* refine_work, void* jacobi_gwork,
                     int refine_steps, cudaStream_t s) {
  BGPU_REQUIRE(kc >= 1 && kc < m, BGPU_ERR_INVALID, "merge SVD needs 1 <= kc < m");
  const uint32_t t = m - kc;
  const uint64_t tt1 = (uint64_t)t * (t + 1);
  char* p = reinterpret_cast<char*>(tailw);
  auto take = [&](size_t bytes) {
    char* q = p;
    p += bytes;
    return q;
  };
  double* L64 = reinterpret_cast<double*>(take((size_t)m * (m + 1) * 8));
  double* Q64 = reinterpret_cast<double*>(take((size_t)m * m * 8));
  double* ubl_t = reinterpret_cast<double*>(take((size_t)m * 8));
  double* sb_t = reinterpret_cast<double*>(take((size_t)m * 8));
  float* L32 = reinterpret_cast<float*>(take((size_t)m * (m + 1) * 4));
  float* Ub_t = reinterpret_cast<float*>(take((size_t)m * m * 4));
  float* Vbt_t = reinterpret_cast<float*>(take((size_t)m * (m + 1) * 4));
  float* Sb_t = reinterpret_cast<float*>(take((size_t)m * 4));
  const MergeWork w = merge_work_carve(mergew, m);

  // 1. the tail's SVD: closed forms for one or two rows, else FP32 Jacobi +
  //    FP64 Newton refinement at size t (an FP64 Jacobi of even a 3-12 row
  //    tail takes longer on this GPU: its rotations are serial FP64 chains)
  if (t <= kMergeClosedTailMax) {
    k_tail_small<<<1, 32, 0, s>>>(B, m, kc, Q64, sb_t);
    BGPU_CHECK_LAUNCH();
  } else {
    const unsigned tb = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(tt1, 256),
                                                                          1024));
    k_build_tail<<<tb, 256, 0, s>>>(B, m, kc, L64, L32);
    BGPU_CHECK_LAUNCH();
    BGPU_TRY(launch_jacobi_svd(L32, nullptr, t, Ub_t, Sb_t, Vbt_t, nullptr, nullptr,
                               jacobi_gwork, nullptr, s));
    BGPU_TRY(launch_svd_refine(L64, t, Ub_t, Sb_t, Vbt_t, ubl_t, sb_t, refine_work,
                               refine_steps, s, Q64));
  }
  // 2. the merge
  k_merge_setup<<<1, 256, (size_t)4 * m * 8 + (size_t)2 * m * 4, s>>>(B, m, kc, Q64,
                                                                      sb_t, w);
  BGPU_CHECK_LAUNCH();
  k_merge_roots<<<m, 32, 0, s>>>(w);
  BGPU_CHECK_LAUNCH();
  k_merge_zhat<<<m, 32, 0, s>>>(w);
  BGPU_CHECK_LAUNCH();
  k_merge_order<<<1, 256, (size_t)m * 8, s>>>(m, w);
  BGPU_CHECK_LAUNCH();
  const size_t vsm = (size_t)3 * m * 8;
  if (vsm > 48 * 1024)
    BGPU_CUDA(cudaFuncSetAttribute(k_merge_vectors,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vsm));
  k_merge_vectors<<<m, 128, vsm, s>>>(B, m, kc, Q64, w, Ub, Sb, Vbt, ub_last, sb64);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
