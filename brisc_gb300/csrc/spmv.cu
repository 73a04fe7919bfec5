// Sparse products on the device layout (matrix.cuh).
//
//  X.v     (brisc/pca.pyx:440-475 matvec_csr_parallel_raw): one group of G lanes
//          per cell row, 128-bit loads of four packed entries starting on a
//          4-entry boundary (the row head and tail are masked), the normalised
//          value log1pf(count * isf[cell]) computed in registers, the gene
//          weight v[gene] / sd[gene] read from shared memory.
//  X^T.u   (brisc/pca.pyx:478-511 rmatvec_csc_parallel_raw): one CTA per
//          (row panel, gene group). The panel's u and size factors are staged
//          in shared memory, so the per-entry gathers hit shared memory instead
//          of L2; one warp reduces one gene's segment (a warp-segmented
//          reduction, no atomics) into a per-panel partial (gene-major
//          layout); a second pass adds the partials of all panels in panel
//          order. These register-vector kernels serve layouts outside the
//          streaming kernels' limits (stream.cu).
//  gene sd (brisc/pca.pyx:51-103 clipped_stddev_csc): same panel traversal,
//          FP64 sums.
#include <algorithm>

#include "matrix.cuh"

namespace bgpu {

namespace {

template <int G, int MODE>
__global__ void __launch_bounds__(256)
k_spmv(CsrView X, const float* __restrict__ v, const float* __restrict__ sd,
       float* __restrict__ y) {
  extern __shared__ float w[];
  for (uint32_t c = threadIdx.x; c < X.g; c += blockDim.x)
    w[c] = sd ? v[c] / sd[c] : v[c];  // pca.pyx:461-462
  __syncthreads();

  constexpr int kRowsPerWarp = 32 / G;
  const int lane = threadIdx.x & (G - 1);
  const int grp = (threadIdx.x & 31) / G;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  // bit 31 of a stored word flags a row head when genes fit in 15 bits
  const uint32_t gm = X.g > 32768u ? 0xffffu : 0x7fffu;
  const uint64_t nbatches = ceil_div_dev(X.n, kRowsPerWarp);
  for (uint64_t bt = warp; bt < nbatches; bt += nwarps) {
    const uint64_t r = bt * kRowsPerWarp + grp;
    const bool valid = r < X.n;
    int64_t e0 = 0, e1 = 0;
    if (valid) { e0 = X.rowptr[r]; e1 = X.rowptr[r + 1]; }
    float acc = 0.f;
    if constexpr (MODE == kCounts) {
      const float f = valid ? X.isf[r] : 0.f;
#pragma unroll 4
      for (int64_t b = (e0 & ~3LL) + 4 * lane; b < e1; b += 4 * G) {
        const uint4 q = ld_stream_u4(X.packed + b);
        const uint32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int64_t e = b + k;
          if (e >= e0 && e < e1)
            acc += norm_count(qq[k] & 0xffffu, f) * w[(qq[k] >> 16) & gm];
        }
      }
    } else {
#pragma unroll 4
      for (int64_t b = (e0 & ~3LL) + 4 * lane; b < e1; b += 4 * G) {
        const uint4 qv = ld_stream_u4(X.val + b);
        const uint2 qc = ld_stream_u2(X.col + b);
        const float vv[4] = {__uint_as_float(qv.x), __uint_as_float(qv.y),
                             __uint_as_float(qv.z), __uint_as_float(qv.w)};
        const uint32_t cc[4] = {qc.x & 0xffffu, qc.x >> 16, qc.y & 0xffffu,
                                qc.y >> 16};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int64_t e = b + k;
          if (e >= e0 && e < e1) acc += vv[k] * w[cc[k]];
        }
      }
    }
    acc = group_sum<G>(acc);
    if (valid && lane == 0) y[r] = X.post ? acc * X.post[r] : acc;
  }
}

template <int MODE>
__global__ void __launch_bounds__(256)
k_rmat_partials(CscView X, const float* __restrict__ u,
                const float* __restrict__ u_scale, float* __restrict__ u_out,
                float* __restrict__ partials, uint32_t colgroup) {
  extern __shared__ float sm[];
  const uint32_t P = 1u << X.pshift;
  const uint32_t p = blockIdx.x;
  const uint64_t r0 = (uint64_t)p << X.pshift;
  const uint32_t rows = (uint32_t)min_u64(P, X.n - r0);
  float* us = sm;
  float* fs = sm + P;
  const float scale = u_scale ? *u_scale : 1.f;
  const bool write_u = u_out && blockIdx.y == 0;
  for (uint32_t i = threadIdx.x; i < rows; i += blockDim.x) {
    const float uu = u_scale ? u[r0 + i] * scale : u[r0 + i];
    if (write_u) u_out[r0 + i] = uu;
    if constexpr (MODE == kCounts) {
      fs[i] = X.isf[r0 + i];
      us[i] = X.post ? uu * X.post[r0 + i] : uu;
    } else {
      us[i] = uu;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int64_t pbase = X.rowptr[r0];
  const int32_t* cp = X.colptr + (uint64_t)p * (X.g + 1);
  const uint32_t c0 = blockIdx.y * colgroup;
  const uint32_t c1 = min(X.g, c0 + colgroup);
  for (uint32_t c = c0 + wid; c < c1; c += nw) {
    const int64_t e0 = pbase + cp[c], e1 = pbase + cp[c + 1];
    float acc = 0.f;
    if constexpr (MODE == kCounts) {
#pragma unroll 4
      for (int64_t b = (e0 & ~3LL) + 4 * lane; b < e1; b += 128) {
        const uint4 q = ld_stream_u4(X.packed + b);
        const uint32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int64_t e = b + k;
          if (e >= e0 && e < e1) {
            const uint32_t lr = (qq[k] >> 16) & (P - 1);  // bit 31 may flag a segment head
            acc += norm_count(qq[k] & 0xffffu, fs[lr]) * us[lr];
          }
        }
      }
    } else {
#pragma unroll 4
      for (int64_t b = (e0 & ~3LL) + 4 * lane; b < e1; b += 128) {
        const uint4 qv = ld_stream_u4(X.val + b);
        const uint2 qr = ld_stream_u2(X.row + b);
        const float vv[4] = {__uint_as_float(qv.x), __uint_as_float(qv.y),
                             __uint_as_float(qv.z), __uint_as_float(qv.w)};
        const uint32_t rr[4] = {qr.x & 0xffffu, qr.x >> 16, qr.y & 0xffffu,
                                qr.y >> 16};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int64_t e = b + k;
          if (e >= e0 && e < e1) acc += vv[k] * us[rr[k]];
        }
      }
    }
    acc = warp_sum(acc);
    if (lane == 0) partials[(uint64_t)c * X.num_panels + p] = acc;
  }
}

template <int MODE>
__global__ void __launch_bounds__(256)
k_gene_moments(CscView X, double2* __restrict__ partials, uint32_t colgroup) {
  extern __shared__ float sm[];
  const uint32_t P = 1u << X.pshift;
  const uint32_t p = blockIdx.x;
  const uint64_t r0 = (uint64_t)p << X.pshift;
  const uint32_t rows = (uint32_t)min_u64(P, X.n - r0);
  float* fs = sm;
  float* qs = sm + P;
  if constexpr (MODE == kCounts) {
    for (uint32_t i = threadIdx.x; i < rows; i += blockDim.x) {
      fs[i] = X.isf[r0 + i];
      qs[i] = X.post ? X.post[r0 + i] : 1.f;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int64_t pbase = X.rowptr[r0];
  const int32_t* cp = X.colptr + (uint64_t)p * (X.g + 1);
  const uint32_t c0 = blockIdx.y * colgroup;
  const uint32_t c1 = min(X.g, c0 + colgroup);
  for (uint32_t c = c0 + wid; c < c1; c += nw) {
    const int64_t e0 = pbase + cp[c], e1 = pbase + cp[c + 1];
    double s1 = 0.0, s2 = 0.0;
    for (int64_t b = (e0 & ~3LL) + 4 * lane; b < e1; b += 128) {
      float vals[4];
      if constexpr (MODE == kCounts) {
        const uint4 q = ld_stream_u4(X.packed + b);
        const uint32_t qq[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const uint32_t lr = (qq[k] >> 16) & (P - 1);  // bit 31 may flag a segment head
          const int64_t e = b + k;
          vals[k] = (e >= e0 && e < e1)
                        ? (X.post ? norm_count(qq[k] & 0xffffu, fs[lr]) * qs[lr]
                                  : norm_count(qq[k] & 0xffffu, fs[lr]))
                        : 0.f;
        }
      } else {
        const uint4 qv = ld_stream_u4(X.val + b);
        const float vv[4] = {__uint_as_float(qv.x), __uint_as_float(qv.y),
                             __uint_as_float(qv.z), __uint_as_float(qv.w)};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int64_t e = b + k;
          vals[k] = (e >= e0 && e < e1) ? vv[k] : 0.f;
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        s1 += (double)vals[k];
        s2 += (double)vals[k] * (double)vals[k];
      }
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) partials[(uint64_t)p * X.g + c] = make_double2(s1, s2);
  }
}

__global__ void k_gene_sd(const double2* __restrict__ partials,
                          uint32_t num_panels, uint32_t g, uint64_t n,
                          float* __restrict__ sd) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g) return;
  double s1 = 0.0, s2 = 0.0;
  for (uint32_t p = 0; p < num_panels; ++p) {
    double2 t = partials[(uint64_t)p * g + c];
    s1 += t.x;
    s2 += t.y;
  }
  const double dn = (double)n;
  // pca.pyx:83-86: sqrt((n * sum_sq - sum^2) / (n (n - 1))), clipped at 1e-8
  double var = (dn * s2 - s1 * s1) / (dn * (dn - 1.0));
  float s = (float)sqrt(var > 0.0 ? var : 0.0);
  sd[c] = s < 1e-8f ? 1e-8f : s;
}

}  // namespace

double matvec_bytes(const Matrix& m) {
  if (m.sell) {  // stream, per-position factors and descriptors, v, sd, y
    const double npos = (double)m.xv.groups * 32.0;
    return (double)m.xv.total_units * 8.0 + npos * (4.0 + 4.0 + 2.0) +
           (m.post ? npos * 4.0 : 0.0) + m.xv.groups * 6.0 + m.g * 8.0 + m.n * 4.0;
  }
  double per = m.mode == kCounts ? 4.0 : 6.0;
  double b = m.nnz * per + (m.n + 1) * 8.0 + m.n * 4.0 + m.g * 8.0;
  if (m.mode == kCounts) b += m.n * 4.0 * (m.post ? 2 : 1);
  return b;
}

double rmatvec_bytes(const Matrix& m) {
  if (m.sell) {  // stream, descriptors, u (read and written scaled), isf, partials
    const double groups = (double)m.xt.groups;
    return (double)m.xt.total_units * 8.0 + m.n * 12.0 + (m.post ? m.n * 4.0 : 0.0) +
           (double)m.xt.ctas * m.g * 4.0 + groups * 70.0 + m.xt.panels * 8.0;
  }
  double per = m.mode == kCounts ? 4.0 : 6.0;
  double b = m.nnz * per + (double)m.num_panels * (m.g + 1) * 4.0 + m.n * 4.0 +
             (double)m.num_panels * m.g * 4.0;
  if (m.mode == kCounts) b += m.n * 4.0 * (m.post ? 2 : 1);
  return b;
}

int launch_matvec(const Matrix& m, const float* v, const float* sd, float* y,
                  cudaStream_t s) {
  const CsrView X = csr_view(m);
  const int blocks = m.spmv_blocks > 0 ? m.spmv_blocks : num_sms() * 8;
  const size_t smem = (size_t)m.g * sizeof(float);
#define BGPU_SPMV_CASE(GG)                                                    \
  case GG:                                                                      \
    if (m.mode == kCounts) {                                                    \
      if (smem > 48 * 1024)                                                     \
        BGPU_CUDA(allow_max_smem(k_spmv<GG, kCounts>));                          \
      k_spmv<GG, kCounts><<<blocks, 256, smem, s>>>(X, v, sd, y);               \
    } else {                                                                    \
      if (smem > 48 * 1024)                                                     \
        BGPU_CUDA(allow_max_smem(k_spmv<GG, kFloat>));                           \
      k_spmv<GG, kFloat><<<blocks, 256, smem, s>>>(X, v, sd, y);                \
    }                                                                           \
    break;
  switch (m.spmv_group) {
    BGPU_SPMV_CASE(2)
    BGPU_SPMV_CASE(4)
    BGPU_SPMV_CASE(8)
    BGPU_SPMV_CASE(16)
    BGPU_SPMV_CASE(32)
    default:
      set_error("unsupported SpMV group size");
      return BGPU_ERR_INVALID;
  }
#undef BGPU_SPMV_CASE
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_rmatvec_partials(const Matrix& m, const float* u,
                            const float* u_scale_dev, float* u_out,
                            float* partials, cudaStream_t s) {
  const CscView X = csc_view(m);
  const uint32_t cg = m.rmat_colgroup;
  dim3 grid(m.num_panels, (unsigned)ceil_div(m.g, cg));
  const size_t smem = (size_t)m.P * 2 * sizeof(float);
  if (m.mode == kCounts) {
    if (smem > 48 * 1024)
      BGPU_CUDA(allow_max_smem(k_rmat_partials<kCounts>));
    k_rmat_partials<kCounts><<<grid, 256, smem, s>>>(X, u, u_scale_dev, u_out,
                                                     partials, cg);
  } else {
    if (smem > 48 * 1024)
      BGPU_CUDA(allow_max_smem(k_rmat_partials<kFloat>));
    k_rmat_partials<kFloat><<<grid, 256, smem, s>>>(X, u, u_scale_dev, u_out,
                                                    partials, cg);
  }
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_gene_stddev(const Matrix& m, double* partials, float* sd,
                       cudaStream_t s) {
  if (m.sell) {  // per-CTA moments over the sliced-ELL panels, CTA order
    BGPU_TRY(launch_xt_moments(m, partials, s));
    k_gene_sd<<<(unsigned)ceil_div(m.g, 256), 256, 0, s>>>(
        (const double2*)partials, m.num_panels, m.g, m.n, sd);
    BGPU_CHECK_LAUNCH();
    return BGPU_OK;
  }
  const CscView X = csc_view(m);
  const uint32_t cg = m.rmat_colgroup;
  dim3 grid(m.num_panels, (unsigned)ceil_div(m.g, cg));
  const size_t smem = (size_t)m.P * 2 * sizeof(float);
  if (m.mode == kCounts) {
    if (smem > 48 * 1024)
      BGPU_CUDA(allow_max_smem(k_gene_moments<kCounts>));
    k_gene_moments<kCounts><<<grid, 256, smem, s>>>(X, (double2*)partials, cg);
  } else {
    if (smem > 48 * 1024)
      BGPU_CUDA(allow_max_smem(k_gene_moments<kFloat>));
    k_gene_moments<kFloat><<<grid, 256, smem, s>>>(X, (double2*)partials, cg);
  }
  BGPU_CHECK_LAUNCH();
  k_gene_sd<<<(unsigned)ceil_div(m.g, 256), 256, 0, s>>>(
      (const double2*)partials, m.num_panels, m.g, m.n, sd);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
