// Sparse products with the fused normalisation (counts layout).
//
// X.v   (brisc/pca.pyx:440-475): 8 lanes own a cell row (about 13 of the
//       row's ~100 entries per lane, so per-row work is amortised). The row's
//       count table (tab[c] = log1pf(c * isf[cell]) for 1 <= c < 16, tab[0] =
//       0, precomputed once per matrix) goes into a padded per-group
//       shared-memory slot, so a count selects its normalised value with one
//       conflict-free load; the next row's offsets are prefetched, and two
//       128-bit loads of packed entries are in flight per lane. The value is
//       exactly log1pf(count * isf), the reference's normalize_csr value
//       (brisc/normalize.pyx:81).
// X^T.u (brisc/pca.pyx:478-511): one CTA per 1024-row panel of the transposed
//       copy. The panel's count table (64 KB, laid out [count][row]) arrives by
//       one bulk copy (TMA) while u * scale (* post) and the panel's gene
//       offsets are staged; 8-lane groups then stream gene segments with
//       128-bit loads and reduce each into partials[gene][panel].
//
// Every loaded word is folded into a per-lane OR; a row or segment holding a
// count >= 16 (beyond the tables) is summed again by an exact out-of-line
// routine, so the common loop carries no per-entry branch. Words of a
// 16-byte window that lie outside the row/segment (only in its first and
// last windows) are zeroed, and a zero word reads table slot 0, which is 0.
//
// Sums: each lane adds its entries in entry order, then a fixed xor tree. The
// result depends only on the data and the layout, not on timing or launch
// shape, so repeated products are bit-identical.
#include <algorithm>
#include <vector>

#include "matrix.cuh"
#include "tma.cuh"

namespace bgpu {

namespace {

__host__ __device__ constexpr uint32_t r128(uint32_t b) { return (b + 127u) & ~127u; }

// Validity mask of the 4 entries of the 16-byte window starting at entry b
// for a segment [e0, e1): bit j set iff e0 <= b + j < e1.
__device__ __forceinline__ uint32_t window_mask(int64_t b, int64_t e0, int64_t e1) {
  const int lo = (int)max(min(e0 - b, (int64_t)4), (int64_t)0);
  const int hi = (int)max(min(e1 - b, (int64_t)4), (int64_t)0);
  return ((1u << hi) - 1u) & ~((1u << lo) - 1u);
}

// Zero the words of a 16-byte window outside [lo, hi) (positions 0..3).
__device__ __forceinline__ uint4 clip_window(uint4 q, int lo, int hi) {
  q.x = (0 >= lo && 0 < hi) ? q.x : 0u;
  q.y = (1 >= lo && 1 < hi) ? q.y : 0u;
  q.z = (2 >= lo && 2 < hi) ? q.z : 0u;
  q.w = (3 >= lo && 3 < hi) ? q.w : 0u;
  return q;
}

// Exact sums for a row (or segment) that holds a count beyond the tables
// (0.03 % of stored counts on count data): the same per-lane entry order as
// the table path, log1pf for the large counts. Out of line so the common loop
// stays small.
__device__ __noinline__ float csr_row_exact8(const uint32_t* __restrict__ packed,
                                             int64_t e0, int64_t e1,
                                             const float* __restrict__ tb, float isf,
                                             const float* __restrict__ w, int lane8) {
  float acc = 0.f;
  for (int64_t b = (e0 & ~3ll) + 4 * lane8; b - 4 * lane8 < e1; b += 32) {
    const uint4 r4 = b < e1 ? ld_stream_u4(packed + b) : make_uint4(0, 0, 0, 0);
    const uint32_t vm = window_mask(b, e0, e1);
    const uint32_t qq[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t cnt = qq[j] & 0xffffu;
      const float val = cnt < (uint32_t)kCountTab ? tb[cnt] : norm_count(cnt, isf);
      if (vm & (1u << j)) acc += val * w[qq[j] >> 16];
    }
  }
  return acc;
}

__device__ __noinline__ float csc_seg_exact8(const uint32_t* __restrict__ packed,
                                             int64_t e0, int64_t e1,
                                             const float* __restrict__ tab,
                                             const float* __restrict__ us,
                                             const float* __restrict__ isf_rows,
                                             uint32_t pshift, int lane8) {
  float acc = 0.f;
  for (int64_t b = (e0 & ~3ll) + 4 * lane8; b - 4 * lane8 < e1; b += 32) {
    const uint4 r4 = b < e1 ? ld_stream_u4(packed + b) : make_uint4(0, 0, 0, 0);
    const uint32_t vm = window_mask(b, e0, e1);
    const uint32_t qq[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t lr = qq[j] >> 16, cnt = qq[j] & 0xffffu;
      const float val = cnt < (uint32_t)kCountTab ? tab[(cnt << pshift) + lr]
                                                  : norm_count(cnt, isf_rows[lr]);
      if (vm & (1u << j)) acc += val * us[lr];
    }
  }
  return acc;
}

// ---------------------------------------------------------------------------
// X.v, counts layout: 8 lanes per cell row.
constexpr int kTabSlot = 17;  // padded per-group table slot (conflict-free)

__global__ void __launch_bounds__(256, 5)
k_spmv_rows(CsrView X, const float* __restrict__ v, const float* __restrict__ sd,
            float* __restrict__ y) {
  extern __shared__ __align__(16) float sm[];
  float* w = sm;                                       // g floats
  float* tabs = sm + ((X.g + 3) & ~3u);                // 32 groups x 2 x kTabSlot
  for (uint32_t c = threadIdx.x; c < X.g; c += blockDim.x)
    w[c] = sd ? v[c] / sd[c] : v[c];  // pca.pyx:461-462
  __syncthreads();

  const int lane8 = threadIdx.x & 7;
  const unsigned gmask = 0xFFu << (threadIdx.x & 24);
  const uint32_t gslot = (threadIdx.x >> 3) * 2 * kTabSlot;
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 3;
  const uint64_t ngroups = (gridDim.x * (uint64_t)blockDim.x) >> 3;
  const float2* rt2 = reinterpret_cast<const float2*>(X.rtab);

  int64_t nx0 = 0, nx1 = 0;  // prefetched offsets of the next row
  if (gid < X.n) { nx0 = X.rowptr[gid]; nx1 = X.rowptr[gid + 1]; }
  int buf = 0;
  for (uint64_t r = gid; r < X.n; r += ngroups, buf ^= 1) {
    const int64_t e0 = nx0, e1 = nx1;
    const uint64_t rn = r + ngroups;
    if (rn < X.n) { nx0 = X.rowptr[rn]; nx1 = X.rowptr[rn + 1]; }
    // the row's count table into this group's (double-buffered) slot
    float* tb = tabs + gslot + buf * kTabSlot;
    const float2 t2 = rt2[r * (kCountTab / 2) + lane8];
    tb[2 * lane8] = t2.x;
    tb[2 * lane8 + 1] = t2.y;
    __syncwarp(gmask);
    // row-relative 32-bit offsets: the row's words are [lead, len) of the
    // 16-byte-aligned span starting at a0
    const int64_t a0 = e0 & ~3ll;
    const uint32_t* rowp = X.packed + a0;
    const int lead = (int)(e0 - a0), len = (int)(e1 - a0);
    float acc = 0.f;
    uint32_t big = 0;  // OR of the loaded words: a count >= 16 shows in 0xfff0
    auto consume = [&](uint4 q, int at) {
      if (at < lead || at + 4 > len) q = clip_window(q, lead - at, len - at);
      big |= q.x | q.y | q.z | q.w;
      acc = fmaf(tb[q.x & (kCountTab - 1)], w[q.x >> 16], acc);
      acc = fmaf(tb[q.y & (kCountTab - 1)], w[q.y >> 16], acc);
      acc = fmaf(tb[q.z & (kCountTab - 1)], w[q.z >> 16], acc);
      acc = fmaf(tb[q.w & (kCountTab - 1)], w[q.w >> 16], acc);
    };
    for (int o = 4 * lane8; o - 4 * lane8 < len; o += 64) {
      const uint4 q0 = o < len ? ld_stream_u4(rowp + o) : make_uint4(0, 0, 0, 0);
      const uint4 q1 = o + 32 < len ? ld_stream_u4(rowp + o + 32) : make_uint4(0, 0, 0, 0);
      if (o < len) consume(q0, o);
      if (o + 32 < len) consume(q1, o + 32);
    }
    if (__any_sync(gmask, (big & 0xfff0u) != 0u))
      acc = csr_row_exact8(X.packed, e0, e1, tb, X.isf[r], w, lane8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
    if (lane8 == 0) y[r] = X.post ? acc * X.post[r] : acc;
  }
}

// ---------------------------------------------------------------------------
// X^T.u, counts layout: 8 lanes per (panel, gene) segment.
struct PanelLayout {
  uint32_t tab, us, cps, total;
  __host__ __device__ PanelLayout(uint32_t P, uint32_t g) {
    tab = 128;
    us = tab + r128(P * kCountTab * 4);
    cps = us + r128(P * 4);
    total = cps + r128((g + 1) * 4);
  }
};

__global__ void __launch_bounds__(512, 2)
k_rmat_panels(CscView X, const float* __restrict__ u, const float* __restrict__ u_scale,
              float* __restrict__ u_out, float* __restrict__ partT,
              int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t P = 1u << X.pshift;
  const PanelLayout L(P, X.g);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  const float* tab = reinterpret_cast<const float*>(smem + L.tab);  // [c][row]
  float* us = reinterpret_cast<float*>(smem + L.us);
  int32_t* cps = reinterpret_cast<int32_t*>(smem + L.cps);

  const uint32_t p = blockIdx.x;
  const uint64_t r0 = (uint64_t)p << X.pshift;
  const uint32_t rows = (uint32_t)min_u64(P, X.n - r0);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    fence_mbar_init();
    const uint32_t tb = P * kCountTab * 4;
    mbar_arrive_expect_tx(&bar[0], tb);
    bulk_g2s(smem + L.tab, X.rtab + (uint64_t)p * kCountTab * P, tb, &bar[0]);
  }
  const float scale = u_scale ? *u_scale : 1.f;
  for (uint32_t i = threadIdx.x; i < rows; i += blockDim.x) {
    const float uu = u_scale ? u[r0 + i] * scale : u[r0 + i];
    if (u_out) u_out[r0 + i] = uu;
    us[i] = X.post ? uu * X.post[r0 + i] : uu;
  }
  for (uint32_t i = rows + threadIdx.x; i < P; i += blockDim.x) us[i] = 0.f;
  const int32_t* cp = X.colptr + (uint64_t)p * (X.g + 1);
  for (uint32_t c = threadIdx.x; c <= X.g; c += blockDim.x) cps[c] = cp[c];
  __syncthreads();  // barrier initialised, us/cps staged
  const bool ok = __syncthreads_and(mbar_wait(&bar[0], 0, err));
  if (!ok) return;  // every thread waited (bounded) for the copy

  const int64_t pbase = X.rowptr[r0];
  const int lane8 = threadIdx.x & 7;
  const unsigned gmask = 0xFFu << (threadIdx.x & 24);
  const uint32_t pshift = X.pshift;
  for (uint32_t c = threadIdx.x >> 3; c < X.g; c += blockDim.x >> 3) {
    const int64_t e0 = pbase + cps[c], e1 = pbase + cps[c + 1];
    const int64_t a0 = e0 & ~3ll;
    const uint32_t* segp = X.packed + a0;
    const int lead = (int)(e0 - a0), len = (int)(e1 - a0);
    float acc = 0.f;
    uint32_t big = 0;
    auto consume = [&](uint4 q, int at) {
      if (at < lead || at + 4 > len) q = clip_window(q, lead - at, len - at);
      big |= q.x | q.y | q.z | q.w;
      // a zeroed word reads tab[0][row 0] = 0
      acc = fmaf(tab[((q.x & (kCountTab - 1)) << pshift) + (q.x >> 16)], us[q.x >> 16], acc);
      acc = fmaf(tab[((q.y & (kCountTab - 1)) << pshift) + (q.y >> 16)], us[q.y >> 16], acc);
      acc = fmaf(tab[((q.z & (kCountTab - 1)) << pshift) + (q.z >> 16)], us[q.z >> 16], acc);
      acc = fmaf(tab[((q.w & (kCountTab - 1)) << pshift) + (q.w >> 16)], us[q.w >> 16], acc);
    };
    for (int o = 4 * lane8; o - 4 * lane8 < len; o += 64) {
      const uint4 q0 = o < len ? ld_stream_u4(segp + o) : make_uint4(0, 0, 0, 0);
      const uint4 q1 = o + 32 < len ? ld_stream_u4(segp + o + 32) : make_uint4(0, 0, 0, 0);
      if (o < len) consume(q0, o);
      if (o + 32 < len) consume(q1, o + 32);
    }
    if (__any_sync(gmask, (big & 0xfff0u) != 0u))
      acc = csc_seg_exact8(X.packed, e0, e1, tab, us, X.isf + r0, pshift, lane8);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
    if (lane8 == 0) partT[(uint64_t)c * X.num_panels + p] = acc;
  }
}

// z[c] = (sum over panels in panel order of partT[c][p]) / sd[c]; one warp per
// gene, lanes stride the panels, fixed xor tree.
__global__ void __launch_bounds__(256)
k_reduce_panels_t(const float* __restrict__ partT, uint32_t num_panels,
                  uint32_t g, const float* __restrict__ sd,
                  float* __restrict__ z) {
  const int lane = threadIdx.x & 31;
  const uint32_t c = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (c >= g) return;
  const float* row = partT + (uint64_t)c * num_panels;
  float t = 0.f;
  for (uint32_t p = lane; p < num_panels; p += 32) t += row[p];
  t = warp_sum(t);
  if (lane == 0) z[c] = sd ? t / sd[c] : t;  // pca.pyx:510-511
}

// Count tables (matrix creation): tab[c] = log1pf(c * isf) for 1 <= c < 16,
// tab[0] = 0 so that a zeroed (masked) word adds nothing.
__global__ void k_count_tables(const float* __restrict__ isf, uint64_t n,
                               uint32_t pshift, float* __restrict__ rtab_r,
                               float* __restrict__ rtab_c) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n * kCountTab) return;
  const uint64_t r = i / kCountTab;
  const uint32_t c = (uint32_t)(i % kCountTab);
  const float f = isf[r];
  const float v = c ? norm_count(c, f) : 0.f;
  rtab_r[i] = v;
  const uint64_t P = 1ull << pshift;
  const uint64_t p = r >> pshift, lr = r & (P - 1);
  rtab_c[(p * kCountTab + c) * P + lr] = v;
}

}  // namespace

bool stream_supported(const Matrix& m) {
  return m.mode == kCounts && m.P <= 2048 &&
         PanelLayout(m.P, m.g).total <= 113 * 1024;
}

int build_stream_tiles(Matrix* m, const std::vector<int64_t>& panel_rowptr,
                       cudaStream_t s, uint64_t* bytes_acc) {
  (void)panel_rowptr;
  if (!stream_supported(*m)) return BGPU_OK;
  const uint64_t nr = m->n * kCountTab;
  const uint64_t nc = (uint64_t)m->num_panels * kCountTab * m->P;
  BGPU_CUDA(cudaMalloc((void**)&m->rtab_r, nr * 4));
  BGPU_CUDA(cudaMalloc((void**)&m->rtab_c, nc * 4));
  *bytes_acc += (nr + nc) * 4;
  BGPU_CUDA(cudaMemsetAsync(m->rtab_c, 0, nc * 4, s));
  k_count_tables<<<(unsigned)ceil_div(nr, 256), 256, 0, s>>>(
      m->isf, m->n, m->pshift, m->rtab_r, m->rtab_c);
  BGPU_CHECK_LAUNCH();
  m->stream_ok = true;
  return BGPU_OK;
}

int launch_matvec_stream(const Matrix& m, const float* v, const float* sd,
                         float* y, int* err, cudaStream_t s) {
  (void)err;
  const CsrView X = csr_view(m);
  const size_t smem = ((size_t)((m.g + 3) & ~3u) + 32 * 2 * kTabSlot) * 4;
  if (smem > 48 * 1024)
    BGPU_CUDA(cudaFuncSetAttribute(k_spmv_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
  k_spmv_rows<<<num_sms() * 5, 256, smem, s>>>(X, v, sd, y);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_rmatvec_stream(const Matrix& m, const float* u, const float* u_scale,
                          float* u_out, float* partT, int* err, cudaStream_t s) {
  const CscView X = csc_view(m);
  const size_t smem = PanelLayout(m.P, m.g).total;
  BGPU_CUDA(cudaFuncSetAttribute(k_rmat_panels, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  k_rmat_panels<<<m.num_panels, 512, smem, s>>>(X, u, u_scale, u_out, partT, err);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_reduce_panels_t(const Matrix& m, const float* partT, const float* sd,
                           float* z, cudaStream_t s) {
  k_reduce_panels_t<<<(unsigned)ceil_div(m.g, 8), 256, 0, s>>>(
      partT, m.num_panels, m.g, sd, z);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
