// k-nearest-neighbour search over cluster-sorted principal components: the
// reference's knn_self (brisc/knn.pyx:13-515), the search half of
// SingleCell.neighbors() (brisc/single_cell.py:12139-12665). Its inputs are
// the k-means results neighbors() prepares: the PCs grouped by cluster, the
// centroids, the cluster sizes and each cell's squared norm.
//
// Same search as the reference, the same candidates in the same order:
//  1. nearest clusters: for each cell, the num_clusters_searched centroids
//     with the smallest partial distance |c|^2 - 2 x.c, candidates visited in
//     ascending centroid order and kept while strictly smaller than the
//     current worst (the reference's max-heap of knn.pyx:150-185);
//  2. neighbours: for each cell, every cell of those clusters except itself,
//     visited by ascending cluster label and then ascending position, with
//     distance |x|^2 + (|c|^2 - 2 x.c) and the same strict-improvement rule
//     (knn.pyx:186-290); the lists come out sorted by ascending distance and
//     the neighbour ids are mapped through sorted_order.
// The dot products are FP32 fused multiply-adds in dimension order; the
// reference's come from sgemm, so distances agree to FP32 rounding of the
// norms and neighbours can differ only where two candidates' distances do.
//
// GPU shape:
//  - k_knn_nearest: 8 warps per CTA, 4 cells per warp. The CTA streams the
//    centroids through shared memory in tiles of 128 ([dim][centroid]: each
//    lane reads its own centroid, conflict-free) and every warp keeps the
//    running best list of its 4 cells spread over its lanes (one slot per
//    lane per 32 entries), replacing the current worst as candidates beat it.
//  - k_knn_search: 32 consecutive cells per CTA (consecutive in cluster
//    order, so they share most of their nearest clusters). The union of their
//    clusters is built in shared memory (a per-cluster bit mask of the cells
//    that search it, compacted in label order), and each cluster's cells are
//    staged in tiles of 64 rows; each warp evaluates its 4 cells against the
//    tile (two candidates per lane) and keeps each cell's best list the same
//    way. Cells that do not search a cluster ignore its candidates.
// No atomics on floating-point data and no order-dependent reductions: the
// result depends only on the inputs.
#include <algorithm>
#include <cfloat>
#include <vector>

#include "common.cuh"
#include "pcg.h"

namespace bgpu {

namespace {

constexpr int kKnnThreads = 256;
constexpr int kKnnWarps = kKnnThreads / 32;
constexpr int kQPerWarp = 4;
constexpr int kQPerCta = kKnnWarps * kQPerWarp;  // 32
constexpr int kCentTile = 128;
constexpr int kCellTile = 64;
constexpr uint32_t kMaxDims = 128;
constexpr uint32_t kMaxSearched = 256;  // 8 slots per lane
constexpr uint32_t kMaxNeighbors = 128; // 4 slots per lane
constexpr uint32_t kMaxClusters = 32768;

// Row stride (floats) of staged rows: a multiple of 4 whose float4 count is
// odd, so 32 lanes reading float4s of 32 different rows hit every bank pair
// once.
__host__ __device__ inline uint32_t row_stride(uint32_t d) {
  uint32_t s = (d + 3u) & ~3u;
  if (((s >> 2) & 1u) == 0u) s += 4u;
  return s;
}

// A best list of up to 32 * R entries spread over the lanes of a warp: entry
// e lives in lane e % 32, slot e / 32. Entries past the list size hold -inf
// and are never the worst.
template <int R>
struct WarpBest {
  float d[R];
  uint32_t id[R];
  float worst;       // warp-uniform
  int worst_lane, worst_slot;

  __device__ void init(uint32_t size, int lane) {
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const uint32_t e = (uint32_t)s * 32u + (uint32_t)lane;
      d[s] = e < size ? FLT_MAX : -INFINITY;
      id[s] = 0xFFFFFFFFu;
    }
    find_worst(lane);
  }
  // the largest entry; ties go to the lowest entry index
  __device__ void find_worst(int lane) {
    float best = -INFINITY;
    int bs = 0;
#pragma unroll
    for (int s = 0; s < R; ++s)
      if (d[s] > best) { best = d[s]; bs = s; }
    int be = bs * 32 + lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oe = __shfl_xor_sync(0xffffffffu, be, o);
      if (ob > best || (ob == best && oe < be)) { best = ob; be = oe; }
    }
    worst = best;
    worst_lane = be & 31;
    worst_slot = be >> 5;
  }
  // Offers the candidates of the lanes in `mask` in ascending lane order.
  __device__ void offer(float cand, uint32_t cid, unsigned mask, int lane) {
    mask &= __ballot_sync(0xffffffffu, cand < worst);
    while (mask) {
      const int src = __ffs(mask) - 1;
      mask &= mask - 1u;
      const float cd = __shfl_sync(0xffffffffu, cand, src);
      const uint32_t ci = __shfl_sync(0xffffffffu, cid, src);
      if (cd < worst) {  // strict, as the reference's heap
        if (lane == worst_lane) {
#pragma unroll
          for (int s = 0; s < R; ++s)
            if (s == worst_slot) { d[s] = cd; id[s] = ci; }
        }
        find_worst(lane);
        mask &= __ballot_sync(0xffffffffu, cand < worst);
      }
    }
  }
  // Writes the list sorted by (distance, id) ascending; scratch holds 32 * R
  // floats and 32 * R ids of this warp.
  __device__ void write_sorted(uint32_t size, float* sd, uint32_t* si, float* out_d,
                               uint32_t* out_id, const uint32_t* id_map, int lane) {
#pragma unroll
    for (int s = 0; s < R; ++s) {
      sd[s * 32 + lane] = d[s];
      si[s * 32 + lane] = id[s];
    }
    __syncwarp();
    for (uint32_t e = lane; e < size; e += 32) {
      const float de = sd[e];
      const uint32_t ie = si[e];
      uint32_t rank = 0;
      for (uint32_t f = 0; f < size; ++f) {
        const float df = sd[f];
        const uint32_t idf = si[f];
        rank += (df < de || (df == de && (idf < ie || (idf == ie && f < e)))) ? 1u : 0u;
      }
      out_d[rank] = de;
      out_id[rank] = (id_map && ie != 0xFFFFFFFFu) ? id_map[ie] : ie;
    }
    __syncwarp();
  }
};

__global__ void k_knn_centroid_norms(const float* __restrict__ C, uint32_t nc,
                                     uint32_t d, float* __restrict__ cn) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nc) return;
  const float* c = C + (uint64_t)i * d;
  float s = c[0] * c[0];
  for (uint32_t j = 1; j < d; ++j) s = fmaf(c[j], c[j], s);
  cn[i] = s;
}

// Cluster offsets (exclusive prefix sum of the sizes) and their total.
__global__ void k_knn_offsets(const uint32_t* __restrict__ sizes, uint32_t nc,
                              uint64_t* __restrict__ off) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  uint64_t s = 0;
  for (uint32_t i = 0; i < nc; ++i) {
    off[i] = s;
    s += sizes[i];
  }
  off[nc] = s;
}

template <int R>
__global__ void __launch_bounds__(kKnnThreads)
k_knn_nearest(const float* __restrict__ X, uint64_t n, uint32_t d,
              const float* __restrict__ C, const float* __restrict__ cn, uint32_t nc,
              uint32_t cs, uint32_t* __restrict__ nearest, float* __restrict__ cdist) {
  extern __shared__ __align__(16) float sm[];
  const uint32_t xs = (d + 3u) & ~3u;
  float* ct = sm;                            // [d][kCentTile]
  float* xq = ct + (size_t)d * kCentTile;    // [kQPerCta][xs]
  float* sdist = xq + (size_t)kQPerCta * xs;  // per warp 32 R
  uint32_t* sid = reinterpret_cast<uint32_t*>(sdist + kKnnWarps * 32 * R);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t q0 = (uint64_t)blockIdx.x * kQPerCta;
  for (uint32_t t = threadIdx.x; t < (uint32_t)kQPerCta * xs; t += kKnnThreads) {
    const uint32_t q = t / xs, j = t % xs;
    xq[t] = (q0 + q < n && j < d) ? X[(q0 + q) * d + j] : 0.f;
  }
  WarpBest<R> best[kQPerWarp];
#pragma unroll
  for (int i = 0; i < kQPerWarp; ++i) best[i].init(cs, lane);
  for (uint32_t t0 = 0; t0 < nc; t0 += kCentTile) {
    const uint32_t tn = min((uint32_t)kCentTile, nc - t0);
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < d * kCentTile; t += kKnnThreads) {
      const uint32_t c = t / d, j = t % d;  // coalesced along the centroid rows
      ct[(size_t)j * kCentTile + c] = c < tn ? C[(uint64_t)(t0 + c) * d + j] : 0.f;
    }
    __syncthreads();
    for (uint32_t c0 = 0; c0 < tn; c0 += 32) {
      const uint32_t c = c0 + lane;
      float acc[kQPerWarp];
#pragma unroll
      for (int i = 0; i < kQPerWarp; ++i) acc[i] = 0.f;
      for (uint32_t j = 0; j < d; j += 4) {
        float cv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          cv[u] = j + u < d ? ct[(size_t)(j + u) * kCentTile + c] : 0.f;
#pragma unroll
        for (int i = 0; i < kQPerWarp; ++i) {
          const float4 x4 =
              *reinterpret_cast<const float4*>(xq + (size_t)(wid * kQPerWarp + i) * xs + j);
          acc[i] = fmaf(x4.x, cv[0], acc[i]);
          acc[i] = fmaf(x4.y, cv[1], acc[i]);
          acc[i] = fmaf(x4.z, cv[2], acc[i]);
          acc[i] = fmaf(x4.w, cv[3], acc[i]);
        }
      }
      const bool valid = c < tn;
      const float cnc = valid ? cn[t0 + c] : 0.f;
      const unsigned vm = __ballot_sync(0xffffffffu, valid);
#pragma unroll
      for (int i = 0; i < kQPerWarp; ++i) {
        const float pd = fmaf(-2.f, acc[i], cnc);  // |c|^2 - 2 x.c
        best[i].offer(valid ? pd : FLT_MAX, t0 + c, vm, lane);
      }
    }
  }
  float* wd = sdist + wid * 32 * R;
  uint32_t* wi = sid + wid * 32 * R;
#pragma unroll
  for (int i = 0; i < kQPerWarp; ++i) {
    const uint64_t q = q0 + (uint64_t)wid * kQPerWarp + i;
    if (q < n)
      best[i].write_sorted(cs, wd, wi, cdist + q * cs, nearest + q * cs, nullptr, lane);
  }
}

template <int R>
__global__ void __launch_bounds__(kKnnThreads)
k_knn_search(const float* __restrict__ X, uint64_t n, uint32_t d,
             const float* __restrict__ norms, const uint32_t* __restrict__ sorted_order,
             const uint64_t* __restrict__ coff, uint32_t nc,
             const uint32_t* __restrict__ nearest, uint32_t cs, uint32_t k,
             uint32_t* __restrict__ nbr, float* __restrict__ dist) {
  extern __shared__ __align__(16) float sm[];
  const uint32_t st = row_stride(d);
  float* tile = sm;                                    // [kCellTile][st]
  float* xq = tile + (size_t)kCellTile * st;           // [kQPerCta][st]
  float* tnorm = xq + (size_t)kQPerCta * st;           // [kCellTile]
  uint32_t* masks = reinterpret_cast<uint32_t*>(tnorm + kCellTile);  // [nc]
  uint32_t* ulab = masks + nc;                         // [kQPerCta * cs]
  float* sdist = reinterpret_cast<float*>(ulab + (size_t)kQPerCta * cs);
  uint32_t* sid = reinterpret_cast<uint32_t*>(sdist + kKnnWarps * 32 * R);
  __shared__ uint32_t wsum[kKnnWarps + 1];
  __shared__ uint32_t nunion;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t q0 = (uint64_t)blockIdx.x * kQPerCta;
  const uint32_t nq = (uint32_t)(n - q0 < (uint64_t)kQPerCta ? n - q0 : (uint64_t)kQPerCta);

  for (uint32_t t = threadIdx.x; t < (uint32_t)kQPerCta * st; t += kKnnThreads) {
    const uint32_t q = t / st, j = t % st;
    xq[t] = (q < nq && j < d) ? X[(q0 + q) * d + j] : 0.f;
  }
  for (uint32_t c = threadIdx.x; c < nc; c += kKnnThreads) masks[c] = 0u;
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < nq * cs; t += kKnnThreads) {
    const uint32_t q = t / cs;
    const uint32_t lab = nearest[(q0 + q) * cs + (t % cs)];
    if (lab < nc) atomicOr(&masks[lab], 1u << q);  // integer OR: order-free
  }
  __syncthreads();
  // compact the searched clusters in ascending label order: each thread
  // takes a contiguous run of labels
  {
    const uint32_t per = (nc + kKnnThreads - 1) / kKnnThreads;
    const uint32_t a = min(nc, threadIdx.x * per), b = min(nc, a + per);
    uint32_t cnt = 0;
    for (uint32_t c = a; c < b; ++c) cnt += masks[c] != 0u;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t s = 0;
      for (int w = 0; w < kKnnWarps; ++w) {
        const uint32_t v = wsum[w];
        wsum[w] = s;
        s += v;
      }
      nunion = s;
    }
    __syncthreads();
    uint32_t pos = wsum[wid] + incl - cnt;
    for (uint32_t c = a; c < b; ++c)
      if (masks[c] != 0u) ulab[pos++] = c;
  }
  __syncthreads();

  WarpBest<R> best[kQPerWarp];
#pragma unroll
  for (int i = 0; i < kQPerWarp; ++i) best[i].init(k, lane);
  float qn[kQPerWarp];
  uint64_t qid[kQPerWarp];
#pragma unroll
  for (int i = 0; i < kQPerWarp; ++i) {
    const uint32_t q = wid * kQPerWarp + i;
    qid[i] = q0 + q;
    qn[i] = q < nq ? norms[q0 + q] : 0.f;
  }
  const uint32_t nu = nunion;
  for (uint32_t u = 0; u < nu; ++u) {
    const uint32_t lab = ulab[u];
    const uint32_t qmask = masks[lab];
    const uint64_t cb = coff[lab], ce = coff[lab + 1];
    for (uint64_t r0 = cb; r0 < ce; r0 += kCellTile) {
      const uint32_t tn = (uint32_t)(ce - r0 < (uint64_t)kCellTile ? ce - r0 : (uint64_t)kCellTile);
      __syncthreads();  // previous tile consumed
      // rows past the cluster and the padding columns d..st are zeroed: the
      // float4 dot reads them (times zero query entries)
      for (uint32_t t = threadIdx.x; t < (uint32_t)kCellTile * st; t += kKnnThreads) {
        const uint32_t r = t / st, j = t % st;
        tile[t] = (r < tn && j < d) ? X[(r0 + r) * d + j] : 0.f;
      }
      for (uint32_t t = threadIdx.x; t < (uint32_t)kCellTile; t += kKnnThreads)
        tnorm[t] = t < tn ? norms[r0 + t] : 0.f;
      __syncthreads();
      if (((qmask >> (wid * kQPerWarp)) & 0xFu) == 0u) continue;  // warp-uniform
      float acc0[kQPerWarp], acc1[kQPerWarp];
#pragma unroll
      for (int i = 0; i < kQPerWarp; ++i) { acc0[i] = 0.f; acc1[i] = 0.f; }
      const float* t0p = tile + (size_t)lane * st;
      const float* t1p = tile + (size_t)(lane + 32) * st;
      for (uint32_t j = 0; j < d; j += 4) {
        const float4 a = *reinterpret_cast<const float4*>(t0p + j);
        const float4 b = *reinterpret_cast<const float4*>(t1p + j);
#pragma unroll
        for (int i = 0; i < kQPerWarp; ++i) {
          const float4 x4 =
              *reinterpret_cast<const float4*>(xq + (size_t)(wid * kQPerWarp + i) * st + j);
          acc0[i] = fmaf(x4.x, a.x, acc0[i]);
          acc0[i] = fmaf(x4.y, a.y, acc0[i]);
          acc0[i] = fmaf(x4.z, a.z, acc0[i]);
          acc0[i] = fmaf(x4.w, a.w, acc0[i]);
          acc1[i] = fmaf(x4.x, b.x, acc1[i]);
          acc1[i] = fmaf(x4.y, b.y, acc1[i]);
          acc1[i] = fmaf(x4.z, b.z, acc1[i]);
          acc1[i] = fmaf(x4.w, b.w, acc1[i]);
        }
      }
      const bool v0 = (uint32_t)lane < tn, v1 = (uint32_t)lane + 32u < tn;
      const float n0 = tnorm[lane], n1 = tnorm[lane + 32];
      const uint64_t cell0 = r0 + lane, cell1 = r0 + lane + 32;
#pragma unroll
      for (int i = 0; i < kQPerWarp; ++i) {
        if (!((qmask >> (wid * kQPerWarp + i)) & 1u)) continue;  // warp-uniform
        const float d0 = qn[i] + fmaf(-2.f, acc0[i], n0);
        const float d1 = qn[i] + fmaf(-2.f, acc1[i], n1);
        const unsigned m0 = __ballot_sync(0xffffffffu, v0 && cell0 != qid[i]);
        const unsigned m1 = __ballot_sync(0xffffffffu, v1 && cell1 != qid[i]);
        best[i].offer(d0, (uint32_t)cell0, m0, lane);
        best[i].offer(d1, (uint32_t)cell1, m1, lane);
      }
    }
  }
  float* wd = sdist + wid * 32 * R;
  uint32_t* wi = sid + wid * 32 * R;
#pragma unroll
  for (int i = 0; i < kQPerWarp; ++i) {
    if (wid * kQPerWarp + i < (int)nq)
      best[i].write_sorted(k, wd, wi, dist + qid[i] * k, nbr + qid[i] * k, sorted_order,
                           lane);
  }
}

template <int R>
int launch_nearest(const float* X, uint64_t n, uint32_t d, const float* C,
                   const float* cn, uint32_t nc, uint32_t cs, uint32_t* nearest,
                   float* cdist, cudaStream_t s) {
  const size_t smem = ((size_t)d * kCentTile + (size_t)kQPerCta * ((d + 3) & ~3u) +
                       (size_t)kKnnWarps * 32 * R * 2) * 4;
  BGPU_CUDA(allow_max_smem(k_knn_nearest<R>));
  k_knn_nearest<R><<<(unsigned)ceil_div(n, kQPerCta), kKnnThreads, smem, s>>>(
      X, n, d, C, cn, nc, cs, nearest, cdist);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

size_t search_smem(uint32_t d, uint32_t nc, uint32_t cs, int R) {
  const uint32_t st = row_stride(d);
  return ((size_t)kCellTile * st + (size_t)kQPerCta * st + kCellTile) * 4 +
         (size_t)nc * 4 + (size_t)kQPerCta * cs * 4 + (size_t)kKnnWarps * 32 * R * 8;
}

template <int R>
int launch_search(const float* X, uint64_t n, uint32_t d, const float* norms,
                  const uint32_t* so, const uint64_t* coff, uint32_t nc,
                  const uint32_t* nearest, uint32_t cs, uint32_t k, uint32_t* nbr,
                  float* dist, cudaStream_t s) {
  const size_t smem = search_smem(d, nc, cs, R);
  BGPU_REQUIRE(smem <= (size_t)device_smem_optin() - 256, BGPU_ERR_UNSUPPORTED,
               "knn_self: too many clusters for the search's shared-memory cluster table");
  BGPU_CUDA(allow_max_smem(k_knn_search<R>));
  k_knn_search<R><<<(unsigned)ceil_div(n, kQPerCta), kKnnThreads, smem, s>>>(
      X, n, d, norms, so, coff, nc, nearest, cs, k, nbr, dist);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace

}  // namespace bgpu

using namespace bgpu;

extern "C" int bgpu_knn_self(const float* X, const uint32_t* sorted_order,
                             const float* centroids,
                             const uint32_t* num_cells_per_cluster, uint32_t* neighbors,
                             float* distances, const float* cell_norms,
                             float* centroid_distances, uint32_t* nearest_clusters,
                             uint64_t num_cells, uint32_t num_dimensions,
                             uint32_t num_clusters, uint32_t num_neighbors,
                             uint32_t num_clusters_searched, void* stream) {
  BGPU_REQUIRE(X && sorted_order && centroids && num_cells_per_cluster && neighbors &&
                   distances && cell_norms && centroid_distances && nearest_clusters,
               BGPU_ERR_INVALID, "knn_self: NULL argument");
  BGPU_REQUIRE(num_cells >= 2 && num_dimensions >= 1 && num_clusters >= 1,
               BGPU_ERR_INVALID, "knn_self: needs >= 2 cells, >= 1 dimension and cluster");
  BGPU_REQUIRE(num_neighbors >= 1 && num_neighbors < num_cells, BGPU_ERR_INVALID,
               "knn_self: num_neighbors must be >= 1 and less than the number of cells");
  BGPU_REQUIRE(num_clusters_searched >= 1 && num_clusters_searched <= num_clusters,
               BGPU_ERR_INVALID,
               "knn_self: num_clusters_searched must be >= 1 and <= the number of clusters");
  BGPU_REQUIRE(num_dimensions <= kMaxDims, BGPU_ERR_UNSUPPORTED,
               "knn_self: at most 128 dimensions");
  BGPU_REQUIRE(num_clusters_searched <= kMaxSearched, BGPU_ERR_UNSUPPORTED,
               "knn_self: num_clusters_searched must be <= 256");
  BGPU_REQUIRE(num_neighbors <= kMaxNeighbors, BGPU_ERR_UNSUPPORTED,
               "knn_self: num_neighbors must be <= 128");
  BGPU_REQUIRE(num_clusters <= kMaxClusters, BGPU_ERR_UNSUPPORTED,
               "knn_self: at most 32768 clusters");
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t n = num_cells;
  const uint32_t d = num_dimensions, nc = num_clusters, cs = num_clusters_searched,
                 k = num_neighbors;
  float* cn = nullptr;
  uint64_t* coff = nullptr;
  BGPU_CUDA(cudaMallocAsync((void**)&cn, (size_t)nc * 4, s));
  BGPU_CUDA(cudaMallocAsync((void**)&coff, ((size_t)nc + 1) * 8, s));
  int rc = BGPU_OK;
  k_knn_centroid_norms<<<(unsigned)ceil_div(nc, 256), 256, 0, s>>>(centroids, nc, d, cn);
  k_knn_offsets<<<1, 32, 0, s>>>(num_cells_per_cluster, nc, coff);
  if (cudaGetLastError() != cudaSuccess) rc = BGPU_ERR_CUDA;
  uint64_t total = 0;
  if (rc == BGPU_OK &&
      cudaMemcpyAsync(&total, coff + nc, 8, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
      cudaStreamSynchronize(s) == cudaSuccess) {
    if (total != n) {
      set_error("knn_self: num_cells_per_cluster does not sum to the number of cells");
      rc = BGPU_ERR_INVALID;
    }
  } else if (rc == BGPU_OK) {
    set_error("knn_self: could not read the cluster sizes");
    rc = BGPU_ERR_CUDA;
  }
  if (rc == BGPU_OK) {
    if (cs <= 32)
      rc = launch_nearest<1>(X, n, d, centroids, cn, nc, cs, nearest_clusters,
                             centroid_distances, s);
    else if (cs <= 64)
      rc = launch_nearest<2>(X, n, d, centroids, cn, nc, cs, nearest_clusters,
                             centroid_distances, s);
    else if (cs <= 128)
      rc = launch_nearest<4>(X, n, d, centroids, cn, nc, cs, nearest_clusters,
                             centroid_distances, s);
    else
      rc = launch_nearest<8>(X, n, d, centroids, cn, nc, cs, nearest_clusters,
                             centroid_distances, s);
  }
  if (rc == BGPU_OK) {
    if (k <= 32)
      rc = launch_search<1>(X, n, d, cell_norms, sorted_order, coff, nc,
                            nearest_clusters, cs, k, neighbors, distances, s);
    else if (k <= 64)
      rc = launch_search<2>(X, n, d, cell_norms, sorted_order, coff, nc,
                            nearest_clusters, cs, k, neighbors, distances, s);
    else
      rc = launch_search<4>(X, n, d, cell_norms, sorted_order, coff, nc,
                            nearest_clusters, cs, k, neighbors, distances, s);
  }
  cudaFreeAsync(cn, s);
  cudaFreeAsync(coff, s);
  if (rc == BGPU_OK) BGPU_CUDA(cudaStreamSynchronize(s));
  return rc;
}

// ---------------------------------------------------------------------------
// k-means: the reference's kmeans (brisc/kmeans.pyx:889-1433), random
// initialisation (its default, kmeans_random_init, kmeans.pyx:13-38), for
// neighbors() to cluster the PCs on the device before knn_self.
//  - init: num_clusters distinct random cells, drawn with PCG32 + Lemire's
//    bounded integers from srand(seed) exactly as the reference draws them
//    (host), gathered on the device;
//  - |x|^2 per cell (kmeans.pyx:954-965), a dimension-ordered float sum;
//  - E step: the nearest centroid by partial distance |c|^2 - 2 x.c, first
//    minimum in centroid order wins (kmeans.pyx:1016-1041) -- k_knn_nearest
//    with one cluster searched;
//  - M step: the sums of each chunk of chunk_size cells per cluster, each a
//    sequence over the chunk's cells in order, then the chunks added in
//    chunk order (kmeans.pyx:1043-1064): the reference's own order, so with
//    the same assignments the centroids are bit-identical; empty clusters
//    take the cells farthest from their centroids (kmeans.pyx:747-820, on
//    the host: it is rare and sequential); the sums are scaled by
//    (float)(1.0 / count);
//  - stop after num_kmeans_iterations, or when the float total of |x|^2 +
//    min distance falls by less than tolerance (kmeans.pyx:1082-1098, summed
//    in cell order on the host);
//  - a final E step for the labels, min distances and counts.
// The centroid buffers swap every iteration as the reference's do: the
// final centroids are in centroids_new when the returned count is odd.
namespace bgpu {
namespace {

__global__ void k_km_cell_norms(const float* __restrict__ X, uint64_t n, uint32_t d,
                                float* __restrict__ out) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* x = X + i * d;
  float s = x[0] * x[0];
  for (uint32_t j = 1; j < d; ++j) s = fmaf(x[j], x[j], s);
  out[i] = s;
}

__global__ void k_km_gather(const float* __restrict__ X, const uint32_t* __restrict__ idx,
                            uint32_t nc, uint32_t d, float* __restrict__ C) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t >= (uint64_t)nc * d) return;
  const uint32_t c = (uint32_t)(t / d), j = (uint32_t)(t % d);
  C[t] = X[(uint64_t)idx[c] * d + j];
}

// One CTA per chunk, one thread per dimension: sums[chunk][label][dim] over
// the chunk's cells in order (zeroed beforehand).
__global__ void k_km_chunk_sums(const float* __restrict__ X, uint64_t n, uint32_t d,
                                const uint32_t* __restrict__ labels, uint32_t chunk,
                                uint32_t nc, float* __restrict__ sums) {
  const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
  const uint64_t c1 = c0 + chunk < n ? c0 + chunk : n;
  float* base = sums + (uint64_t)blockIdx.x * nc * d;
  for (uint32_t j = threadIdx.x; j < d; j += blockDim.x)
    for (uint64_t i = c0; i < c1; ++i) {
      float* p = base + (uint64_t)labels[i] * d + j;
      *p = *p + X[i * d + j];
    }
}

// centroids_new[c][j] = 0 + the chunk sums in chunk order.
__global__ void k_km_reduce(const float* __restrict__ sums, uint32_t nchunks, uint32_t nc,
                            uint32_t d, float* __restrict__ Cn) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t per = (uint64_t)nc * d;
  if (t >= per) return;
  float s = 0.f;
  for (uint32_t ch = 0; ch < nchunks; ++ch) s += sums[ch * per + t];
  Cn[t] = s;
}

__global__ void k_km_counts(const uint32_t* __restrict__ labels, uint64_t n,
                            uint32_t* __restrict__ counts) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&counts[labels[i]], 1u);  // integer: order-free
}

__global__ void k_km_normalize(float* __restrict__ Cn, const uint32_t* __restrict__ counts,
                               uint32_t nc, uint32_t d) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (t >= (uint64_t)nc * d) return;
  const uint32_t cnt = counts[t / d];
  if (cnt > 0) Cn[t] *= (float)(1.0 / (double)cnt);  // kmeans.pyx:1070-1074
}

// Squared distance of each cell to its assigned centroid, a dimension-ordered
// float sum (relocate_empty_clusters, kmeans.pyx:785-791).
__global__ void k_km_assigned(const float* __restrict__ X, const uint32_t* __restrict__ lab,
                              const float* __restrict__ C, uint64_t n, uint32_t d,
                              float* __restrict__ out) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* x = X + i * d;
  const float* c = C + (uint64_t)lab[i] * d;
  float diff = x[0] - c[0];
  float s = diff * diff;
  for (uint32_t j = 1; j < d; ++j) {
    diff = x[j] - c[j];
    s = fmaf(diff, diff, s);
  }
  out[i] = s;
}

// E step: labels, min distances (= partial distances) and, when counts is
// given, the cluster sizes.
int km_estep(const float* X, uint64_t n, uint32_t d, const float* C, float* cn,
             uint32_t nc, uint32_t* labels, float* mind, uint32_t* counts, cudaStream_t s) {
  k_knn_centroid_norms<<<(unsigned)ceil_div(nc, 256), 256, 0, s>>>(C, nc, d, cn);
  BGPU_CHECK_LAUNCH();
  BGPU_TRY(launch_nearest<1>(X, n, d, C, cn, nc, 1, labels, mind, s));
  if (counts) {
    BGPU_CUDA(cudaMemsetAsync(counts, 0, (size_t)nc * 4, s));
    k_km_counts<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(labels, n, counts);
    BGPU_CHECK_LAUNCH();
  }
  return BGPU_OK;
}

// Float sum of the values in order, starting from init (host; the
// reference's sequential loops).
float seq_sum(float init, const std::vector<float>& v) {
  float t = init;
  for (float x : v) t += x;
  return t;
}

}  // namespace
}  // namespace bgpu

extern "C" int bgpu_kmeans(const float* X, uint32_t* cluster_labels, float* centroids,
                           float* centroids_new, uint32_t* num_cells_per_cluster,
                           float* min_distances, float* cell_norms, int kmeans_barbar,
                           uint32_t num_kmeans_iterations, float tolerance,
                           uint32_t chunk_size, uint64_t seed, uint64_t num_cells,
                           uint32_t num_dimensions, uint32_t num_clusters,
                           uint32_t* iterations, void* stream) {
  BGPU_REQUIRE(X && cluster_labels && centroids && centroids_new && num_cells_per_cluster &&
                   min_distances && iterations,
               BGPU_ERR_INVALID, "kmeans: NULL argument");
  BGPU_REQUIRE(!kmeans_barbar, BGPU_ERR_UNSUPPORTED,
               "kmeans: only the random initialisation (kmeans_barbar=False, the "
               "reference's default) runs on the GPU");
  const uint64_t n = num_cells;
  const uint32_t d = num_dimensions, nc = num_clusters;
  BGPU_REQUIRE(n >= 1 && d >= 1 && nc >= 1 && nc <= n, BGPU_ERR_INVALID,
               "kmeans: needs 1 <= num_clusters <= num_cells and >= 1 dimension");
  BGPU_REQUIRE(d <= kMaxDims, BGPU_ERR_UNSUPPORTED, "kmeans: at most 128 dimensions");
  BGPU_REQUIRE(nc <= kMaxClusters, BGPU_ERR_UNSUPPORTED, "kmeans: at most 32768 clusters");
  BGPU_REQUIRE(chunk_size >= 1 && num_kmeans_iterations >= 1, BGPU_ERR_INVALID,
               "kmeans: chunk_size and num_kmeans_iterations must be >= 1");
  BGPU_REQUIRE(n <= 0xFFFFFFFFull, BGPU_ERR_UNSUPPORTED, "kmeans: at most 2^32 - 1 cells");
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t nchunks = (uint32_t)ceil_div(n, chunk_size);
  const uint64_t per = (uint64_t)nc * d;
  const uint64_t sums_bytes = (uint64_t)nchunks * per * 4;
  BGPU_REQUIRE(sums_bytes <= (64ull << 30), BGPU_ERR_UNSUPPORTED,
               "kmeans: the per-chunk sums would exceed 64 GB; raise chunk_size");

  // random initialisation (kmeans.pyx:13-38)
  std::vector<uint32_t> init(nc);
  {
    std::vector<uint64_t> bits((n + 63) / 64, 0);
    uint64_t state = pcg_srand(seed);
    for (uint32_t i = 0; i < nc; ++i) {
      while (true) {
        const uint32_t j = pcg_randint((uint32_t)n, &state);
        if (!(bits[j >> 6] & (1ull << (j & 63)))) {
          bits[j >> 6] |= 1ull << (j & 63);
          init[i] = j;
          break;
        }
      }
    }
  }
  uint32_t* didx = nullptr;
  float *cn = nullptr, *sums = nullptr, *norms = cell_norms, *own_norms = nullptr;
  BGPU_CUDA(cudaMallocAsync((void**)&didx, (size_t)nc * 4, s));
  BGPU_CUDA(cudaMallocAsync((void**)&cn, (size_t)nc * 4, s));
  BGPU_CUDA(cudaMallocAsync((void**)&sums, sums_bytes, s));
  if (!norms) {
    BGPU_CUDA(cudaMallocAsync((void**)&own_norms, n * 4, s));
    norms = own_norms;
  }
  auto cleanup = [&]() {
    cudaFreeAsync(didx, s);
    cudaFreeAsync(cn, s);
    cudaFreeAsync(sums, s);
    if (own_norms) cudaFreeAsync(own_norms, s);
  };
  auto run = [&]() -> int {
    BGPU_CUDA(cudaMemcpyAsync(didx, init.data(), (size_t)nc * 4, cudaMemcpyHostToDevice, s));
    float* Cc = centroids;
    float* Cn = centroids_new;
    k_km_gather<<<(unsigned)ceil_div(per, 256), 256, 0, s>>>(X, didx, nc, d, Cc);
    BGPU_CHECK_LAUNCH();
    k_km_cell_norms<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(X, n, d, norms);
    BGPU_CHECK_LAUNCH();
    std::vector<float> hnorm(n), hmin;
    BGPU_CUDA(cudaMemcpyAsync(hnorm.data(), norms, n * 4, cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaStreamSynchronize(s));
    const float sum_sq = seq_sum(0.f, hnorm);  // kmeans.pyx:954-965
    float old_total = 0.f;
    uint32_t it = 0;
    std::vector<uint32_t> hcount(nc);
    while (true) {
      BGPU_TRY(km_estep(X, n, d, Cc, cn, nc, cluster_labels, min_distances,
                        num_cells_per_cluster, s));
      BGPU_CUDA(cudaMemsetAsync(sums, 0, sums_bytes, s));
      k_km_chunk_sums<<<nchunks, std::min<uint32_t>(128, (d + 31) & ~31u), 0, s>>>(
          X, n, d, cluster_labels, chunk_size, nc, sums);
      BGPU_CHECK_LAUNCH();
      k_km_reduce<<<(unsigned)ceil_div(per, 256), 256, 0, s>>>(sums, nchunks, nc, d, Cn);
      BGPU_CHECK_LAUNCH();
      BGPU_CUDA(cudaMemcpyAsync(hcount.data(), num_cells_per_cluster, (size_t)nc * 4,
                                cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaStreamSynchronize(s));
      std::vector<uint32_t> empty;
      for (uint32_t c = 0; c < nc; ++c)
        if (hcount[c] == 0) empty.push_back(c);
      if (!empty.empty()) {  // relocate_empty_clusters (kmeans.pyx:747-820)
        float* dist = nullptr;
        BGPU_CUDA(cudaMallocAsync((void**)&dist, n * 4, s));
        k_km_assigned<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(X, cluster_labels, Cc,
                                                                  n, d, dist);
        std::vector<float> hd(n), hx, hcn(per);
        std::vector<uint32_t> hl(n);
        cudaMemcpyAsync(hd.data(), dist, n * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hl.data(), cluster_labels, n * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hcn.data(), Cn, per * 4, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(dist, s);
        BGPU_CUDA(cudaStreamSynchronize(s));
        // the num_empty largest distances, an earlier cell winning ties, in
        // descending order
        const size_t ne = empty.size();
        std::vector<uint64_t> order(n);
        for (uint64_t i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](uint64_t a, uint64_t b) { return hd[a] > hd[b]; });
        BGPU_REQUIRE(hd[order[0]] != 0.f, BGPU_ERR_INVALID,
                     "kmeans: num_clusters is greater than the number of cells with "
                     "distinct principal component loadings; decrease num_clusters");
        std::vector<float> row(d);
        for (size_t e = 0; e < ne; ++e) {
          const uint64_t j = order[e];
          const uint32_t oldc = hl[j], newc = empty[e];
          BGPU_CUDA(cudaMemcpy(row.data(), X + j * d, (size_t)d * 4, cudaMemcpyDeviceToHost));
          for (uint32_t k = 0; k < d; ++k) {
            hcn[(uint64_t)oldc * d + k] -= row[k];
            hcn[(uint64_t)newc * d + k] = row[k];
          }
          hcount[oldc] -= 1;
          hcount[newc] += 1;
        }
        BGPU_CUDA(cudaMemcpyAsync(Cn, hcn.data(), per * 4, cudaMemcpyHostToDevice, s));
        BGPU_CUDA(cudaMemcpyAsync(num_cells_per_cluster, hcount.data(), (size_t)nc * 4,
                                  cudaMemcpyHostToDevice, s));
      }
      k_km_normalize<<<(unsigned)ceil_div(per, 256), 256, 0, s>>>(Cn, num_cells_per_cluster,
                                                                  nc, d);
      BGPU_CHECK_LAUNCH();
      std::swap(Cc, Cn);
      ++it;
      if (it == num_kmeans_iterations) break;
      hmin.resize(n);
      BGPU_CUDA(cudaMemcpyAsync(hmin.data(), min_distances, n * 4, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaStreamSynchronize(s));
      const float total = seq_sum(sum_sq, hmin);  // kmeans.pyx:1088-1098
      if (it > 1 && old_total - total < tolerance * old_total) break;
      old_total = total;
    }
    // the final E step (kmeans.pyx:1100-1153)
    BGPU_TRY(km_estep(X, n, d, Cc, cn, nc, cluster_labels, min_distances,
                      num_cells_per_cluster, s));
    *iterations = it;
    return BGPU_OK;
  };
  const int rc = run();
  cleanup();
  if (rc == BGPU_OK) BGPU_CUDA(cudaStreamSynchronize(s));
  return rc;
}
