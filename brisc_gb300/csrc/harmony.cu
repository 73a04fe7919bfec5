// Harmony batch correction of the PCs: the reference's harmony
// (brisc/harmonize.pyx:269-871), called by SingleCell.harmonize
// (brisc/single_cell.py:13224-13876) after its k-means of the row-normalised
// PCs.
//
// The algorithm is the reference's, step for step:
//  - initial soft assignments R = softmax_j(2/sigma (Z.Y_j - 1)) per cell
//    (Y not yet normalised), cluster sizes E = Pr_b R_sum and per-batch
//    sums O, and the objective (harmonize.pyx:412-498);
//  - per clustering iteration: Y = normalise(R^T Z); then the cells in a
//    random order (inside-out Fisher-Yates with PCG32 from srand(seed),
//    harmonize.pyx:503-509) in blocks of ceil(block_proportion n); the
//    chunks of a block all see E and O as the block found them, each takes
//    its own cells' contributions out, recomputes R for its cells as
//    exp(2/sigma Z.Y_j) ((E+1)/(O+E+1))^theta exp(-2/sigma), normalised, and
//    puts them back; E and O take the block's changes in chunk order
//    (harmonize.pyx:533-654); the objective after the last clustering
//    iteration (or each, with early stopping);
//  - the correction: per cluster a ridge regression of the PCs on the batch
//    indicators weighted by R (the (B+1) x (B+1) inverse in closed form,
//    harmonize.pyx:758-812), Z = PCs - sum_k R_k W_k[batch]; stop when the
//    objective's relative decrease is below tolerance (Z left as corrected),
//    else normalise Z's rows and iterate.
// The reference's products are sgemm calls and its sums run per thread, so
// the GPU's results agree with it to float rounding, not bit for bit.
//
// GPU shape: one CTA per chunk. Distances and new assignments run a warp per
// cell (lanes over clusters, the cell's row of Z from shared memory, Y in
// shared memory as [dim][cluster]); every per-chunk sum over cells is a
// thread per cluster walking the chunk's cells in order; sums over chunks
// and clusters are in fixed order. The small (B+1)-sized algebra of the
// correction runs on the host.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "pcg.h"

namespace bgpu {
namespace {

constexpr int kHThreads = 256;
constexpr int kHWarps = kHThreads / 32;
constexpr uint32_t kHMaxClusters = 256;
constexpr uint32_t kHMaxDims = 128;
constexpr uint32_t kHMaxBatches = 64;
constexpr uint32_t kHMaxChunk = 1024;

// Y (C x d, row-major) into shared memory as [dim][cluster].
__device__ void stage_y(const float* __restrict__ Y, uint32_t C, uint32_t d, float* ys) {
  for (uint32_t t = threadIdx.x; t < C * d; t += blockDim.x) {
    const uint32_t j = t / d, k = t % d;
    ys[k * C + j] = Y[t];
  }
}

// Row i of the chunk's cells: cells[i] when a list is given, else c0 + i.
__device__ __forceinline__ uint64_t cell_at(const uint32_t* cells, uint64_t c0, uint32_t i) {
  return cells ? (uint64_t)cells[c0 + i] : c0 + i;
}

// For each cell of the chunk, a warp computes the dot products with every
// centroid (lanes over clusters) and hands them to `f(cell, lane-column
// dots[], count)`; Z rows are read from global (L1) once per cell.
template <int CPL, typename Fn>
__device__ void for_each_cell_dots(const float* __restrict__ Z, uint32_t d, uint32_t C,
                                   const float* ys, const uint32_t* cells, uint64_t c0,
                                   uint32_t ncell, Fn f) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint32_t i = wid; i < ncell; i += kHWarps) {
    const uint64_t cell = cell_at(cells, c0, i);
    const float* z = Z + cell * d;
    float dot[CPL];
#pragma unroll
    for (int q = 0; q < CPL; ++q) dot[q] = 0.f;
    for (uint32_t k = 0; k < d; ++k) {
      const float zk = z[k];  // broadcast
      const float* yk = ys + (uint64_t)k * C;
#pragma unroll
      for (int q = 0; q < CPL; ++q) {
        const uint32_t j = lane + 32u * q;
        if (j < C) dot[q] = fmaf(zk, yk[j], dot[q]);
      }
    }
    f(i, cell, dot);
  }
}

// Init (harmonize.pyx:412-441): R = exp(2/sigma (dot - 1)), normalised; per
// chunk: R sums, per-batch sums, k-means error and entropy partials.
template <int CPL>
__global__ void __launch_bounds__(kHThreads)
k_h_init(const float* __restrict__ Z, const float* __restrict__ Y, const uint32_t* __restrict__ batch,
         uint64_t n, uint32_t d, uint32_t C, uint32_t B, uint32_t chunk, float tos,
         float* __restrict__ R, float* __restrict__ rsum, float* __restrict__ bsum,
         double* __restrict__ obj_part) {
  extern __shared__ float sm[];
  float* ys = sm;                  // d x C
  float* bs = ys + (size_t)d * C;  // B x C
  __shared__ double red[2][kHWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
  const uint32_t ncell = (uint32_t)min_u64(chunk, n - c0);
  stage_y(Y, C, d, ys);
  __syncthreads();
  double ke = 0.0, en = 0.0;  // per lane, over its cells and clusters
  for_each_cell_dots<CPL>(Z, d, C, ys, nullptr, c0, ncell,
      [&](uint32_t, uint64_t cell, const float (&dot)[CPL]) {
        float r[CPL], s = 0.f;
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t j = lane + 32u * q;
          r[q] = j < C ? expf(tos * (dot[q] - 1.f)) : 0.f;
          s += r[q];
        }
        const float inv = 1.f / warp_sum(s);
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t j = lane + 32u * q;
          if (j < C) {
            const float v = r[q] * inv;
            R[cell * C + j] = v;
            ke += (double)(v * (1.f - dot[q]));
            en += v > 0.f ? (double)(v * logf(v)) : 0.0;
          }
        }
      });
  // fixed-order block reduction of the objective partials
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ke += __shfl_xor_sync(0xffffffffu, ke, o);
    en += __shfl_xor_sync(0xffffffffu, en, o);
  }
  if (lane == 0) { red[0][wid] = ke; red[1][wid] = en; }
  __syncthreads();  // R of the chunk is written (same CTA)
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kHWarps; ++w) { a += red[0][w]; b += red[1][w]; }
    obj_part[2 * blockIdx.x] = a;
    obj_part[2 * blockIdx.x + 1] = b;
  }
  // per-cluster sums over the chunk's cells in order
  for (uint32_t j = threadIdx.x; j < C; j += blockDim.x) {
    for (uint32_t b = 0; b < B; ++b) bs[b * C + j] = 0.f;
    float s = 0.f;
    for (uint32_t i = 0; i < ncell; ++i) {
      const uint64_t cell = c0 + i;
      const float v = R[cell * C + j];
      s += v;
      bs[batch[cell] * C + j] += v;
    }
    rsum[(uint64_t)blockIdx.x * C + j] = s;
    for (uint32_t b = 0; b < B; ++b)
      bsum[((uint64_t)blockIdx.x * B + b) * C + j] = bs[b * C + j];
  }
}

// One block of the clustering pass (harmonize.pyx:566-647): one CTA per
// chunk of the block's cells (cell_order[bstart + ...]).
template <int CPL>
__global__ void __launch_bounds__(kHThreads)
k_h_block(const float* __restrict__ Z, const float* __restrict__ Y, const uint32_t* __restrict__ batch,
          const uint32_t* __restrict__ order, uint64_t bstart, uint64_t blen, uint32_t d,
          uint32_t C, uint32_t B, uint32_t chunk, float tos, float ens,
          const float* __restrict__ E, const float* __restrict__ O,
          const float* __restrict__ Pr, const float* __restrict__ theta, float* __restrict__ R,
          float* __restrict__ dE, float* __restrict__ dO) {
  extern __shared__ float sm[];
  float* ys = sm;                    // d x C
  float* ratio = ys + (size_t)d * C; // B x C
  float* bold = ratio + (size_t)B * C;  // B x C: the chunk's old per-batch sums
  float* bnew = bold + (size_t)B * C;   // B x C
  float* rold = bnew + (size_t)B * C;   // C
  const int lane = threadIdx.x & 31;
  const uint64_t c0 = bstart + (uint64_t)blockIdx.x * chunk;
  const uint32_t ncell = (uint32_t)min_u64(chunk, bstart + blen - c0);
  stage_y(Y, C, d, ys);
  // old contributions, per cluster over the chunk's cells in order
  for (uint32_t j = threadIdx.x; j < C; j += blockDim.x) {
    for (uint32_t b = 0; b < B; ++b) bold[b * C + j] = 0.f;
    float s = 0.f;
    for (uint32_t i = 0; i < ncell; ++i) {
      const uint64_t cell = order[c0 + i];
      const float v = R[cell * C + j];
      s += v;
      bold[batch[cell] * C + j] += v;
    }
    rold[j] = s;
    for (uint32_t b = 0; b < B; ++b) {
      const float dEij = -Pr[b] * s;
      const float Eij = E[b * C + j] + dEij;
      const float Oij = O[b * C + j] - bold[b * C + j];
      ratio[b * C + j] = ens * powf((Eij + 1.f) / (Oij + Eij + 1.f), theta[b]);
    }
  }
  __syncthreads();
  for_each_cell_dots<CPL>(Z, d, C, ys, order, c0, ncell,
      [&](uint32_t, uint64_t cell, const float (&dot)[CPL]) {
        const float* rt = ratio + (size_t)batch[cell] * C;
        float r[CPL], s = 0.f;
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t j = lane + 32u * q;
          r[q] = j < C ? expf(tos * dot[q]) * rt[j] : 0.f;
          s += r[q];
        }
        const float inv = 1.f / warp_sum(s);
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t j = lane + 32u * q;
          if (j < C) R[cell * C + j] = r[q] * inv;
        }
      });
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < C; j += blockDim.x) {
    for (uint32_t b = 0; b < B; ++b) bnew[b * C + j] = 0.f;
    float s = 0.f;
    for (uint32_t i = 0; i < ncell; ++i) {
      const uint64_t cell = order[c0 + i];
      const float v = R[cell * C + j];
      s += v;
      bnew[batch[cell] * C + j] += v;
    }
    for (uint32_t b = 0; b < B; ++b) {
      const uint64_t o = ((uint64_t)blockIdx.x * B + b) * C + j;
      dE[o] = -Pr[b] * rold[j] + Pr[b] * s;
      dO[o] = -bold[b * C + j] + bnew[b * C + j];
    }
  }
}

// E += sum of the chunks' dE, O += ..., in chunk order (one thread per entry).
__global__ void k_h_block_reduce(float* __restrict__ E, float* __restrict__ O,
                                 const float* __restrict__ dE, const float* __restrict__ dO,
                                 uint32_t nchunks, uint32_t BC) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= BC) return;
  float e = 0.f, o = 0.f;
  for (uint32_t c = 0; c < nchunks; ++c) {
    e += dE[(uint64_t)c * BC + t];
    o += dO[(uint64_t)c * BC + t];
  }
  E[t] += e;
  O[t] += o;
}

// part[chunk][j][k] = sum over the chunk's cells (in order) of R[cell][j] M[cell][k];
// cells = list (or identity), chunk boundaries given by starts[] (nchunks + 1).
__global__ void __launch_bounds__(kHThreads)
k_h_rtm(const float* __restrict__ R, const float* __restrict__ M, const uint32_t* __restrict__ cells,
        const uint64_t* __restrict__ starts, uint32_t d, uint32_t C, float* __restrict__ part) {
  const uint64_t a = starts[blockIdx.x], b = starts[blockIdx.x + 1];
  for (uint32_t t = threadIdx.x; t < C * d; t += blockDim.x) {
    const uint32_t j = t / d, k = t % d;
    float s = 0.f;
    for (uint64_t i = a; i < b; ++i) {
      const uint64_t cell = cells ? (uint64_t)cells[i] : i;
      s = fmaf(R[cell * C + j], M[cell * d + k], s);
    }
    part[(uint64_t)blockIdx.x * C * d + t] = s;
  }
}

// out[j][k] = sum over chunks c in [c0, c1) of part[c][j][k], in order; with
// normalise, each row scaled by 1 / sqrt(sum of squares) (one CTA per row).
__global__ void k_h_rtm_reduce(const float* __restrict__ part, uint32_t c0, uint32_t c1,
                               uint32_t d, uint32_t C, int normalise, float* __restrict__ out) {
  __shared__ float red[4];
  __shared__ float scale;
  const uint32_t j = blockIdx.x;
  float v = 0.f;
  const uint32_t k = threadIdx.x;
  if (k < d)
    for (uint32_t c = c0; c < c1; ++c) v += part[((uint64_t)c * C + j) * d + k];
  if (normalise) {
    float sq = warp_sum(k < d ? v * v : 0.f);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
      float t = 0.f;
      for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) t += red[w];
      scale = 1.f / sqrtf(t);
    }
    __syncthreads();
    v *= scale;
  }
  if (k < d) out[(uint64_t)j * d + k] = v;
}

// Objective partials (harmonize.pyx:658-684): per chunk, sum R (1 - Z.Y_j)
// and sum R log R.
template <int CPL>
__global__ void __launch_bounds__(kHThreads)
k_h_objective(const float* __restrict__ Z, const float* __restrict__ Y, const float* __restrict__ R,
              uint64_t n, uint32_t d, uint32_t C, uint32_t chunk, double* __restrict__ obj_part) {
  extern __shared__ float sm[];
  float* ys = sm;
  __shared__ double red[2][kHWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t c0 = (uint64_t)blockIdx.x * chunk;
  const uint32_t ncell = (uint32_t)min_u64(chunk, n - c0);
  stage_y(Y, C, d, ys);
  __syncthreads();
  double ke = 0.0, en = 0.0;
  for_each_cell_dots<CPL>(Z, d, C, ys, nullptr, c0, ncell,
      [&](uint32_t, uint64_t cell, const float (&dot)[CPL]) {
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t j = lane + 32u * q;
          if (j < C) {
            const float v = R[cell * C + j];
            ke += (double)(v * (1.f - dot[q]));
            en += v > 0.f ? (double)(v * logf(v)) : 0.0;
          }
        }
      });
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ke += __shfl_xor_sync(0xffffffffu, ke, o);
    en += __shfl_xor_sync(0xffffffffu, en, o);
  }
  if (lane == 0) { red[0][wid] = ke; red[1][wid] = en; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < kHWarps; ++w) { a += red[0][w]; b += red[1][w]; }
    obj_part[2 * blockIdx.x] = a;
    obj_part[2 * blockIdx.x + 1] = b;
  }
}

// Z = PCs - sum_k R[cell][k] W[k][batch][:] (harmonize.pyx:814-818), then,
// with normalise, each row scaled to unit norm. One warp per cell.
__global__ void __launch_bounds__(kHThreads)
k_h_correct(const float* __restrict__ PCs, const float* __restrict__ R, const float* __restrict__ W,
            const uint32_t* __restrict__ batch, uint64_t n, uint32_t d, uint32_t C, uint32_t B,
            int normalise, float* __restrict__ Z) {
  const int lane = threadIdx.x & 31;
  const uint64_t cell = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (cell >= n) return;
  const uint32_t b = batch[cell];
  float z[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t k = lane + 32u * q;
    z[q] = k < d ? PCs[cell * d + k] : 0.f;
  }
  for (uint32_t c = 0; c < C; ++c) {
    const float r = R[cell * C + c];
    const float* w = W + ((uint64_t)c * (B + 1) + b) * d;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t k = lane + 32u * q;
      if (k < d) z[q] -= w[k] * r;
    }
  }
  float scale = 1.f;
  if (normalise) {
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q) s += z[q] * z[q];
    scale = 1.f / sqrtf(warp_sum(s));
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t k = lane + 32u * q;
    if (k < d) Z[cell * d + k] = z[q] * scale;
  }
}

// out = arr with each row times 1 / sqrt(sum of squares) (harmonize.pyx:
// 244-266). One warp per row.
__global__ void __launch_bounds__(kHThreads)
k_h_normalize_rows(const float* __restrict__ in, float* __restrict__ out, uint64_t rows,
                   uint32_t cols) {
  const int lane = threadIdx.x & 31;
  const uint64_t row = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (row >= rows) return;
  const float* a = in + row * cols;
  float s = 0.f;
  for (uint32_t k = lane; k < cols; k += 32) s = fmaf(a[k], a[k], s);
  const float scale = 1.f / sqrtf(warp_sum(s));
  for (uint32_t k = lane; k < cols; k += 32) out[row * cols + k] = a[k] * scale;
}

struct HDev {
  float *E, *O, *Pr, *theta, *rsum, *bsum, *dE, *dO, *part, *W;
  double* obj;
  uint32_t *order, *border;
  uint64_t *starts_nat, *starts_b;
};

template <int CPL>
int harmony_run(const float* PCs, float* Z, float* Y, float* R, const uint32_t* batch,
                uint64_t n, uint32_t d, uint32_t C, uint32_t B, uint32_t max_iter,
                uint32_t max_ci, float block_prop, float tol, int early, float ctol,
                float theta, float tau, float alpha, float sigma, uint32_t chunk, uint64_t seed,
                uint32_t* iters, cudaStream_t s) {
  const uint32_t BC = B * C;
  const uint32_t nchunks = (uint32_t)ceil_div(n, chunk);
  // the reference multiplies an unsigned long long by a float: float product
  const uint64_t block = (uint64_t)std::ceil((float)n * block_prop);
  const uint32_t max_cpb = (uint32_t)ceil_div(block, chunk);
  const float tos = 2.f / sigma;
  const float ens = std::exp(-tos);
  // host-side batch bookkeeping, the random cell order, batch-sorted order
  std::vector<uint32_t> hb(n);
  BGPU_CUDA(cudaMemcpyAsync(hb.data(), batch, n * 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  std::vector<uint64_t> Nb(B, 0);
  for (uint64_t i = 0; i < n; ++i) {
    BGPU_REQUIRE(hb[i] < B, BGPU_ERR_INVALID, "harmony: a batch label is >= num_batches");
    ++Nb[hb[i]];
  }
  std::vector<float> Pr(B), th(B);
  for (uint32_t b = 0; b < B; ++b) {
    Pr[b] = (float)Nb[b] / (float)n;
    if (tau > 0.f) {
      // the reference negates its unsigned count (harmonize.pyx:416): -N_b
      // wraps to 2^32 - N_b, base overflows to inf (1 for an empty batch) and
      // theta becomes -inf; kept for identical results
      const uint32_t neg = 0u - (uint32_t)Nb[b];
      const float base = (float)std::exp((double)((float)neg / ((float)C * tau)));
      th[b] = theta * (1.f - base * base);
    } else {
      th[b] = theta;
    }
  }
  std::vector<uint32_t> order(n);
  {
    uint64_t state = pcg_srand(seed);
    for (uint64_t i = 0; i < n; ++i) {
      const uint32_t j = pcg_randint((uint32_t)(i + 1), &state);
      order[i] = order[j];
      order[j] = (uint32_t)i;
    }
  }
  // batch-sorted cells (stable) and chunk starts that never straddle batches
  std::vector<uint32_t> border(n);
  std::vector<uint64_t> bstart(B + 1, 0), starts_b, starts_nat;
  for (uint32_t b = 0; b < B; ++b) bstart[b + 1] = bstart[b] + Nb[b];
  {
    std::vector<uint64_t> pos(bstart.begin(), bstart.end() - 1);
    for (uint64_t i = 0; i < n; ++i) border[pos[hb[i]]++] = (uint32_t)i;
  }
  const uint64_t rchunk = 4096;
  std::vector<uint32_t> bchunk0(B + 1, 0);
  for (uint32_t b = 0; b < B; ++b) {
    bchunk0[b] = (uint32_t)starts_b.size();
    for (uint64_t a = bstart[b]; a < bstart[b + 1]; a += rchunk) starts_b.push_back(a);
  }
  bchunk0[B] = (uint32_t)starts_b.size();
  starts_b.push_back(n);
  for (uint64_t a = 0; a < n; a += rchunk) starts_nat.push_back(a);
  starts_nat.push_back(n);
  const uint32_t nrc_nat = (uint32_t)starts_nat.size() - 1;
  const uint32_t nrc_b = (uint32_t)starts_b.size() - 1;

  HDev D{};
  std::vector<void*> allocs;
  auto dalloc = [&](void** p, size_t bytes) -> int {
    BGPU_CUDA(cudaMallocAsync(p, std::max<size_t>(bytes, 16), s));
    allocs.push_back(*p);
    return BGPU_OK;
  };
  const uint32_t npart = std::max(nrc_nat, nrc_b);
  int rc = BGPU_OK;
  auto body = [&]() -> int {
    BGPU_TRY(dalloc((void**)&D.E, BC * 4ull));
    BGPU_TRY(dalloc((void**)&D.O, BC * 4ull));
    BGPU_TRY(dalloc((void**)&D.Pr, B * 4ull));
    BGPU_TRY(dalloc((void**)&D.theta, B * 4ull));
    BGPU_TRY(dalloc((void**)&D.rsum, (uint64_t)nchunks * C * 4));
    BGPU_TRY(dalloc((void**)&D.bsum, (uint64_t)nchunks * BC * 4));
    BGPU_TRY(dalloc((void**)&D.dE, (uint64_t)max_cpb * BC * 4));
    BGPU_TRY(dalloc((void**)&D.dO, (uint64_t)max_cpb * BC * 4));
    BGPU_TRY(dalloc((void**)&D.part, (uint64_t)npart * C * d * 4));
    BGPU_TRY(dalloc((void**)&D.W, (uint64_t)C * (B + 1) * d * 4));
    BGPU_TRY(dalloc((void**)&D.obj, (uint64_t)nchunks * 16));
    BGPU_TRY(dalloc((void**)&D.order, n * 4));
    BGPU_TRY(dalloc((void**)&D.border, n * 4));
    BGPU_TRY(dalloc((void**)&D.starts_nat, starts_nat.size() * 8));
    BGPU_TRY(dalloc((void**)&D.starts_b, starts_b.size() * 8));
    BGPU_CUDA(cudaMemcpyAsync(D.Pr, Pr.data(), B * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(D.theta, th.data(), B * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(D.order, order.data(), n * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(D.border, border.data(), n * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(D.starts_nat, starts_nat.data(), starts_nat.size() * 8,
                              cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(D.starts_b, starts_b.data(), starts_b.size() * 8,
                              cudaMemcpyHostToDevice, s));

    std::vector<float> hE(BC), hO(BC), hpart;
    std::vector<double> hobj;
    auto objective = [&](double ke, double en) -> float {
      // diversity penalty (harmonize.pyx:466-476, 687-695) on the host
      double pen = 0.0;
      for (uint32_t j = 0; j < C; ++j) {
        float cj = 0.f;
        for (uint32_t b = 0; b < B; ++b) {
          const float o = hO[b * C + j], e = hE[b * C + j];
          cj += (o * std::log((o + e + 1.f) / (e + 1.f))) * th[b];
        }
        pen += cj;
      }
      return (float)(2.0 * ke) + (float)(sigma * en) + (float)(sigma * pen);
    };
    auto fetch_eo = [&]() -> int {
      BGPU_CUDA(cudaMemcpyAsync(hE.data(), D.E, BC * 4ull, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaMemcpyAsync(hO.data(), D.O, BC * 4ull, cudaMemcpyDeviceToHost, s));
      return BGPU_OK;
    };
    auto fetch_obj = [&](double* ke, double* en) -> int {
      hobj.resize(2ull * nchunks);
      BGPU_CUDA(cudaMemcpyAsync(hobj.data(), D.obj, hobj.size() * 8, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaStreamSynchronize(s));
      *ke = 0.0;
      *en = 0.0;
      for (uint32_t c = 0; c < nchunks; ++c) { *ke += hobj[2 * c]; *en += hobj[2 * c + 1]; }
      return BGPU_OK;
    };
    const size_t sm_y = (size_t)d * C * 4;
    // initialisation
    k_h_init<CPL><<<nchunks, kHThreads, sm_y + (size_t)BC * 4, s>>>(
        Z, Y, batch, n, d, C, B, chunk, tos, R, D.rsum, D.bsum, D.obj);
    BGPU_CHECK_LAUNCH();
    {
      std::vector<float> hr((uint64_t)nchunks * C), hbs((uint64_t)nchunks * BC);
      BGPU_CUDA(cudaMemcpyAsync(hr.data(), D.rsum, hr.size() * 4, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaMemcpyAsync(hbs.data(), D.bsum, hbs.size() * 4, cudaMemcpyDeviceToHost, s));
      double ke, en;
      BGPU_TRY(fetch_obj(&ke, &en));
      for (uint32_t j = 0; j < C; ++j) {
        float rs = 0.f;
        for (uint32_t c = 0; c < nchunks; ++c) rs += hr[(uint64_t)c * C + j];
        for (uint32_t b = 0; b < B; ++b) {
          hE[b * C + j] = Pr[b] * rs;
          float o = 0.f;
          for (uint32_t c = 0; c < nchunks; ++c) o += hbs[((uint64_t)c * B + b) * C + j];
          hO[b * C + j] = o;
        }
      }
      BGPU_CUDA(cudaMemcpyAsync(D.E, hE.data(), BC * 4ull, cudaMemcpyHostToDevice, s));
      BGPU_CUDA(cudaMemcpyAsync(D.O, hO.data(), BC * 4ull, cudaMemcpyHostToDevice, s));
      float prev = objective(ke, en);
      // normalise Y's rows (harmonize.pyx:501)
      BGPU_CUDA(cudaMemcpyAsync(D.part, Y, (uint64_t)C * d * 4, cudaMemcpyDeviceToDevice, s));
      k_h_rtm_reduce<<<C, 128, 0, s>>>(D.part, 0, 1, d, C, 1, Y);
      BGPU_CHECK_LAUNCH();
      float objective_v = prev;
      const size_t sm_blk = sm_y + (size_t)3 * BC * 4 + (size_t)C * 4;
      uint32_t it = 0;
      for (it = 1; it <= max_iter; ++it) {
        float past[3] = {0.f, 0.f, 0.f};
        for (uint32_t ci = 1; ci <= max_ci; ++ci) {
          // Y = normalise(R^T Z) over natural chunks
          k_h_rtm<<<nrc_nat, kHThreads, 0, s>>>(R, Z, nullptr, D.starts_nat, d, C, D.part);
          BGPU_CHECK_LAUNCH();
          k_h_rtm_reduce<<<C, 128, 0, s>>>(D.part, 0, nrc_nat, d, C, 1, Y);
          BGPU_CHECK_LAUNCH();
          for (uint64_t b0 = 0; b0 < n; b0 += block) {
            const uint64_t blen = std::min<uint64_t>(block, n - b0);
            const uint32_t ncb = (uint32_t)ceil_div(blen, chunk);
            k_h_block<CPL><<<ncb, kHThreads, sm_blk, s>>>(
                Z, Y, batch, D.order, b0, blen, d, C, B, chunk, tos, ens, D.E, D.O, D.Pr,
                D.theta, R, D.dE, D.dO);
            BGPU_CHECK_LAUNCH();
            k_h_block_reduce<<<(unsigned)ceil_div(BC, 256), 256, 0, s>>>(D.E, D.O, D.dE,
                                                                        D.dO, ncb, BC);
            BGPU_CHECK_LAUNCH();
          }
          if (early || ci == max_ci) {
            k_h_objective<CPL><<<nchunks, kHThreads, sm_y, s>>>(Z, Y, R, n, d, C, chunk,
                                                                D.obj);
            BGPU_CHECK_LAUNCH();
            BGPU_TRY(fetch_eo());
            BGPU_TRY(fetch_obj(&ke, &en));
            objective_v = objective(ke, en);
            if (early) {
              if (ci <= 3) {
                past[ci - 1] = objective_v;
              } else {
                const float last_two = past[1] + past[2];
                const float old = past[0] + last_two, nw = last_two + objective_v;
                if (old - nw < ctol * std::fabs(old)) break;
                past[0] = past[1];
                past[1] = past[2];
                past[2] = objective_v;
              }
            }
          }
        }
        // correction: R-weighted per-batch PC sums per cluster
        k_h_rtm<<<nrc_b, kHThreads, 0, s>>>(R, PCs, D.border, D.starts_b, d, C, D.part);
        BGPU_CHECK_LAUNCH();
        hpart.resize((uint64_t)nrc_b * C * d);
        BGPU_CUDA(cudaMemcpyAsync(hpart.data(), D.part, hpart.size() * 4,
                                  cudaMemcpyDeviceToHost, s));
        BGPU_CUDA(cudaStreamSynchronize(s));
        std::vector<float> W((uint64_t)C * (B + 1) * d, 0.f);
        std::vector<float> inv1((B + 1) * (B + 1)), inv2((B + 1) * (B + 1)),
            inv((B + 1) * (B + 1)), rs((uint64_t)d * (B + 1));
        for (uint32_t i = 0; i < (B + 1) * (B + 1); ++i) inv2[i] = 0.f;
        for (uint32_t i = 0; i <= B; ++i) inv2[i * (B + 1) + i] = 1.f;
        for (uint32_t k = 0; k < C; ++k) {
          std::fill(inv1.begin(), inv1.end(), 0.f);
          float norm = 0.f;
          for (uint32_t i = 0; i < B; ++i) {
            const float o = hO[i * C + k], e = hE[i * C + k];
            if (o < 1e-5f * (float)Nb[i]) {
              inv2[B * (B + 1) + i] = 0.f;
            } else {
              float factor = 1.f / (o + e * alpha);
              inv1[i * (B + 1) + i] = factor;
              factor *= -o;
              inv2[B * (B + 1) + i] = factor;
              norm += o * (1.f + factor);
            }
          }
          norm = 1.f / norm;
          inv1[B * (B + 1) + B] = norm;
          for (uint32_t i = 0; i < B; ++i) inv1[B * (B + 1) + i] = inv2[B * (B + 1) + i] * norm;
          for (uint32_t r = 0; r <= B; ++r)  // inv = inv1^T inv2
            for (uint32_t c = 0; c <= B; ++c) {
              float t = 0.f;
              for (uint32_t q = 0; q <= B; ++q) t += inv1[q * (B + 1) + r] * inv2[q * (B + 1) + c];
              inv[r * (B + 1) + c] = t;
            }
          for (uint32_t j = 0; j < d; ++j) {
            float total = 0.f;
            for (uint32_t b = 0; b < B; ++b) {
              float bt = 0.f;
              if (!(hO[b * C + k] < 1e-5f * (float)Nb[b]))
                for (uint32_t c = bchunk0[b]; c < bchunk0[b + 1]; ++c)
                  bt += hpart[((uint64_t)c * C + k) * d + j];
              rs[j * (B + 1) + b] = bt;
              total += bt;
            }
            rs[j * (B + 1) + B] = total;
          }
          for (uint32_t r = 0; r <= B; ++r)  // W[k] = inv rs^T
            for (uint32_t j = 0; j < d; ++j) {
              float t = 0.f;
              for (uint32_t q = 0; q <= B; ++q) t += inv[r * (B + 1) + q] * rs[j * (B + 1) + q];
              W[((uint64_t)k * (B + 1) + r) * d + j] = t;
            }
        }
        BGPU_CUDA(cudaMemcpyAsync(D.W, W.data(), W.size() * 4, cudaMemcpyHostToDevice, s));
        const bool done = prev - objective_v < tol * std::fabs(prev);
        k_h_correct<<<(unsigned)ceil_div(n * 32, kHThreads), kHThreads, 0, s>>>(
            PCs, R, D.W, batch, n, d, C, B, done ? 0 : 1, Z);
        BGPU_CHECK_LAUNCH();
        BGPU_CUDA(cudaStreamSynchronize(s));
        if (done) break;
        prev = objective_v;
      }
      *iters = std::min(it, max_iter);
    }
    return BGPU_OK;
  };
  rc = body();
  for (void* p : allocs) cudaFreeAsync(p, s);
  if (rc == BGPU_OK) BGPU_CUDA(cudaStreamSynchronize(s));
  return rc;
}

}  // namespace
}  // namespace bgpu

using namespace bgpu;

extern "C" int bgpu_harmony(const float* PCs, float* Z, float* Y, float* R,
                            const uint32_t* batch_labels, uint32_t num_batches,
                            uint32_t max_iterations, uint32_t max_clustering_iterations,
                            float block_proportion, float tolerance, int early_stopping,
                            float clustering_tolerance, float theta, float tau, float alpha,
                            float sigma, uint32_t chunk_size, uint64_t seed,
                            uint64_t num_cells, uint32_t num_PCs, uint32_t num_clusters,
                            uint32_t* iterations, void* stream) {
  BGPU_REQUIRE(PCs && Z && Y && R && batch_labels && iterations, BGPU_ERR_INVALID,
               "harmony: NULL argument");
  const uint64_t n = num_cells;
  const uint32_t d = num_PCs, C = num_clusters, B = num_batches;
  BGPU_REQUIRE(n >= 2 && d >= 1 && C >= 1 && B >= 1, BGPU_ERR_INVALID,
               "harmony: needs >= 2 cells, >= 1 PC, cluster and batch");
  BGPU_REQUIRE(C <= kHMaxClusters && d <= kHMaxDims && B <= kHMaxBatches, BGPU_ERR_UNSUPPORTED,
               "harmony: at most 256 clusters, 128 PCs and 64 batches");
  BGPU_REQUIRE(chunk_size >= 1 && chunk_size <= kHMaxChunk, BGPU_ERR_UNSUPPORTED,
               "harmony: chunk_size must be in [1, 1024]");
  BGPU_REQUIRE(block_proportion > 0.f && block_proportion <= 1.f, BGPU_ERR_INVALID,
               "harmony: block_proportion must be in (0, 1]");
  BGPU_REQUIRE(sigma > 0.f, BGPU_ERR_INVALID, "harmony: sigma must be > 0");
  BGPU_REQUIRE(n <= 0xFFFFFFFFull, BGPU_ERR_UNSUPPORTED, "harmony: at most 2^32 - 1 cells");
  const size_t smem = (size_t)d * C * 4 + (size_t)3 * B * C * 4 + (size_t)C * 4;
  BGPU_REQUIRE(smem <= 200 * 1024, BGPU_ERR_UNSUPPORTED,
               "harmony: num_PCs x num_clusters + 3 num_batches x num_clusters too large");
  cudaStream_t s = (cudaStream_t)stream;
  auto go = [&](auto cpl) -> int {
    constexpr int CPL = decltype(cpl)::value;
    for (auto fn : {(const void*)k_h_init<CPL>, (const void*)k_h_block<CPL>,
                    (const void*)k_h_objective<CPL>})
      BGPU_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
    return harmony_run<CPL>(PCs, Z, Y, R, batch_labels, n, d, C, B, max_iterations,
                            max_clustering_iterations, block_proportion, tolerance,
                            early_stopping, clustering_tolerance, theta, tau, alpha, sigma,
                            chunk_size, seed, iterations, s);
  };
  if (C <= 32) return go(std::integral_constant<int, 1>{});
  if (C <= 64) return go(std::integral_constant<int, 2>{});
  if (C <= 128) return go(std::integral_constant<int, 4>{});
  return go(std::integral_constant<int, 8>{});
}

extern "C" int bgpu_normalize_rows(const float* arr, float* out, uint64_t num_rows,
                                   uint32_t num_columns, void* stream) {
  BGPU_REQUIRE(arr && out, BGPU_ERR_INVALID, "normalize_rows: NULL argument");
  BGPU_REQUIRE(num_columns >= 1, BGPU_ERR_INVALID, "normalize_rows: no columns");
  if (num_rows == 0) return BGPU_OK;
  k_h_normalize_rows<<<(unsigned)ceil_div(num_rows * 32, kHThreads), kHThreads, 0,
                       (cudaStream_t)stream>>>(arr, out, num_rows, num_columns);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}
