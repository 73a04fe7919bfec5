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
// the GPU's results agree with it to float rounding, not bit for bit; every
// sum here runs in a fixed order, so runs are bit-identical.
//
// GPU shape. The block-sequential update is the critical path: one launch
// of k_h_block per block (one CTA per chunk), each CTA
//  - sorts its chunk's cells by batch (stable) in shared memory, so per-batch
//    sums over the chunk are runs of one batch: a register per cluster;
//  - stages tiles of the cells' R rows and Z rows in shared memory; a thread
//    per cluster sums the old R (old cluster/batch sums), then computes its
//    cluster's ratio for every batch;
//  - computes the new R rows, a warp per four cells (lanes over clusters,
//    Y in shared memory as [dim][cluster]), writes them to R and to the tile,
//    and sums them per cluster and batch; with the objective wanted, also
//    the cells' k-means error and entropy terms (those of the final R with
//    the Y of the pass: the objective after the pass);
//  - writes its chunk's changes of E and O; the last CTA of each group of 16
//    chunks (an atomic ticket after a fence, no waiting) sums the group's in
//    chunk order, and the last group adds the group sums to E and O in group
//    order, so the next block's launch sees them.
// R^T Z and the correction's R-weighted PC sums run as a register-tiled
// SIMT reduction over cell ranges (k_h_rtm), its partials summed in range
// order; the correction itself as a small GEMM per tile of one batch's cells
// (k_h_correct). The (B+1)-sized algebra of the ridge runs on the host.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "pcg.h"
#include "tma.cuh"

namespace bgpu {
namespace {

constexpr int kHThreads = 256;
constexpr int kHWarps = kHThreads / 32;
constexpr uint32_t kHMaxClusters = 256;
constexpr uint32_t kHMaxDims = 128;
constexpr uint32_t kHMaxBatches = 64;
constexpr uint32_t kHMaxChunk = 1024;
constexpr uint32_t kHCellsPerWarp = 4;       // cells a warp scores at once
constexpr size_t kHSmemBudget = 110 * 1024;      // two block CTAs per SM
constexpr size_t kHSmemBudgetOne = 220 * 1024;   // one block CTA per SM
constexpr uint32_t kHFoldGroup = 16;  // chunks folded together before the final fold

struct BlockArgs {
  const float* Z;
  const float* Y;          // d x C row-major
  const uint32_t* batch;
  const uint32_t* order;   // cell order (nullptr: natural order)
  uint64_t start, len;     // positions [start, start + len) of the order
  uint32_t d, C, B, chunk, tile;
  float tos;               // 2 / sigma
  float ens;               // exp(-2 / sigma)
  const float* Pr;         // B
  const float* theta;      // B
  float* E;                // B x C
  float* O;                // B x C
  float* R;                // n x C
  float* dE;               // chunks x B x C
  float* dO;
  float* gE;               // fold groups x B x C: per-group sums of dE, dO
  float* gO;
  double* obj;             // 2 per chunk (nullptr: objective not wanted)
  uint32_t* ticket;        // [0]: groups done; [1 + g]: chunks of group g done
  int init;                // initial assignments: no old sums, exp(tos (dot - 1))
};

// 4-byte asynchronous copy global -> shared (every copy of a tile in flight
// at once); with valid false nothing is read and zero is written.
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Shared-memory layout of k_h_block (offsets in bytes, each 16-aligned).
struct BlockSmem {
  size_t ys, zs, rs, ratio, bold, bnew, cid, cb, rid, rb, rk, seg, total;
  uint32_t cp, yst, dp;  // padded cluster count (CPL x 32), Y's row stride
                         // (cp + 1: conflict-free transposed stores), Z's
};

__host__ __device__ inline BlockSmem block_smem(uint32_t d, uint32_t C, uint32_t B,
                                                uint32_t chunk, uint32_t tile, int cpl) {
  BlockSmem L;
  L.cp = (uint32_t)cpl * 32u;
  L.yst = L.cp + 1u;
  L.dp = (d + 3u) & ~3u;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 15) & ~size_t(15);
    return at;
  };
  L.ys = take((size_t)d * L.yst * 4);
  // the sort's scratch (cells, labels, ranks in load order) is dead before
  // the first Z tile is staged: it shares the Z tile's space
  L.zs = take(std::max((size_t)tile * L.dp * 4, (size_t)chunk * 12));
  L.rid = L.zs;
  L.rb = L.zs + (size_t)chunk * 4;
  L.rk = L.zs + (size_t)chunk * 8;
  L.rs = take((size_t)tile * C * 4);
  L.ratio = take((size_t)B * C * 4);
  L.bold = take((size_t)B * C * 4);
  L.bnew = take((size_t)B * C * 4);
  L.cid = take((size_t)chunk * 4);
  L.cb = take((size_t)chunk * 4);
  L.seg = take((size_t)(B + 1) * 4);
  L.total = o;
  return L;
}

// Per-batch sums of column j over a tile of batch-sorted cells (positions
// [t0, t0 + tn) of the chunk, rows [0, tn) of rs): each batch's cells are
// the positions [seg[b], seg[b+1]); dst[b][j] += the tile's part of them
// (four interleaved partial sums, combined in a fixed order).
__device__ __forceinline__ void segment_sums(const float* rs, const uint32_t* seg, uint32_t B,
                                             uint32_t t0, uint32_t tn, uint32_t C,
                                             uint32_t j, float* dst) {
  for (uint32_t b = 0; b < B; ++b) {
    const uint32_t lo = max(seg[b], t0), hi = min(seg[b + 1], t0 + tn);
    if (lo >= hi) continue;
    float p[4] = {0.f, 0.f, 0.f, 0.f};
    const float* col = rs + (size_t)(lo - t0) * C + j;
    const uint32_t m = hi - lo;
    uint32_t i = 0;
    for (; i + 4 <= m; i += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) p[u] += col[(size_t)(i + u) * C];
    }
    for (int u = 0; i < m; ++i, ++u) p[u] += col[(size_t)i * C];
    dst[b * C + j] += (p[0] + p[1]) + (p[2] + p[3]);
  }
}

// Column sums of two row-major arrays (rows of `stride` floats, `rows` rows,
// read through L2: written by other CTAs): four interleaved partial sums per
// column (rows 4i..4i+3 in order, the remainder into the first), combined in
// a fixed order.
__device__ __forceinline__ void sum_rows4(const float* a, const float* b, uint32_t rows,
                                          uint32_t stride, float* sa, float* sb) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f, b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
  uint32_t k = 0;
  for (; k + 4 <= rows; k += 4) {
    a0 += __ldcg(a + (uint64_t)k * stride);
    a1 += __ldcg(a + (uint64_t)(k + 1) * stride);
    a2 += __ldcg(a + (uint64_t)(k + 2) * stride);
    a3 += __ldcg(a + (uint64_t)(k + 3) * stride);
    b0 += __ldcg(b + (uint64_t)k * stride);
    b1 += __ldcg(b + (uint64_t)(k + 1) * stride);
    b2 += __ldcg(b + (uint64_t)(k + 2) * stride);
    b3 += __ldcg(b + (uint64_t)(k + 3) * stride);
  }
  for (; k < rows; ++k) {
    a0 += __ldcg(a + (uint64_t)k * stride);
    b0 += __ldcg(b + (uint64_t)k * stride);
  }
  *sa = (a0 + a1) + (a2 + a3);
  *sb = (b0 + b1) + (b2 + b3);
}

template <int CPL>
__global__ void __launch_bounds__(kHThreads, 2) k_h_block(BlockArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t d = a.d, C = a.C, B = a.B;
  const BlockSmem L = block_smem(d, C, B, a.chunk, a.tile, CPL);
  float* ys = (float*)(smem + L.ys);
  float* zs = (float*)(smem + L.zs);
  float* rs = (float*)(smem + L.rs);
  float* ratio = (float*)(smem + L.ratio);
  float* bold = (float*)(smem + L.bold);
  float* bnew = (float*)(smem + L.bnew);
  uint32_t* cid = (uint32_t*)(smem + L.cid);
  uint32_t* cb = (uint32_t*)(smem + L.cb);
  uint32_t* rid = (uint32_t*)(smem + L.rid);
  uint32_t* rb = (uint32_t*)(smem + L.rb);
  uint32_t* rk = (uint32_t*)(smem + L.rk);
  uint32_t* seg = (uint32_t*)(smem + L.seg);
  __shared__ double red[2][kHWarps];
  __shared__ uint32_t wcnt[kHWarps][kHMaxBatches];
  __shared__ uint32_t running[kHMaxBatches];
  __shared__ int is_last;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint64_t p0 = a.start + (uint64_t)blockIdx.x * a.chunk;
  const uint32_t ncell = (uint32_t)min_u64(a.chunk, a.start + a.len - p0);
  const uint32_t cp = L.cp, yst = L.yst, dp = L.dp;

  // Y transposed ([dim][cluster], rows of yst) and zero-padded to cp
  // clusters, by asynchronous copies: a warp per cluster, lanes over dims
  for (uint32_t jj = wid; jj < cp; jj += kHWarps)
    for (uint32_t k = lane; k < d; k += 32) {
      if (jj < C)
        cp_async4(ys + k * yst + jj, a.Y + (uint64_t)jj * d + k, true);
      else
        ys[k * yst + jj] = 0.f;
    }
  for (uint32_t i = tid; i < ncell; i += kHThreads) {
    const uint32_t c = a.order ? a.order[p0 + i] : (uint32_t)(p0 + i);
    rid[i] = c;
    rb[i] = a.batch[c];
  }
  for (uint32_t t = tid; t < B * C; t += kHThreads) {
    bold[t] = 0.f;
    bnew[t] = 0.f;
  }
  for (uint32_t t = tid; t < kHWarps * kHMaxBatches; t += kHThreads) (&wcnt[0][0])[t] = 0u;
  if (tid < (int)kHMaxBatches) running[tid] = 0u;
  __syncthreads();
  // stable counting sort by batch: a cell's rank among earlier cells of its
  // batch from warp matches and per-warp counts, 256 cells per round
  for (uint32_t r0 = 0; r0 < ncell; r0 += kHThreads) {
    const uint32_t i = r0 + tid;
    const bool valid = i < ncell;
    const uint32_t b = valid ? rb[i] : kHMaxBatches;
    const uint32_t peers = __match_any_sync(0xffffffffu, b);
    const uint32_t below = peers & ((1u << lane) - 1u);
    if (valid && below == 0u) wcnt[wid][b] = __popc(peers);
    __syncthreads();
    if (valid) {
      uint32_t rank = running[b] + __popc(below);
      for (int w = 0; w < wid; ++w) rank += wcnt[w][b];
      rk[i] = rank;
    }
    __syncthreads();
    if (tid < (int)B) {
      uint32_t t = 0;
      for (int w = 0; w < kHWarps; ++w) {
        t += wcnt[w][tid];
        wcnt[w][tid] = 0u;
      }
      running[tid] += t;
    }
    __syncthreads();
  }
  if (tid == 0) {
    uint32_t t = 0;
    for (uint32_t b = 0; b < B; ++b) {
      seg[b] = t;
      t += running[b];
    }
    seg[B] = t;
  }
  __syncthreads();
  for (uint32_t i = tid; i < ncell; i += kHThreads) {
    const uint32_t b = rb[i], pos = seg[b] + rk[i];
    cid[pos] = rid[i];
    cb[pos] = b;
  }
  __syncthreads();
  // tile 0 of the old R rows and of the Z rows, with Y, in one wait; a warp
  // per cell row, lanes along it
  auto stage_r = [&](uint32_t t0, uint32_t tn) {
    for (uint32_t i = wid; i < tn; i += kHWarps) {
      const float* src = a.R + (uint64_t)cid[t0 + i] * C;
      for (uint32_t c = lane; c < C; c += 32) cp_async4(rs + i * C + c, src + c, true);
    }
  };
  auto stage_z = [&](uint32_t t0, uint32_t tn) {
    for (uint32_t i = wid; i < tn; i += kHWarps) {
      const float* src = a.Z + (uint64_t)cid[t0 + i] * d;
      for (uint32_t k = lane; k < dp; k += 32)
        cp_async4(zs + i * dp + k, k < d ? src + k : src, k < d);
    }
  };
  if (!a.init) stage_r(0, min(a.tile, ncell));
  stage_z(0, min(a.tile, ncell));
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();

  const uint32_t j = tid;  // the thread's cluster in the per-cluster phases
  float rold = 0.f;
  if (!a.init) {
    // old contributions of the chunk's cells
    for (uint32_t t0 = 0; t0 < ncell; t0 += a.tile) {
      const uint32_t tn = min(a.tile, ncell - t0);
      if (t0 > 0) {
        stage_r(t0, tn);
        cp_async_commit();
        cp_async_wait<0>();
        __syncthreads();
      }
      if (j < C) segment_sums(rs, seg, B, t0, tn, C, j, bold);
      __syncthreads();
    }
    if (j < C) {
      for (uint32_t b = 0; b < B; ++b) rold += bold[b * C + j];
      // the block's ratio for this cluster (harmonize.pyx:585-598)
      for (uint32_t b = 0; b < B; ++b) {
        const float Eij = a.E[b * C + j] + -a.Pr[b] * rold;
        const float Oij = a.O[b * C + j] - bold[b * C + j];
        ratio[b * C + j] = a.ens * powf((Eij + 1.f) / (Oij + Eij + 1.f), a.theta[b]);
      }
    }
    __syncthreads();
  }

  // new assignments, tile by tile
  double ke = 0.0, en = 0.0;
  for (uint32_t t0 = 0; t0 < ncell; t0 += a.tile) {
    const uint32_t tn = min(a.tile, ncell - t0);
    if (t0 > 0) {
      stage_z(t0, tn);
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
    }
    const uint32_t groups = (tn + kHCellsPerWarp - 1) / kHCellsPerWarp;
    for (uint32_t g = wid; g < groups; g += kHWarps) {
      const uint32_t i0 = g * kHCellsPerWarp;
      float dot[kHCellsPerWarp][CPL];
#pragma unroll
      for (int c = 0; c < (int)kHCellsPerWarp; ++c)
#pragma unroll
        for (int q = 0; q < CPL; ++q) dot[c][q] = 0.f;
      // rows past the tile re-read its last row: in bounds, results unused
      const float* z0 = zs + (size_t)min(i0 + 0, tn - 1) * dp;
      const float* z1 = zs + (size_t)min(i0 + 1, tn - 1) * dp;
      const float* z2 = zs + (size_t)min(i0 + 2, tn - 1) * dp;
      const float* z3 = zs + (size_t)min(i0 + 3, tn - 1) * dp;
      for (uint32_t k = 0; k < dp; k += 4) {
        const float4 v0 = *(const float4*)(z0 + k), v1 = *(const float4*)(z1 + k);
        const float4 v2 = *(const float4*)(z2 + k), v3 = *(const float4*)(z3 + k);
        const float za[4][4] = {{v0.x, v0.y, v0.z, v0.w}, {v1.x, v1.y, v1.z, v1.w},
                                {v2.x, v2.y, v2.z, v2.w}, {v3.x, v3.y, v3.z, v3.w}};
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          if (k + kk >= d) break;
          const float* yk = ys + (size_t)(k + kk) * yst + lane;
#pragma unroll
          for (int q = 0; q < CPL; ++q) {
            const float y = yk[32 * q];
#pragma unroll
            for (int c = 0; c < (int)kHCellsPerWarp; ++c)
              dot[c][q] = fmaf(za[c][kk], y, dot[c][q]);
          }
        }
      }
#pragma unroll
      for (int c = 0; c < (int)kHCellsPerWarp; ++c) {
        const uint32_t i = i0 + c;
        if (i >= tn) break;
        const uint32_t cell = cid[t0 + i], b = cb[t0 + i];
        float r[CPL], s = 0.f;
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t jj = lane + 32u * q;
          float v = 0.f;
          if (jj < C)
            v = a.init ? expf(a.tos * (dot[c][q] - 1.f))
                       : expf(a.tos * dot[c][q]) * ratio[b * C + jj];
          r[q] = v;
          s += v;
        }
        const float inv = 1.f / warp_sum(s);
#pragma unroll
        for (int q = 0; q < CPL; ++q) {
          const uint32_t jj = lane + 32u * q;
          if (jj < C) {
            const float v = r[q] * inv;
            a.R[(uint64_t)cell * C + jj] = v;
            rs[i * C + jj] = v;
            if (a.obj) {
              ke += (double)(v * (1.f - dot[c][q]));
              if (v > 0.f) en += (double)(v * logf(v));
            }
          }
        }
      }
    }
    __syncthreads();
    if (j < C) segment_sums(rs, seg, B, t0, tn, C, j, bnew);
    __syncthreads();
  }
  if (j < C) {
    float rnew = 0.f;
    for (uint32_t b = 0; b < B; ++b) rnew += bnew[b * C + j];
    for (uint32_t b = 0; b < B; ++b) {
      const uint64_t o = ((uint64_t)blockIdx.x * B + b) * C + j;
      a.dE[o] = -a.Pr[b] * rold + a.Pr[b] * rnew;
      a.dO[o] = -bold[b * C + j] + bnew[b * C + j];
    }
  }
  if (a.obj) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ke += __shfl_xor_sync(0xffffffffu, ke, o);
      en += __shfl_xor_sync(0xffffffffu, en, o);
    }
    if (lane == 0) {
      red[0][wid] = ke;
      red[1][wid] = en;
    }
    __syncthreads();
    if (tid == 0) {
      double x = 0.0, y = 0.0;
      for (int w = 0; w < kHWarps; ++w) {
        x += red[0][w];
        y += red[1][w];
      }
      a.obj[2 * blockIdx.x] = x;
      a.obj[2 * blockIdx.x + 1] = y;
    }
  }
  // Fold every chunk's changes into E and O in two levels, with atomic
  // tickets after fences (no waiting): the last CTA of each group of
  // kHFoldGroup consecutive chunks sums the group's changes in chunk order;
  // the last group to finish adds the group sums to E and O in group order.
  __threadfence();
  __syncthreads();
  const uint32_t BC = B * C, nch = gridDim.x;
  const uint32_t gi = blockIdx.x / kHFoldGroup, ngroups = (nch + kHFoldGroup - 1) / kHFoldGroup;
  const uint32_t c0 = gi * kHFoldGroup, gsz = min(kHFoldGroup, nch - c0);
  if (tid == 0) is_last = atomicAdd(a.ticket + 1 + gi, 1u) == gsz - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (uint32_t t = tid; t < BC; t += kHThreads) {
    float e, o;
    sum_rows4(a.dE + (uint64_t)c0 * BC + t, a.dO + (uint64_t)c0 * BC + t, gsz, BC, &e, &o);
    a.gE[(uint64_t)gi * BC + t] = e;
    a.gO[(uint64_t)gi * BC + t] = o;
  }
  if (tid == 0) a.ticket[1 + gi] = 0u;
  __threadfence();
  __syncthreads();
  if (tid == 0) is_last = atomicAdd(a.ticket, 1u) == ngroups - 1;
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (uint32_t t = tid; t < BC; t += kHThreads) {
    float e, o;
    sum_rows4(a.gE + t, a.gO + t, ngroups, BC, &e, &o);
    a.E[t] += e;
    a.O[t] += o;
  }
  if (tid == 0) *a.ticket = 0u;
}

// part[r][j][k] = sum over the cells of range r (positions starts[r] ..
// starts[r+1] of `cells`, or the cells themselves when cells is nullptr) of
// R[cell][j] M[cell][k]. A CTA per (range, 128 x 64 output slab); each
// thread an 8 x 4 register tile; tiles of 32 cells double-buffered in shared
// memory by asynchronous copies. Summation over cells in range order.
constexpr uint32_t kRtmCells = 32, kRtmJ = 128, kRtmK = 64;
constexpr uint32_t kRtmStage = kRtmCells * (kRtmJ + kRtmK);  // floats per buffer
constexpr size_t kRtmSmem = 2ull * kRtmStage * 4;             // 48 KB
__global__ void __launch_bounds__(kHThreads)
k_h_rtm(const float* __restrict__ R, const float* __restrict__ M,
        const uint32_t* __restrict__ cells, const uint64_t* __restrict__ starts, uint32_t d,
        uint32_t C, uint32_t kslabs, float* __restrict__ part) {
  extern __shared__ __align__(16) float rsm[];
  const int tid = threadIdx.x;
  const uint32_t j0 = (blockIdx.y / kslabs) * kRtmJ, k0 = (blockIdx.y % kslabs) * kRtmK;
  const uint32_t tj = tid >> 4, tk = tid & 15;
  const uint64_t a = starts[blockIdx.x], b = starts[blockIdx.x + 1];
  float acc[8][4];
#pragma unroll
  for (int x = 0; x < 8; ++x)
#pragma unroll
    for (int y = 0; y < 4; ++y) acc[x][y] = 0.f;
  auto stage = [&](uint32_t buf, uint64_t base) {
    float* rt = rsm + buf * kRtmStage;  // [32][128]
    float* mt = rt + kRtmCells * kRtmJ;  // [32][64]
    for (uint32_t e = tid; e < kRtmCells * kRtmJ; e += kHThreads) {
      const uint32_t i = e / kRtmJ, c = e % kRtmJ;
      const uint64_t pos = base + i;
      const bool v = pos < b && j0 + c < C;
      const uint64_t cell = v ? (cells ? (uint64_t)cells[pos] : pos) : 0;
      cp_async4(rt + e, R + (v ? cell * C + j0 + c : 0), v);
    }
    for (uint32_t e = tid; e < kRtmCells * kRtmK; e += kHThreads) {
      const uint32_t i = e / kRtmK, c = e % kRtmK;
      const uint64_t pos = base + i;
      const bool v = pos < b && k0 + c < d;
      const uint64_t cell = v ? (cells ? (uint64_t)cells[pos] : pos) : 0;
      cp_async4(mt + e, M + (v ? cell * d + k0 + c : 0), v);
    }
    cp_async_commit();
  };
  const uint64_t ntiles = (b - a + kRtmCells - 1) / kRtmCells;
  if (ntiles) stage(0, a);
  for (uint64_t t = 0; t < ntiles; ++t) {
    // buffer (t + 1) & 1 was last read in iteration t - 1, which ended in a
    // barrier
    if (t + 1 < ntiles) {
      stage((uint32_t)((t + 1) & 1), a + (t + 1) * kRtmCells);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* rt = rsm + (t & 1) * kRtmStage;
    const float* mt = rt + kRtmCells * kRtmJ;
#pragma unroll 4
    for (uint32_t i = 0; i < kRtmCells; ++i) {
      const float4 x0 = *(const float4*)(rt + i * kRtmJ + tj * 8);
      const float4 x1 = *(const float4*)(rt + i * kRtmJ + tj * 8 + 4);
      const float4 y = *(const float4*)(mt + i * kRtmK + tk * 4);
      const float xv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
      const float yv[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
      for (int p = 0; p < 8; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(xv[p], yv[q], acc[p][q]);
    }
    __syncthreads();
  }
  float* out = part + (uint64_t)blockIdx.x * C * d;
#pragma unroll
  for (int p = 0; p < 8; ++p) {
    const uint32_t jj = j0 + tj * 8 + p;
    if (jj >= C) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t kk = k0 + tk * 4 + q;
      if (kk < d) out[(uint64_t)jj * d + kk] = acc[p][q];
    }
  }
}

// out[j][k] = sum over ranges c in [c0, c1) of part[c][j][k] (four
// interleaved partial sums, combined in a fixed order); with normalise, each
// row scaled by 1 / sqrt(sum of squares). One CTA per row, a thread per
// dimension (d <= 128).
__global__ void k_h_rtm_reduce(const float* __restrict__ part, uint32_t c0, uint32_t c1,
                               uint32_t d, uint32_t C, int normalise, float* __restrict__ out) {
  __shared__ float red[4];
  __shared__ float scale;
  const uint32_t j = blockIdx.x, k = threadIdx.x;
  float v = 0.f;
  if (k < d) {
    float p[4] = {0.f, 0.f, 0.f, 0.f};
    uint32_t c = c0;
    for (; c + 4 <= c1; c += 4)
#pragma unroll
      for (int u = 0; u < 4; ++u) p[u] += part[((uint64_t)(c + u) * C + j) * d + k];
    for (int u = 0; c < c1; ++c, ++u) p[u] += part[((uint64_t)c * C + j) * d + k];
    v = (p[0] + p[1]) + (p[2] + p[3]);
  }
  if (normalise) {
    const float sq = warp_sum(k < d ? v * v : 0.f);
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

// Z = PCs - sum_k R[cell][k] W[k][batch][:] (harmonize.pyx:814-818), then,
// with normalise, each row scaled to unit norm. A CTA per tile of up to 64
// consecutive cells of the batch-sorted order, all of one batch: a small
// GEMM (cells x clusters) x (clusters x dims) with W's rows for that batch.
// Each thread 4 cells x KPT dims; 32 clusters at a time staged in shared
// memory (R transposed, W's rows), by asynchronous copies.
constexpr uint32_t kCorCells = 64, kCorC = 32, kCorRt = 68;  // 16-byte rows of rt
template <int KPT>
__global__ void __launch_bounds__(kHThreads)
k_h_correct(const float* __restrict__ PCs, const float* __restrict__ R, const float* __restrict__ W,
            const uint32_t* __restrict__ border, const uint64_t* __restrict__ tiles,
            const uint32_t* __restrict__ tile_batch, uint32_t d, uint32_t C, uint32_t B,
            int normalise, float* __restrict__ Z) {
  constexpr uint32_t kp = 16 * KPT;
  __shared__ __align__(16) float rt[kCorC][kCorRt];  // [cluster][cell]
  __shared__ __align__(16) float wt[kCorC][kp];      // [cluster][dim]
  __shared__ uint32_t ids[kCorCells];
  const int tid = threadIdx.x, ti = tid >> 4, tk = tid & 15;
  const uint64_t p0 = tiles[blockIdx.x];
  const uint32_t nc = (uint32_t)(tiles[blockIdx.x + 1] - p0), b = tile_batch[blockIdx.x];
  if (tid < (int)nc) ids[tid] = border[p0 + tid];
  __syncthreads();
  float acc[4][KPT];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < KPT; ++q) acc[p][q] = 0.f;
  for (uint32_t c0 = 0; c0 < C; c0 += kCorC) {
    for (uint32_t e = tid; e < kCorCells * kCorC; e += kHThreads) {
      const uint32_t i = e / kCorC, c = e % kCorC;
      const bool v = i < nc && c0 + c < C;
      cp_async4(&rt[c][i], R + (v ? (uint64_t)ids[i] * C + c0 + c : 0), v);
    }
    for (uint32_t e = tid; e < kCorC * kp; e += kHThreads) {
      const uint32_t c = e / kp, k = e % kp;
      const bool v = c0 + c < C && k < d;
      cp_async4(&wt[c][k], W + (v ? ((uint64_t)(c0 + c) * (B + 1) + b) * d + k : 0), v);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
#pragma unroll 4
    for (uint32_t c = 0; c < kCorC; ++c) {
      const float4 x = *(const float4*)&rt[c][ti * 4];
      const float xv[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int u = 0; u < KPT / 4; ++u) {
        const float4 w = *(const float4*)&wt[c][tk * KPT + 4 * u];
        const float wv[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int p = 0; p < 4; ++p)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[p][4 * u + q] = fmaf(xv[p], wv[q], acc[p][4 * u + q]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const uint32_t i = ti * 4 + p;
    const bool valid = i < nc;
    const uint64_t cell = valid ? ids[i] : 0;
    float z[KPT], sq = 0.f;
#pragma unroll
    for (int q = 0; q < KPT; ++q) {
      const uint32_t k = tk * KPT + q;
      z[q] = (valid && k < d) ? PCs[cell * d + k] - acc[p][q] : 0.f;
      sq += z[q] * z[q];
    }
    float scale = 1.f;
    if (normalise) {  // the cell's 16 threads are 16 consecutive lanes
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
      scale = 1.f / sqrtf(sq);
    }
#pragma unroll
    for (int q = 0; q < KPT; ++q) {
      const uint32_t k = tk * KPT + q;
      if (valid && k < d) Z[cell * d + k] = z[q] * scale;
    }
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

// Tile (cells staged at once) of the block kernel: the chunk split into the
// fewest equal tiles (a multiple of 4 cells) whose layout fits the budget; 0
// when even 4 cells do not fit.
uint32_t block_tile(uint32_t d, uint32_t C, uint32_t B, uint32_t chunk, int cpl,
                    size_t budget) {
  for (uint32_t nt = 1; nt <= chunk; ++nt) {
    const uint32_t tile = (uint32_t)round_up(ceil_div(chunk, nt), 4);
    if (block_smem(d, C, B, chunk, tile, cpl).total <= budget) return tile;
    if (tile == 4) break;
  }
  return 0;
}

// Two CTAs per SM when a tile of at least 32 cells (or the whole chunk) fits
// in half the shared memory, else one CTA per SM with the larger tile.
uint32_t choose_tile(uint32_t d, uint32_t C, uint32_t B, uint32_t chunk, int cpl) {
  const uint32_t two = block_tile(d, C, B, chunk, cpl, kHSmemBudget);
  if (two >= std::min<uint32_t>(chunk, 32)) return two;
  return std::max(two, block_tile(d, C, B, chunk, cpl, kHSmemBudgetOne));
}

int ranges_rtm(const float* R, const float* M, const uint32_t* cells, const uint64_t* starts,
               uint32_t nranges, uint32_t d, uint32_t C, float* part, cudaStream_t s) {
  const uint32_t jslabs = (uint32_t)ceil_div(C, kRtmJ), kslabs = (uint32_t)ceil_div(d, kRtmK);
  k_h_rtm<<<dim3(nranges, jslabs * kslabs), kHThreads, kRtmSmem, s>>>(R, M, cells, starts, d,
                                                                     C, kslabs, part);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

template <int CPL>
int harmony_run(const float* PCs, float* Z, float* Y, float* R, const uint32_t* batch,
                uint64_t n, uint32_t d, uint32_t C, uint32_t B, uint32_t max_iter,
                uint32_t max_ci, float block_prop, float tol, int early, float ctol,
                float theta, float tau, float alpha, float sigma, uint32_t chunk, uint64_t seed,
                uint32_t tile, uint32_t* iters, cudaStream_t s) {
  const uint32_t BC = B * C;
  const uint32_t nchunks = (uint32_t)ceil_div(n, chunk);
  // the reference multiplies an unsigned long long by a float: float product
  const uint64_t block = (uint64_t)std::ceil((float)n * block_prop);
  const uint32_t max_cpb = (uint32_t)ceil_div(block, chunk);
  const uint32_t nblocks = (uint32_t)ceil_div(n, block);
  const float tos = 2.f / sigma;
  const size_t smem_blk = block_smem(d, C, B, chunk, tile, CPL).total;
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
  // batch-sorted cells (stable) and ranges that never straddle batches
  std::vector<uint32_t> border(n);
  std::vector<uint64_t> bstart(B + 1, 0), starts_b, starts_nat;
  for (uint32_t b = 0; b < B; ++b) bstart[b + 1] = bstart[b] + Nb[b];
  {
    std::vector<uint64_t> pos(bstart.begin(), bstart.end() - 1);
    for (uint64_t i = 0; i < n; ++i) border[pos[hb[i]]++] = (uint32_t)i;
  }
  const uint64_t rchunk = 2048;
  std::vector<uint32_t> brange0(B + 1, 0);
  for (uint32_t b = 0; b < B; ++b) {
    brange0[b] = (uint32_t)starts_b.size();
    for (uint64_t p = bstart[b]; p < bstart[b + 1]; p += rchunk) starts_b.push_back(p);
  }
  brange0[B] = (uint32_t)starts_b.size();
  starts_b.push_back(n);
  for (uint64_t p = 0; p < n; p += rchunk) starts_nat.push_back(p);
  starts_nat.push_back(n);
  std::vector<uint64_t> cor_tiles;
  std::vector<uint32_t> cor_batch;
  for (uint32_t b = 0; b < B; ++b)
    for (uint64_t p = bstart[b]; p < bstart[b + 1]; p += kCorCells) {
      cor_tiles.push_back(p);
      cor_batch.push_back(b);
    }
  cor_tiles.push_back(n);
  const uint32_t ncor = (uint32_t)cor_batch.size();
  const uint32_t nr_nat = (uint32_t)starts_nat.size() - 1;
  const uint32_t nr_b = (uint32_t)starts_b.size() - 1;
  const uint32_t npart = std::max(nr_nat, nr_b);
  const uint32_t nobj = std::max(nchunks, nblocks * max_cpb);
  const uint32_t max_launch_chunks = std::max(nchunks, max_cpb);
  const uint32_t max_groups = (uint32_t)ceil_div(max_launch_chunks, kHFoldGroup);

  float *E, *O, *Pr_d, *th_d, *dE, *dO, *gE, *gO, *part, *W;
  double* obj;
  uint32_t *order_d, *border_d, *ticket;
  uint64_t *starts_nat_d, *starts_b_d, *cor_tiles_d;
  uint32_t* cor_batch_d;
  std::vector<void*> allocs;
  auto dalloc = [&](auto** p, size_t bytes) -> int {
    void* q = nullptr;
    BGPU_CUDA(cudaMallocAsync(&q, std::max<size_t>(bytes, 16), s));
    allocs.push_back(q);
    *p = (std::remove_reference_t<decltype(**p)>*)q;
    return BGPU_OK;
  };
  auto body = [&]() -> int {
    BGPU_TRY(dalloc(&E, BC * 4ull));
    BGPU_TRY(dalloc(&O, BC * 4ull));
    BGPU_TRY(dalloc(&Pr_d, B * 4ull));
    BGPU_TRY(dalloc(&th_d, B * 4ull));
    BGPU_TRY(dalloc(&dE, (uint64_t)max_launch_chunks * BC * 4));
    BGPU_TRY(dalloc(&dO, (uint64_t)max_launch_chunks * BC * 4));
    BGPU_TRY(dalloc(&gE, (uint64_t)max_groups * BC * 4));
    BGPU_TRY(dalloc(&gO, (uint64_t)max_groups * BC * 4));
    BGPU_TRY(dalloc(&part, (uint64_t)npart * C * d * 4));
    BGPU_TRY(dalloc(&W, (uint64_t)C * (B + 1) * d * 4));
    BGPU_TRY(dalloc(&obj, (uint64_t)nobj * 16));
    BGPU_TRY(dalloc(&order_d, n * 4));
    BGPU_TRY(dalloc(&border_d, n * 4));
    BGPU_TRY(dalloc(&ticket, (1ull + max_groups) * 4));
    BGPU_TRY(dalloc(&starts_nat_d, starts_nat.size() * 8));
    BGPU_TRY(dalloc(&starts_b_d, starts_b.size() * 8));
    BGPU_TRY(dalloc(&cor_tiles_d, cor_tiles.size() * 8));
    BGPU_TRY(dalloc(&cor_batch_d, cor_batch.size() * 4));
    BGPU_CUDA(cudaMemcpyAsync(cor_tiles_d, cor_tiles.data(), cor_tiles.size() * 8,
                              cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(cor_batch_d, cor_batch.data(), cor_batch.size() * 4,
                              cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(Pr_d, Pr.data(), B * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(th_d, th.data(), B * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(order_d, order.data(), n * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(border_d, border.data(), n * 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(starts_nat_d, starts_nat.data(), starts_nat.size() * 8,
                              cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(starts_b_d, starts_b.data(), starts_b.size() * 8,
                              cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemsetAsync(ticket, 0, (1ull + max_groups) * 4, s));
    BGPU_CUDA(cudaMemsetAsync(E, 0, BC * 4ull, s));
    BGPU_CUDA(cudaMemsetAsync(O, 0, BC * 4ull, s));
    BGPU_CUDA(cudaMemsetAsync(obj, 0, (uint64_t)nobj * 16, s));

    std::vector<float> hE(BC), hO(BC), hpart;
    std::vector<double> hobj(2ull * nobj);
    // objective (harmonize.pyx:466-498, 658-695): k-means error and entropy
    // from the per-chunk partials, the diversity penalty from E and O
    auto objective = [&](float* out) -> int {
      BGPU_CUDA(cudaMemcpyAsync(hE.data(), E, BC * 4ull, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaMemcpyAsync(hO.data(), O, BC * 4ull, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaMemcpyAsync(hobj.data(), obj, hobj.size() * 8, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaStreamSynchronize(s));
      double ke = 0.0, en = 0.0, pen = 0.0;
      for (uint32_t c = 0; c < nobj; ++c) {
        ke += hobj[2 * c];
        en += hobj[2 * c + 1];
      }
      for (uint32_t j = 0; j < C; ++j) {
        float cj = 0.f;
        for (uint32_t b = 0; b < B; ++b) {
          const float o = hO[b * C + j], e = hE[b * C + j];
          cj += (o * std::log((o + e + 1.f) / (e + 1.f))) * th[b];
        }
        pen += cj;
      }
      *out = (float)(2.0 * ke) + (float)(sigma * en) + (float)(sigma * pen);
      return BGPU_OK;
    };
    BlockArgs ba{};
    ba.Z = Z;
    ba.Y = Y;
    ba.batch = batch;
    ba.d = d;
    ba.C = C;
    ba.B = B;
    ba.chunk = chunk;
    ba.tile = tile;
    ba.tos = tos;
    ba.ens = std::exp(-tos);
    ba.Pr = Pr_d;
    ba.theta = th_d;
    ba.E = E;
    ba.O = O;
    ba.R = R;
    ba.dE = dE;
    ba.dO = dO;
    ba.gE = gE;
    ba.gO = gO;
    ba.ticket = ticket;
    // initialisation over natural chunks, with the unnormalised Y
    ba.order = nullptr;
    ba.start = 0;
    ba.len = n;
    ba.obj = obj;
    ba.init = 1;
    k_h_block<CPL><<<nchunks, kHThreads, smem_blk, s>>>(ba);
    BGPU_CHECK_LAUNCH();
    float prev;
    BGPU_TRY(objective(&prev));
    // normalise Y's rows (harmonize.pyx:501)
    BGPU_CUDA(cudaMemcpyAsync(part, Y, (uint64_t)C * d * 4, cudaMemcpyDeviceToDevice, s));
    k_h_rtm_reduce<<<C, 128, 0, s>>>(part, 0, 1, d, C, 1, Y);
    BGPU_CHECK_LAUNCH();
    float objective_v = prev;
    ba.order = order_d;
    ba.init = 0;
    uint32_t it = 0;
    for (it = 1; it <= max_iter; ++it) {
      float past[3] = {0.f, 0.f, 0.f};
      for (uint32_t ci = 1; ci <= max_ci; ++ci) {
        // Y = normalise(R^T Z)
        BGPU_TRY(ranges_rtm(R, Z, nullptr, starts_nat_d, nr_nat, d, C, part, s));
        k_h_rtm_reduce<<<C, 128, 0, s>>>(part, 0, nr_nat, d, C, 1, Y);
        BGPU_CHECK_LAUNCH();
        const bool want = early || ci == max_ci;
        if (want) BGPU_CUDA(cudaMemsetAsync(obj, 0, (uint64_t)nobj * 16, s));
        for (uint32_t bi = 0; bi < nblocks; ++bi) {
          ba.start = (uint64_t)bi * block;
          ba.len = std::min<uint64_t>(block, n - ba.start);
          ba.obj = want ? obj + 2ull * bi * max_cpb : nullptr;
          k_h_block<CPL><<<(unsigned)ceil_div(ba.len, chunk), kHThreads, smem_blk, s>>>(ba);
          BGPU_CHECK_LAUNCH();
        }
        if (want) {
          BGPU_TRY(objective(&objective_v));
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
      BGPU_TRY(ranges_rtm(R, PCs, border_d, starts_b_d, nr_b, d, C, part, s));
      hpart.resize((uint64_t)nr_b * C * d);
      BGPU_CUDA(cudaMemcpyAsync(hpart.data(), part, hpart.size() * 4, cudaMemcpyDeviceToHost,
                                s));
      BGPU_CUDA(cudaStreamSynchronize(s));
      std::vector<float> Wh((uint64_t)C * (B + 1) * d, 0.f);
      std::vector<float> inv1((B + 1) * (B + 1)), inv2((B + 1) * (B + 1), 0.f),
          inv((B + 1) * (B + 1)), rs((uint64_t)d * (B + 1));
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
        for (uint32_t jd = 0; jd < d; ++jd) {
          float total = 0.f;
          for (uint32_t b = 0; b < B; ++b) {
            float bt = 0.f;
            if (!(hO[b * C + k] < 1e-5f * (float)Nb[b]))
              for (uint32_t c = brange0[b]; c < brange0[b + 1]; ++c)
                bt += hpart[((uint64_t)c * C + k) * d + jd];
            rs[jd * (B + 1) + b] = bt;
            total += bt;
          }
          rs[jd * (B + 1) + B] = total;
        }
        for (uint32_t r = 0; r <= B; ++r)  // W[k] = inv rs^T
          for (uint32_t jd = 0; jd < d; ++jd) {
            float t = 0.f;
            for (uint32_t q = 0; q <= B; ++q) t += inv[r * (B + 1) + q] * rs[jd * (B + 1) + q];
            Wh[((uint64_t)k * (B + 1) + r) * d + jd] = t;
          }
      }
      BGPU_CUDA(cudaMemcpyAsync(W, Wh.data(), Wh.size() * 4, cudaMemcpyHostToDevice, s));
      const bool done = prev - objective_v < tol * std::fabs(prev);
      if (d <= 64)
        k_h_correct<4><<<ncor, kHThreads, 0, s>>>(PCs, R, W, border_d, cor_tiles_d, cor_batch_d,
                                                   d, C, B, done ? 0 : 1, Z);
      else
        k_h_correct<8><<<ncor, kHThreads, 0, s>>>(PCs, R, W, border_d, cor_tiles_d, cor_batch_d,
                                                   d, C, B, done ? 0 : 1, Z);
      BGPU_CHECK_LAUNCH();
      BGPU_CUDA(cudaStreamSynchronize(s));  // Wh is read by the copy above
      if (done) break;
      prev = objective_v;
    }
    *iters = std::min(it, max_iter);
    return BGPU_OK;
  };
  const int rc = body();
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
  cudaStream_t s = (cudaStream_t)stream;
  auto go = [&](auto cpl) -> int {
    constexpr int CPL = decltype(cpl)::value;
    const uint32_t tile = choose_tile(d, C, B, chunk_size, CPL);
    BGPU_REQUIRE(tile > 0, BGPU_ERR_UNSUPPORTED,
                 "harmony: num_PCs x num_clusters + 3 num_batches x num_clusters too large");
    BGPU_CUDA(cudaFuncSetAttribute(k_h_block<CPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kHSmemBudgetOne));
    BGPU_CUDA(cudaFuncSetAttribute(k_h_rtm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kRtmSmem));
    return harmony_run<CPL>(PCs, Z, Y, R, batch_labels, n, d, C, B, max_iterations,
                            max_clustering_iterations, block_proportion, tolerance,
                            early_stopping, clustering_tolerance, theta, tau, alpha, sigma,
                            chunk_size, seed, tile, iterations, s);
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
