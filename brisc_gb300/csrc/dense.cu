// Dense kernels of the IRLBA solve: the fused U pass of brisc/pca.pyx:997-1090
// split into fixed-block dot / update kernels (classical Gram-Schmidt: once as
// the reference, a second time only where the first cancels, or always twice
// for CGS2), the V-side step of pca.pyx:1103-1171 and the tall-skinny
// rotations of pca.pyx:1210-1255.
//
// Determinism: every sum is either a per-thread sequence in a fixed order, a
// fixed xor-shuffle tree, or a sum over fixed 1024-row blocks in block order.
#include <algorithm>

#include <cooperative_groups.h>

#include "dense.cuh"
#include "tma.cuh"

namespace cg = cooperative_groups;

namespace bgpu {

namespace {

// The kernel bodies below are shared by a single-solve kernel and its
// multi-task form (multi.cuh). Their products and sums are written with
// explicit rounding intrinsics: the compiler may not fuse a multiply and an
// add one way in one kernel and another way in the other, so both compute
// the same bits.
__device__ __forceinline__ float dot4(float4 a, float4 b) {
  return __fmaf_rn(a.w, b.w, __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x))));
}
__device__ __forceinline__ float sumsq4(float a, float b, float c, float d) {
  return __fmaf_rn(d, d, __fmaf_rn(c, c, __fmaf_rn(b, b, __fmul_rn(a, a))));
}

// Adaptive second Gram-Schmidt pass: gate = {|y1|^2, |y0 - mean|^2} of the
// first pass. When the first pass kept at least half of the squared norm, y1
// is orthogonal to U to working precision (Kahan-Parlett "twice is enough")
// and the second pass's kernels return at once. Every block of every kernel
// reads the same two numbers and takes the same decision.
__device__ __forceinline__ bool second_pass_skipped(const float* gate) {
  return gate != nullptr && gate[0] >= 0.5f * gate[1];
}

// Per-warp column sums go to shared memory ([warp][column], no block barrier
// per chunk, so a warp's next 16 loads issue while the others reduce); one
// barrier at the end, then part[b][c] = the 8 warp sums in warp order.
// __launch_bounds__(256, 8): 32 registers, so the 1024-row blocks of a
// million-cell basis (977) all run in one wave (8 per SM, 2048 threads, each
// with kDotCols 16-byte loads in flight).
constexpr int kDotCols = 4;

__device__ __forceinline__ void udots_body(const float* __restrict__ U, uint64_t ldu,
                                           uint32_t ncols, const float* __restrict__ y,
                                           float* __restrict__ part, uint32_t pstride,
                                           int with_sum, const float* __restrict__ gate,
                                           uint64_t b) {
  if (second_pass_skipped(gate)) return;
  extern __shared__ float wsum[];  // 8 x (ncols + 1)
  const uint32_t ld = ncols + 1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint64_t row0 = b * kRowBlock + threadIdx.x * 4ull;
  const bool in = row0 < ldu;
  const float4 yv = in ? *reinterpret_cast<const float4*>(y + row0)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
  if (with_sum) {
    const float s = warp_sum(yv.x + yv.y + yv.z + yv.w);
    if (lane == 0) wsum[wid * ld + ncols] = s;
  }
  for (uint32_t c0 = 0; c0 < ncols; c0 += kDotCols) {
    float acc[kDotCols];
#pragma unroll
    for (int k = 0; k < kDotCols; ++k) {
      const uint32_t c = c0 + k;
      acc[k] = 0.f;
      if (in && c < ncols) {
        const float4 u = __ldcs(reinterpret_cast<const float4*>(U + c * ldu + row0));
        acc[k] = dot4(u, yv);
      }
    }
#pragma unroll
    for (int k = 0; k < kDotCols; ++k) acc[k] = warp_sum(acc[k]);
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < kDotCols; ++k)
        if (c0 + k < ncols) wsum[wid * ld + c0 + k] = acc[k];
    }
  }
  __syncthreads();
  const uint32_t nout = ncols + (with_sum ? 1u : 0u);
  for (uint32_t c = threadIdx.x; c < nout; c += blockDim.x) {
    float t = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += wsum[w * ld + c];
    part[b * pstride + c] = t;
  }
}

__global__ void __launch_bounds__(256, 8)
k_udots(const float* __restrict__ U, uint64_t ldu, uint32_t ncols,
        const float* __restrict__ y, float* __restrict__ part,
        uint32_t pstride, int with_sum, const float* __restrict__ gate) {
  udots_body(U, ldu, ncols, y, part, pstride, with_sum, gate, blockIdx.x);
}

__global__ void __launch_bounds__(256, 8)
k_udots_multi(const __grid_constant__ TaskList<UdotsTask> L) {
  const uint32_t i = task_of(L.first, L.count, blockIdx.x);
  const UdotsTask& t = L.t[i];
  udots_body(t.U, t.ldu, t.ncols, t.y, t.part, t.pstride, t.with_sum, t.gate,
             blockIdx.x - L.first[i]);
}

// alpha = max(sqrt(sum_b part[b * pstride]), 1e-8) in FP64 (clip_val,
// pca.pyx:1084-1086); B[j, j] = alpha, scal = {alpha, 1 / alpha}; with_centred:
// gate = {sum of column 0, sum of column 1}. One 256-thread block, each
// thread summing blocks tid, tid + 256, ... then a fixed shuffle tree and the
// warps in order. Partials written by other blocks are read through L2.
__device__ void finish_norm_block(const float* part, uint64_t nblocks,
                                  uint32_t pstride, int with_centred,
                                  const NormFinish& fin) {
  __shared__ double dred[2][8];
  double t = 0.0, tc = 0.0;
  for (uint64_t b = threadIdx.x; b < nblocks; b += blockDim.x) {
    t += (double)__ldcg(part + b * pstride);
    if (with_centred) tc += (double)__ldcg(part + b * pstride + 1);
  }
  t = warp_sum(t);
  tc = warp_sum(tc);
  if ((threadIdx.x & 31) == 0) {
    dred[0][threadIdx.x >> 5] = t;
    dred[1][threadIdx.x >> 5] = tc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, sc = 0.0;
    for (int w = 0; w < 8; ++w) {
      s += dred[0][w];
      sc += dred[1][w];
    }
    double a = sqrt(s);
    if (a < 1e-8) a = 1e-8;  // clip_val, pca.pyx:1084-1085
    fin.B[fin.j + (uint64_t)fin.j * fin.m] = a;
    const float af = (float)a;
    fin.scal[0] = af;
    fin.scal[1] = 1.f / af;  // inverse_alpha, pca.pyx:1086
    if (fin.gate) {
      fin.gate[0] = (float)s;
      fin.gate[1] = (float)sc;
    }
    *fin.counter = 0u;  // every block has taken its ticket
  }
}

// b: the block; nblocks: the blocks of the launch (the last to finish
// finishes the norm)
__device__ __forceinline__ void uupdate_body(
    const float* __restrict__ U, uint64_t ldu, uint32_t ncols,
    const float* __restrict__ coef, const float* __restrict__ mean_sum, uint64_t n,
    const float* y_in, float* y_out,  // may be the same
    float* __restrict__ norm_part, uint32_t pstride, int with_centred,
    const float* __restrict__ gate, unsigned long long* __restrict__ taken,
    const NormFinish& fin, uint64_t b, uint32_t nblocks) {
  if (second_pass_skipped(gate)) return;
  if (taken && b == 0 && threadIdx.x == 0) {
    taken[0] += 1ull;
    taken[1] += ncols;
  }
  extern __shared__ float cs[];
  __shared__ float red[2][8];
  for (uint32_t c = threadIdx.x; c < ncols; c += blockDim.x) cs[c] = coef[c];
  __syncthreads();
  const uint64_t row0 = b * kRowBlock + threadIdx.x * 4ull;
  float sq = 0.f, sqc = 0.f;
  if (row0 < ldu) {
    float4 yv = *reinterpret_cast<const float4*>(y_in + row0);
    const float mean = mean_sum ? (*mean_sum) / (float)n : 0.f;  // pca.pyx:1025-1028
    if (with_centred) {  // |y_in - mean|^2 over the block's rows < n
      const float cx = (row0 + 0 < n) ? yv.x - mean : 0.f;
      const float cy = (row0 + 1 < n) ? yv.y - mean : 0.f;
      const float cz = (row0 + 2 < n) ? yv.z - mean : 0.f;
      const float cw = (row0 + 3 < n) ? yv.w - mean : 0.f;
      sqc = sumsq4(cx, cy, cz, cw);
    }
    float4 t = make_float4(mean, mean, mean, mean);
#pragma unroll 4
    for (uint32_t c = 0; c < ncols; ++c) {
      const float4 u = __ldcs(reinterpret_cast<const float4*>(U + c * ldu + row0));
      const float w = cs[c];
      t.x = __fmaf_rn(u.x, w, t.x);
      t.y = __fmaf_rn(u.y, w, t.y);
      t.z = __fmaf_rn(u.z, w, t.z);
      t.w = __fmaf_rn(u.w, w, t.w);
    }
    yv.x = (row0 + 0 < n) ? yv.x - t.x : 0.f;
    yv.y = (row0 + 1 < n) ? yv.y - t.y : 0.f;
    yv.z = (row0 + 2 < n) ? yv.z - t.z : 0.f;
    yv.w = (row0 + 3 < n) ? yv.w - t.w : 0.f;
    *reinterpret_cast<float4*>(y_out + row0) = yv;
    sq = sumsq4(yv.x, yv.y, yv.z, yv.w);
  }
  if (norm_part) {
    sq = warp_sum(sq);
    if (with_centred) sqc = warp_sum(sqc);
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = sq;
      red[1][threadIdx.x >> 5] = sqc;
    }
    __syncthreads();
    if (threadIdx.x < (with_centred ? 2u : 1u)) {
      float t = 0.f;
      for (int w = 0; w < 8; ++w) t += red[threadIdx.x][w];
      norm_part[b * pstride + threadIdx.x] = t;
    }
    if (fin.B) {
      // The block that finishes last (one atomic ticket per block, no
      // waiting) sums every block's partials, in block order whichever
      // block it is.
      __shared__ bool last;
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) last = atomicAdd(fin.counter, 1u) == nblocks - 1;
      __syncthreads();
      if (!last) return;
      __threadfence();
      finish_norm_block(norm_part, nblocks, pstride, with_centred, fin);
    }
  }
}

__global__ void __launch_bounds__(256, 8)  // one wave, as k_udots
k_uupdate(const float* __restrict__ U, uint64_t ldu, uint32_t ncols,
          const float* __restrict__ coef, const float* __restrict__ mean_sum,
          uint64_t n, const float* y_in, float* y_out,  // may be the same
          float* __restrict__ norm_part, uint32_t pstride, int with_centred,
          const float* __restrict__ gate, unsigned long long* __restrict__ taken,
          NormFinish fin) {
  uupdate_body(U, ldu, ncols, coef, mean_sum, n, y_in, y_out, norm_part, pstride,
               with_centred, gate, taken, fin, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(256, 8)
k_uupdate_multi(const __grid_constant__ TaskList<UupdateTask> L) {
  const uint32_t i = task_of(L.first, L.count, blockIdx.x);
  const UupdateTask& t = L.t[i];
  uupdate_body(t.U, t.ldu, t.ncols, t.coef, t.mean_sum, t.n, t.y_in, t.y_out,
               t.norm_part, t.pstride, t.with_centred, t.gate, t.taken, t.fin,
               blockIdx.x - L.first[i], L.first[i + 1] - L.first[i]);
}

// CGS2 middle pass, fused: for one 256-row block, y1 = y0 - (mean + U c1)
// (as k_uupdate) and the block's partial dots of the second pass,
// part[b * pstride + c] = sum_r U[r, c] * y1[r], from one shared-memory copy
// of the block's U tile (U is read once for both).
constexpr int kFuseRows = 256;

__global__ void __launch_bounds__(kFuseRows)
k_uupdate_dots(const float* __restrict__ U, uint64_t ldu, uint32_t ncols,
               const float* __restrict__ coef, const float* __restrict__ mean_sum,
               uint64_t n, const float* __restrict__ y_in, float* __restrict__ y_out,
               float* __restrict__ part, uint32_t pstride) {
  extern __shared__ __align__(16) float fsm[];
  float* us = fsm;                              // ncols x kFuseRows
  float* cs = us + (size_t)ncols * kFuseRows;   // ncols
  float* ys = cs + ((ncols + 3) & ~3u);         // kFuseRows
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint64_t b = blockIdx.x;
  const uint64_t row0 = b * kFuseRows;
  for (uint32_t c = tid; c < ncols; c += kFuseRows) cs[c] = coef[c];
  // tile: columns of 256 rows by asynchronous 16-byte global -> shared copies
  // (cp.async: every copy of the tile is in flight at once, no register
  // staging); rows past ldu are zero-filled
  const uint32_t q4 = kFuseRows / 4;
  for (uint32_t t = tid; t < ncols * q4; t += kFuseRows) {
    const uint32_t c = t / q4, r4 = (t % q4) * 4;
    float* dst = us + (size_t)c * kFuseRows + r4;
    if (row0 + r4 < ldu) {
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)),
                   "l"(U + (uint64_t)c * ldu + row0 + r4)
                   : "memory");
    } else {
      *reinterpret_cast<float4*>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  const uint64_t r = row0 + tid;
  const float mean = mean_sum ? (*mean_sum) / (float)n : 0.f;  // pca.pyx:1025-1028
  float y1 = 0.f;
  if (r < n) {
    float t = mean;
    for (uint32_t c = 0; c < ncols; ++c) t += us[(size_t)c * kFuseRows + tid] * cs[c];
    y1 = y_in[r] - t;
  }
  if (r < ldu) y_out[r] = y1;
  ys[tid] = y1;
  __syncthreads();
  for (uint32_t c = wid; c < ncols; c += kFuseRows / 32) {
    const float* uc = us + (size_t)c * kFuseRows;
    float d = 0.f;
#pragma unroll
    for (int i = 0; i < kFuseRows / 32; ++i) d += uc[lane + 32 * i] * ys[lane + 32 * i];
    d = warp_sum(d);
    if (lane == 0) part[b * pstride + c] = d;
  }
}

// out[c] = sum over blocks b of part[b * pstride + c]. A CTA owns 32 columns
// (lane = column, so every load is one coalesced 128-byte row run); its 32
// warps take blocks b = w, w + 32, ... and the 32 warp sums are added in warp
// order, a fixed order whatever the timing.
__device__ __forceinline__ void reduce_cols_body(const float* __restrict__ part,
                                                 uint64_t nblocks, uint32_t pstride,
                                                 uint32_t ncols, float* __restrict__ out,
                                                 const float* __restrict__ gate,
                                                 uint32_t b) {
  if (second_pass_skipped(gate)) return;
  __shared__ float ws[32][33];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t c = b * 32 + lane;
  float t = 0.f;
  if (c < ncols) {
    // eight loads in flight, added in block order
    uint64_t b = wid;
    for (; b + 32 * 7 < nblocks; b += 32 * 8) {
      float v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = part[(b + 32 * i) * pstride + c];
#pragma unroll
      for (int i = 0; i < 8; ++i) t += v[i];
    }
    for (; b < nblocks; b += 32) t += part[b * pstride + c];
  }
  ws[wid][lane] = t;
  __syncthreads();
  if (wid == 0 && c < ncols) {
    float r = 0.f;
    for (int w = 0; w < 32; ++w) r += ws[w][lane];
    out[c] = r;
  }
}

__global__ void __launch_bounds__(1024)
k_reduce_cols(const float* __restrict__ part, uint64_t nblocks, uint32_t pstride,
              uint32_t ncols, float* __restrict__ out, const float* __restrict__ gate) {
  reduce_cols_body(part, nblocks, pstride, ncols, out, gate, blockIdx.x);
}

__global__ void __launch_bounds__(1024)
k_reduce_cols_multi(const __grid_constant__ TaskList<ReduceColsTask> L) {
  const uint32_t i = task_of(L.first, L.count, blockIdx.x);
  const ReduceColsTask& t = L.t[i];
  reduce_cols_body(t.part, t.nblocks, t.pstride, t.ncols, t.out, t.gate,
                   blockIdx.x - L.first[i]);
}

__global__ void __launch_bounds__(1024)
k_vstep(const float* __restrict__ zin, float* __restrict__ V, uint64_t ldv,
        uint32_t g, uint32_t j, uint32_t m, const float* __restrict__ scal,
        double* __restrict__ B, float* __restrict__ rem, int passes) {
  extern __shared__ float dots[];  // m floats
  __shared__ double red[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const float alpha = scal[0];
  float* z = (j + 1 < m) ? V + (uint64_t)(j + 1) * ldv : rem;
  const float* vj = V + (uint64_t)j * ldv;
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x)
    z[c] = zin[c] - alpha * vj[c];  // pca.pyx:1104-1105
  __syncthreads();
  for (int pass = 0; pass < passes; ++pass) {
    for (uint32_t col = wid; col <= j; col += 32) {
      const float* vc = V + (uint64_t)col * ldv;
      float d = 0.f;
      for (uint32_t c = lane; c < g; c += 32) d += vc[c] * z[c];
      d = warp_sum(d);
      if (lane == 0) dots[col] = d;
    }
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) {
      float t = 0.f;
      for (uint32_t col = 0; col <= j; ++col) t += V[c + (uint64_t)col * ldv] * dots[col];
      z[c] -= t;
    }
    __syncthreads();
  }
  if (j + 1 < m) {
    double ss = 0.0;
    for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) ss += (double)z[c] * z[c];
    ss = warp_sum(ss);
    if (lane == 0) red[wid] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < 32; ++w) s += red[w];
      double beta = sqrt(s);
      if (beta < 1e-8) beta = 1e-8;  // pca.pyx:1165-1166
      B[j + (uint64_t)(j + 1) * m] = beta;
      red[0] = beta;
    }
    __syncthreads();
    const float inv = 1.f / (float)red[0];
    for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) z[c] *= inv;
  }
}

// V-side step on one 8-CTA thread-block cluster: CTA q owns genes
// [q*slice, (q+1)*slice) and keeps its part of z in shared memory; the
// Gram-Schmidt dots and the norm are all-reduced through distributed shared
// memory, every CTA summing the 8 partials in rank order (so all CTAs hold
// the same bits and the result does not depend on timing).
constexpr int kVCluster = 8;
static_assert(kVCluster == (int)kVStepCtas, "one V-step task is one cluster");
constexpr int kVThreads = 1024;
constexpr int kVSplit = 4;  // threads sharing one gene's update sum

__device__ __forceinline__ void vstep_cluster_body(
    const float* __restrict__ zin, float* __restrict__ V, uint64_t ldv, uint32_t g,
    uint32_t j, uint32_t m, const float* __restrict__ scal, double* __restrict__ B,
    float* __restrict__ rem, int passes) {
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) float vsm[];
  const uint32_t slice = (g + kVCluster - 1) / kVCluster;
  // passes == 0: adaptive, a second pass only where the first kept less than
  // half of the squared norm of z - alpha v_j (all CTAs take one decision)
  const bool adaptive = passes == 0;
  const int npass = adaptive ? 2 : passes;
  float* zs = vsm;                            // slice
  float* pd = zs + ((slice + 3) & ~3u);       // 2 x (m + 1) partials (per pass)
  float* dots = pd + 2 * (m + 1);             // m + 1
  float* upd = dots + ((m + 4) & ~3u);        // kVSplit x slice partial updates
  __shared__ double pn;                       // partial squared norm
  __shared__ double wred[kVThreads / 32];
  __shared__ float wz[kVThreads / 32];
  __shared__ float pz1;                       // partial |z after pass 0|^2
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t q = cluster.block_rank();
  const uint32_t c0 = q * slice, c1 = min(g, c0 + slice);
  const float alpha = scal[0];
  const float* vj = V + (uint64_t)j * ldv;
  for (uint32_t c = c0 + threadIdx.x; c < c1; c += kVThreads)
    zs[c - c0] = __fmaf_rn(-alpha, vj[c], zin[c]);  // pca.pyx:1104-1105
  __syncthreads();
  for (int pass = 0; pass < npass; ++pass) {
    float* pdp = pd + (pass & 1) * (m + 1);
    // adaptive: pass 0 also sums |z|^2 as column j + 1
    const uint32_t ncol = j + 1 + (adaptive && pass == 0 ? 1u : 0u);
    for (uint32_t col = wid; col < ncol; col += kVThreads / 32) {
      float d = 0.f;
      if (col <= j) {
        const float* vc = V + (uint64_t)col * ldv;
        for (uint32_t c = c0 + lane; c < c1; c += 32) d = __fmaf_rn(vc[c], zs[c - c0], d);
      } else {
        for (uint32_t c = c0 + lane; c < c1; c += 32) d = __fmaf_rn(zs[c - c0], zs[c - c0], d);
      }
      d = warp_sum(d);
      if (lane == 0) pdp[col] = d;
    }
    cluster.sync();  // every CTA's partials are visible
    for (uint32_t col = threadIdx.x; col < ncol; col += kVThreads) {
      float t = 0.f;
      for (uint32_t r = 0; r < kVCluster; ++r) t += cluster.map_shared_rank(pdp, r)[col];
      dots[col] = t;
    }
    __syncthreads();
    // each gene's sum over columns split in kVSplit fixed strands (col = h,
    // h + kVSplit, ...), added in strand order
    for (uint32_t t = threadIdx.x; t < kVSplit * slice; t += kVThreads) {
      const uint32_t h = t / slice, c = c0 + t % slice;
      float acc = 0.f;
      if (c < c1)
        for (uint32_t col = h; col <= j; col += kVSplit)
          acc = __fmaf_rn(V[c + (uint64_t)col * ldv], dots[col], acc);
      upd[t] = acc;
    }
    __syncthreads();
    for (uint32_t c = c0 + threadIdx.x; c < c1; c += kVThreads) {
      const uint32_t i = c - c0;
      float t = 0.f;
#pragma unroll
      for (int h = 0; h < kVSplit; ++h) t += upd[h * slice + i];
      zs[i] -= t;
    }
    __syncthreads();
    if (adaptive && pass == 0) {
      float s1 = 0.f;
      for (uint32_t c = c0 + threadIdx.x; c < c1; c += kVThreads)
        s1 = __fmaf_rn(zs[c - c0], zs[c - c0], s1);
      s1 = warp_sum(s1);
      if (lane == 0) wz[wid] = s1;
      __syncthreads();
      if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < kVThreads / 32; ++w) t += wz[w];
        pz1 = t;
      }
      cluster.sync();
      float z1 = 0.f;
      for (uint32_t r = 0; r < kVCluster; ++r) z1 += *cluster.map_shared_rank(&pz1, r);
      if (z1 >= 0.5f * dots[j + 1]) break;  // the same in every CTA
    }
  }
  float* out = (j + 1 < m) ? V + (uint64_t)(j + 1) * ldv : rem;
  if (j + 1 < m) {
    double ss = 0.0;
    for (uint32_t c = c0 + threadIdx.x; c < c1; c += kVThreads)
      ss = __fma_rn((double)zs[c - c0], (double)zs[c - c0], ss);
    ss = warp_sum(ss);
    if (lane == 0) wred[wid] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kVThreads / 32; ++w) t += wred[w];
      pn = t;
    }
    cluster.sync();
    double s2 = 0.0;
    for (uint32_t r = 0; r < kVCluster; ++r) s2 += *cluster.map_shared_rank(&pn, r);
    double beta = sqrt(s2);
    if (beta < 1e-8) beta = 1e-8;  // pca.pyx:1165-1166
    if (q == 0 && threadIdx.x == 0) B[j + (uint64_t)(j + 1) * m] = beta;
    const float inv = 1.f / (float)beta;
    for (uint32_t c = c0 + threadIdx.x; c < c1; c += kVThreads) out[c] = zs[c - c0] * inv;
  } else {
    for (uint32_t c = c0 + threadIdx.x; c < c1; c += kVThreads) out[c] = zs[c - c0];
  }
  cluster.sync();  // no CTA leaves while another may read its shared memory
}

__global__ void __cluster_dims__(kVCluster, 1, 1) __launch_bounds__(kVThreads)
k_vstep_cluster(const float* __restrict__ zin, float* __restrict__ V, uint64_t ldv,
                uint32_t g, uint32_t j, uint32_t m, const float* __restrict__ scal,
                double* __restrict__ B, float* __restrict__ rem, int passes) {
  vstep_cluster_body(zin, V, ldv, g, j, m, scal, B, rem, passes);
}

// one cluster per task: CTAs [8 i, 8 i + 8) of the grid
__global__ void __cluster_dims__(kVCluster, 1, 1) __launch_bounds__(kVThreads)
k_vstep_cluster_multi(const __grid_constant__ TaskList<VstepTask> L) {
  const VstepTask& t = L.t[blockIdx.x / kVCluster];
  vstep_cluster_body(t.z, t.V, t.ldv, t.g, t.j, t.m, t.scal, t.B, t.rem, t.passes);
}

// Tall-skinny SIMT GEMM: CTA tile 128 rows x 128 columns, K in steps of 16.
constexpr int BM = 128, BN = 128, BK = 16;

__global__ void __launch_bounds__(256)
k_gemm_ts(const float* __restrict__ A, uint64_t lda, uint64_t rows, uint32_t K,
          const float* __restrict__ Bp, uint64_t bsr, uint64_t bsc,
          const float* __restrict__ cs, uint32_t ncols, float* __restrict__ C,
          uint64_t ldc, int c_rowmajor) {
  __shared__ __align__(16) float As[BK][BM];
  __shared__ __align__(16) float Bs[BK][BN];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  const uint64_t r0 = (uint64_t)blockIdx.x * BM;
  const uint32_t c0 = blockIdx.y * BN;
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) acc[i][jj] = 0.f;

  for (uint32_t k0 = 0; k0 < K; k0 += BK) {
    // A tile: 16 columns x 128 rows; thread loads 8 floats (2 x float4)
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int idx = tid + t * 256;       // 0..511 float4 slots
      const int kk = idx >> 5;             // 0..15
      const int rr = (idx & 31) * 4;       // 0..124
      const uint64_t r = r0 + rr;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k0 + kk < K) {
        const float* src = A + (uint64_t)(k0 + kk) * lda + r;
        if (r + 3 < rows) {
          v = *reinterpret_cast<const float4*>(src);
        } else {
          if (r + 0 < rows) v.x = src[0];
          if (r + 1 < rows) v.y = src[1];
          if (r + 2 < rows) v.z = src[2];
        }
      }
      *reinterpret_cast<float4*>(&As[kk][rr]) = v;
    }
    // B tile: 16 x 128, strided gather (small operand, L2-resident)
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int idx = tid + t * 256;  // 0..2047
      const int kk = idx >> 7;
      const int cc = idx & 127;
      float v = 0.f;
      if (k0 + kk < K && c0 + cc < ncols) {
        v = Bp[(uint64_t)(k0 + kk) * bsr + (uint64_t)(c0 + cc) * bsc];
        if (cs) v *= cs[c0 + cc];
      }
      Bs[kk][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[kk][64 + tx * 4]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int jj = 0; jj < 8; ++jj) acc[i][jj] += a[i] * bb[jj];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint64_t r = r0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
    if (r >= rows) continue;
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const uint32_t c = c0 + (jj < 4 ? tx * 4 + jj : 64 + tx * 4 + (jj - 4));
      if (c >= ncols) continue;
      if (c_rowmajor)
        C[r * ldc + c] = acc[i][jj];
      else
        C[r + (uint64_t)c * ldc] = acc[i][jj];
    }
  }
}

__global__ void k_b_to_float(const double* __restrict__ B, uint64_t count,
                             float* __restrict__ Bf) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < count) Bf[i] = (float)B[i];
}

}  // namespace

int launch_udots(const float* U, uint64_t ldu, uint32_t ncols, const float* y,
                 uint64_t nblocks, float* part, uint32_t pstride, bool with_sum,
                 cudaStream_t s, const float* gate) {
  const size_t smem = 8ull * (ncols + 1) * sizeof(float);
  BGPU_REQUIRE(smem <= 227 * 1024, BGPU_ERR_UNSUPPORTED, "U dots: too many columns");
  if (smem > 48 * 1024) BGPU_CUDA(allow_max_smem(k_udots));
  k_udots<<<(unsigned)nblocks, 256, smem, s>>>(U, ldu, ncols, y, part, pstride,
                                               with_sum ? 1 : 0, gate);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_uupdate(const float* U, uint64_t ldu, uint32_t ncols,
                   const float* coef, const float* mean_sum, uint64_t n,
                   const float* y_in, float* y_out, uint64_t nblocks,
                   float* norm_part, uint32_t pstride, cudaStream_t s,
                   bool with_centred, const float* gate,
                   unsigned long long* taken, NormFinish fin) {
  BGPU_REQUIRE(!fin.B || (norm_part && fin.counter && fin.scal), BGPU_ERR_INVALID,
               "U update: norm finish needs partials, a ticket counter and scal");
  k_uupdate<<<(unsigned)nblocks, 256, std::max<size_t>(ncols, 1) * 4, s>>>(
      U, ldu, ncols, coef, mean_sum, n, y_in, y_out, norm_part, pstride,
      with_centred ? 1 : 0, gate, taken, fin);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

size_t uupdate_dots_smem(uint32_t ncols) {
  return ((size_t)ncols * kFuseRows + ((ncols + 3) & ~3u) + kFuseRows) * sizeof(float);
}

uint64_t uupdate_dots_blocks(uint64_t n) { return ceil_div(n, kFuseRows); }

int launch_uupdate_dots(const float* U, uint64_t ldu, uint32_t ncols,
                        const float* coef, const float* mean_sum, uint64_t n,
                        const float* y_in, float* y_out, float* part,
                        uint32_t pstride, cudaStream_t s) {
  const size_t smem = uupdate_dots_smem(ncols);
  BGPU_REQUIRE(smem <= 227 * 1024, BGPU_ERR_UNSUPPORTED, "fused U pass tile too large");
  if (smem > 48 * 1024)
    BGPU_CUDA(allow_max_smem(k_uupdate_dots));
  k_uupdate_dots<<<(unsigned)uupdate_dots_blocks(n), kFuseRows, smem, s>>>(
      U, ldu, ncols, coef, mean_sum, n, y_in, y_out, part, pstride);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_reduce_cols(const float* part, uint64_t nblocks, uint32_t pstride,
                       uint32_t ncols, float* out, cudaStream_t s,
                       const float* gate) {
  if (ncols == 0) return BGPU_OK;
  k_reduce_cols<<<(unsigned)ceil_div(ncols, 32), 1024, 0, s>>>(part, nblocks,
                                                               pstride, ncols, out,
                                                               gate);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

static size_t vstep_cluster_smem(uint32_t g, uint32_t m) {
  const uint32_t slice = (g + kVCluster - 1) / kVCluster;
  return ((size_t)((slice + 3) & ~3u) + 2ull * (m + 1) + ((m + 4) & ~3u) +
          (size_t)kVSplit * slice) * sizeof(float);
}

bool vstep_cluster_fits(uint32_t g, uint32_t m) {
  return vstep_cluster_smem(g, m) <= 48 * 1024;
}

int launch_vstep(const float* z, float* V, uint64_t ldv, uint32_t g,
                 uint32_t j, uint32_t m, const float* scal, double* B,
                 float* rem, int passes, cudaStream_t s) {
  const size_t csm = vstep_cluster_smem(g, m);
  if (csm <= 48 * 1024) {
    k_vstep_cluster<<<kVCluster, kVThreads, csm, s>>>(z, V, ldv, g, j, m, scal, B,
                                                     rem, passes);
  } else {
    k_vstep<<<1, 1024, (size_t)m * sizeof(float), s>>>(  // adaptive: 2 passes
        z, V, ldv, g, j, m, scal, B, rem, passes == 0 ? 2 : passes);
  }
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_udots_multi(const TaskList<UdotsTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  uint32_t nc = 0;
  for (uint32_t i = 0; i < L.count; ++i) nc = std::max(nc, L.t[i].ncols);
  const size_t smem = 8ull * (nc + 1) * sizeof(float);
  BGPU_REQUIRE(smem <= 227 * 1024, BGPU_ERR_UNSUPPORTED, "U dots: too many columns");
  if (smem > 48 * 1024) BGPU_CUDA(allow_max_smem(k_udots_multi));
  k_udots_multi<<<L.grid(), 256, smem, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_reduce_cols_multi(const TaskList<ReduceColsTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  k_reduce_cols_multi<<<L.grid(), 1024, 0, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_uupdate_multi(const TaskList<UupdateTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  uint32_t nc = 1;
  for (uint32_t i = 0; i < L.count; ++i) {
    const UupdateTask& t = L.t[i];
    BGPU_REQUIRE(!t.fin.B || (t.norm_part && t.fin.counter && t.fin.scal), BGPU_ERR_INVALID,
                 "U update: norm finish needs partials, a ticket counter and scal");
    nc = std::max(nc, t.ncols);
  }
  k_uupdate_multi<<<L.grid(), 256, (size_t)nc * 4, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_vstep_multi(const TaskList<VstepTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  size_t csm = 0;
  for (uint32_t i = 0; i < L.count; ++i) {
    BGPU_REQUIRE(L.first[i + 1] - L.first[i] == kVStepCtas &&
                     vstep_cluster_fits(L.t[i].g, L.t[i].m),
                 BGPU_ERR_INVALID, "V step: a task is one cluster of kVStepCtas CTAs");
    csm = std::max(csm, vstep_cluster_smem(L.t[i].g, L.t[i].m));
  }
  k_vstep_cluster_multi<<<L.grid(), kVThreads, csm, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_gemm_ts(const float* A, uint64_t lda, uint64_t rows, uint32_t K,
                   const float* Bp, uint64_t bsr, uint64_t bsc, const float* cs,
                   uint32_t ncols, float* C, uint64_t ldc, bool c_rowmajor,
                   cudaStream_t s) {
  if (rows == 0 || ncols == 0) return BGPU_OK;
  dim3 grid((unsigned)ceil_div(rows, BM), (unsigned)ceil_div(ncols, BN));
  k_gemm_ts<<<grid, 256, 0, s>>>(A, lda, rows, K, Bp, bsr, bsc, cs, ncols, C,
                                 ldc, c_rowmajor ? 1 : 0);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_b_to_float(const double* B, uint32_t m, float* Bf, cudaStream_t s) {
  uint64_t count = (uint64_t)m * (m + 1);
  k_b_to_float<<<(unsigned)ceil_div(count, 256), 256, 0, s>>>(B, count, Bf);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
