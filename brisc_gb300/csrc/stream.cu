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
#include <climits>
#include <cstdlib>
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
                                             const float* __restrict__ w, uint32_t gm,
                                             int lane8) {
  float acc = 0.f;
  for (int64_t b = (e0 & ~3ll) + 4 * lane8; b - 4 * lane8 < e1; b += 32) {
    const uint4 r4 = b < e1 ? ld_stream_u4(packed + b) : make_uint4(0, 0, 0, 0);
    const uint32_t vm = window_mask(b, e0, e1);
    const uint32_t qq[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t cnt = qq[j] & 0xffffu;
      const float val = cnt < (uint32_t)kCountTab ? tb[cnt] : norm_count(cnt, isf);
      if (vm & (1u << j)) acc += val * w[(qq[j] >> 16) & gm];
    }
  }
  return acc;
}

// ---------------------------------------------------------------------------
// X.v, counts layout: 8 lanes per cell row.
constexpr int kTabSlot = 17;  // padded per-group table slot (conflict-free)

constexpr int kSpmvRowsCtas = 5;  // resident CTAs per SM (48 registers)

__global__ void __launch_bounds__(256, kSpmvRowsCtas)
k_spmv_rows(CsrView X, const int32_t* __restrict__ order, const float* __restrict__ v,
            const float* __restrict__ sd, float* __restrict__ y) {
  extern __shared__ __align__(16) float sm[];
  float* w = sm;                                       // g floats
  float* tabs = sm + ((X.g + 3) & ~3u);                // 32 groups x 2 x kTabSlot
  for (uint32_t c = threadIdx.x; c < X.g; c += blockDim.x)
    w[c] = sd ? v[c] / sd[c] : v[c];  // pca.pyx:461-462
  __syncthreads();

  const int lane8 = threadIdx.x & 7;
  const unsigned gmask = 0xFFu << (threadIdx.x & 24);
  const uint32_t gslot = (threadIdx.x >> 3) * 2 * kTabSlot;
  // bit 31 of a stored word flags a row head when genes fit in 15 bits
  const uint32_t gm = X.g > 32768u ? 0xffffu : 0x7fffu;
  const uint64_t gid = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 3;
  const uint64_t ngroups = (gridDim.x * (uint64_t)blockDim.x) >> 3;
  const float2* rt2 = reinterpret_cast<const float2*>(X.rtab);

  // Rows are taken in `order` (longest first, by 32-entry windows), so the
  // four groups of a warp work on rows of about the same length; each row's
  // sum is the same whichever group computes it.
  auto row_at = [&](uint64_t i) -> uint64_t { return order ? (uint64_t)order[i] : i; };
  // offsets and count table of the next row, loaded one row ahead
  int64_t nx0 = 0, nx1 = 0;
  float2 nt2 = make_float2(0.f, 0.f);
  uint64_t nrow = 0;
  if (gid < X.n) {
    nrow = row_at(gid);
    nx0 = X.rowptr[nrow];
    nx1 = X.rowptr[nrow + 1];
    nt2 = rt2[nrow * (kCountTab / 2) + lane8];
  }
  int buf = 0;
  for (uint64_t i = gid; i < X.n; i += ngroups, buf ^= 1) {
    const uint64_t r = nrow;
    const int64_t e0 = nx0, e1 = nx1;
    const float2 t2 = nt2;
    // row-relative 32-bit offsets: the row's words are [lead, len) of the
    // 16-byte-aligned span starting at a0
    const int64_t a0 = e0 & ~3ll;
    const uint32_t* rowp = X.packed + a0;
    const int lead = (int)(e0 - a0), len = (int)(e1 - a0);
    // the row's first 128 words: four 16-byte loads per lane in flight
    const int o = 4 * lane8;
    const uint4 z4 = make_uint4(0, 0, 0, 0);
    const uint4 q0 = o < len ? ld_stream_u4(rowp + o) : z4;
    const uint4 q1 = o + 32 < len ? ld_stream_u4(rowp + o + 32) : z4;
    const uint4 q2 = o + 64 < len ? ld_stream_u4(rowp + o + 64) : z4;
    const uint4 q3 = o + 96 < len ? ld_stream_u4(rowp + o + 96) : z4;
    if (i + ngroups < X.n) {
      nrow = row_at(i + ngroups);
      nx0 = X.rowptr[nrow];
      nx1 = X.rowptr[nrow + 1];
      nt2 = rt2[nrow * (kCountTab / 2) + lane8];
    }
    // the row's count table into this group's (double-buffered) slot
    float* tb = tabs + gslot + buf * kTabSlot;
    tb[2 * lane8] = t2.x;
    tb[2 * lane8 + 1] = t2.y;
    __syncwarp(gmask);
    float acc = 0.f;
    uint32_t big = 0;  // OR of the loaded words: a count >= 16 shows in 0xfff0
    auto consume = [&](uint4 q, int at) {
      if (at < lead || at + 4 > len) q = clip_window(q, lead - at, len - at);
      big |= q.x | q.y | q.z | q.w;
      acc = fmaf(tb[q.x & (kCountTab - 1)], w[(q.x >> 16) & gm], acc);
      acc = fmaf(tb[q.y & (kCountTab - 1)], w[(q.y >> 16) & gm], acc);
      acc = fmaf(tb[q.z & (kCountTab - 1)], w[(q.z >> 16) & gm], acc);
      acc = fmaf(tb[q.w & (kCountTab - 1)], w[(q.w >> 16) & gm], acc);
    };
    if (o < len) consume(q0, o);
    if (o + 32 < len) consume(q1, o + 32);
    if (o + 64 < len) consume(q2, o + 64);
    if (o + 96 < len) consume(q3, o + 96);
    for (int ob = 128; ob < len; ob += 64) {  // rows longer than 128 words
      const int oo = ob + o;
      const uint4 p0 = oo < len ? ld_stream_u4(rowp + oo) : z4;
      const uint4 p1 = oo + 32 < len ? ld_stream_u4(rowp + oo + 32) : z4;
      if (oo < len) consume(p0, oo);
      if (oo + 32 < len) consume(p1, oo + 32);
    }
    if (__any_sync(gmask, (big & 0xfff0u) != 0u))
      acc = csr_row_exact8(X.packed, e0, e1, tb, X.isf[r], w, gm, lane8);
#pragma unroll
    for (int s2 = 4; s2 > 0; s2 >>= 1) acc += __shfl_xor_sync(gmask, acc, s2);
    if (lane8 == 0) y[r] = X.post ? acc * X.post[r] : acc;
  }
}

// ---------------------------------------------------------------------------
// X^T.u, counts layout: one CTA per row panel, the panel's words as one flat
// stream. The first word of every (panel, gene) segment carries a head flag
// (bit 31); warps take contiguous runs of whole segments, lanes take 8
// consecutive words, and a warp-segmented scan closes each segment where the
// next head starts. No lane idles on short segments.
constexpr uint32_t kHeadBit = 0x80000000u;
constexpr int kSegThreads = 512;
constexpr int kMaxPanelRows = 2048;  // rows per panel the staged table allows
constexpr int kSegWarps = kSegThreads / 32;

constexpr int kRmatThreads = 384;
constexpr int kRmatWarps = kRmatThreads / 32;
constexpr int kStageLd = 33;  // per-warp [position][lane] staging, padded

// Bytes of one block's staged running sums: 7 positions x 32 lanes per warp.
__host__ __device__ constexpr uint32_t stage_bytes(int warps) {
  return (uint32_t)warps * 7u * kStageLd * 4u;
}

struct SegLayout {
  uint32_t tab, cps, nz, misc, stage, total;
  __host__ __device__ SegLayout(uint32_t P, uint32_t g) {
    tab = 128;                             // mbarrier
    cps = tab + r128(P * kCountTab * 4);   // table scaled by u: [count][row]
    nz = cps + r128((g + 1) * 4);          // gene offsets, then per-gene sums
    misc = nz + r128(g * 2);               // non-empty genes in order (u16)
    stage = misc + 128;                    // warp totals (above), then the
    total = stage + r128(stage_bytes(kRmatWarps));  // lanes' running sums
  }
};

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// u * scale (* post) of panel row r, as the product kernels stage it.
__device__ __forceinline__ float scaled_u(const CscView& X, const float* u,
                                          const float* u_scale, float scale,
                                          uint64_t r) {
  const float uu = u_scale ? u[r] * scale : u[r];
  return X.post ? uu * X.post[r] : uu;
}

__global__ void __launch_bounds__(kRmatThreads, 2)
k_rmat_seg(CscView X, const float* __restrict__ u, const float* __restrict__ u_scale,
           float* __restrict__ u_out, float* __restrict__ partT,
           int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t P = 1u << X.pshift;
  const SegLayout L(P, X.g);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  float* ut = reinterpret_cast<float*>(smem + L.tab);      // [count][row]
  int32_t* cps = reinterpret_cast<int32_t*>(smem + L.cps);
  float* gsum = reinterpret_cast<float*>(smem + L.cps);    // after the ranges
  uint16_t* nz = reinterpret_cast<uint16_t*>(smem + L.nz);
  int32_t* wtot = reinterpret_cast<int32_t*>(smem + L.misc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

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
  float usr[(kMaxPanelRows + kRmatThreads - 1) / kRmatThreads];
#pragma unroll
  for (int k = 0; k < (kMaxPanelRows + kRmatThreads - 1) / kRmatThreads; ++k) {
    const uint32_t i = threadIdx.x + k * kRmatThreads;
    float us = 0.f;
    if (i < rows) {
      if (u_out) u_out[r0 + i] = u_scale ? u[r0 + i] * scale : u[r0 + i];
      us = scaled_u(X, u, u_scale, scale, r0 + i);
    }
    usr[k] = us;
  }
  const int32_t* cp = X.colptr + (uint64_t)p * (X.g + 1);
  for (uint32_t c = threadIdx.x; c <= X.g; c += kRmatThreads) cps[c] = cp[c];
  __syncthreads();

  // Non-empty genes of the panel, in gene order.
  uint32_t S = 0;
  for (uint32_t base = 0; base < X.g; base += kRmatThreads) {
    const uint32_t c = base + threadIdx.x;
    const bool f = c < X.g && cps[c + 1] > cps[c];
    const uint32_t bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wtot[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, tot = 0;
#pragma unroll
    for (int j = 0; j < kRmatWarps; ++j) {
      const uint32_t t = (uint32_t)wtot[j];
      before += j < wid ? t : 0u;
      tot += t;
    }
    if (f) nz[S + before + __popc(bal & lanemask_lt())] = (uint16_t)c;
    S += tot;
    __syncthreads();
  }
  const uint32_t W = (uint32_t)cps[X.g];

  // The table arrives; scale it by u in place (count 0 stays 0).
  const bool ok = __syncthreads_and(mbar_wait(&bar[0], 0, err));
  if (!ok) return;  // every thread waited (bounded) for the copy
#pragma unroll
  for (int k = 0; k < (kMaxPanelRows + kRmatThreads - 1) / kRmatThreads; ++k) {
    const uint32_t i = threadIdx.x + k * kRmatThreads;
    if (i < P)
#pragma unroll
      for (int c = 1; c < kCountTab; ++c) ut[c * P + i] *= usr[k];
  }

  // This warp's run of segments: ordinals [i0, i1), words [s0, s1).
  auto first_at = [&](uint64_t t) {  // first ordinal whose segment starts >= t
    uint32_t lo = 0, hi = S;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if ((uint64_t)cps[nz[mid]] < t) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  const uint32_t i0 = first_at((uint64_t)W * wid / kRmatWarps);
  const uint32_t i1 = wid == kRmatWarps - 1 ? S : first_at((uint64_t)W * (wid + 1) / kRmatWarps);
  const uint32_t s0 = i0 < S ? (uint32_t)cps[nz[i0]] : W;
  const uint32_t s1 = i1 < S ? (uint32_t)cps[nz[i1]] : W;
  __syncthreads();  // cps is no longer read: its space holds the gene sums
  for (uint32_t c = threadIdx.x; c < X.g; c += kRmatThreads) gsum[c] = 0.f;
  __syncthreads();

  const int64_t pbase = X.rowptr[r0];
  const int64_t beg = pbase + s0, end = pbase + s1;
  const uint32_t pshift = X.pshift, lrmask = P - 1;
  const uint32_t lt = lanemask_lt();
  float* stg = reinterpret_cast<float*>(smem + L.stage) + wid * 7 * kStageLd + lane;
  float carry = 0.f;  // open segment's sum entering the next iteration
  uint32_t kb = 0;    // heads seen in earlier iterations
  // software-pipelined: the next iteration's 32 bytes per lane are in flight
  // while this iteration's words are summed
  const uint4 z4 = make_uint4(0, 0, 0, 0);
  uint4 qa = z4, qb = z4;
  {
    const int64_t wb0 = (beg & ~7ll) + 8 * lane;
    if (wb0 < end) {
      qa = ld_stream_u4(X.packed + wb0);
      qb = ld_stream_u4(X.packed + wb0 + 4);
    }
  }
  for (int64_t b = beg & ~7ll; b < end; b += 256) {
    const int64_t wb = b + 8 * lane;
    uint4 na = z4, nb = z4;
    if (wb + 256 < end) {
      na = ld_stream_u4(X.packed + wb + 256);
      nb = ld_stream_u4(X.packed + wb + 260);
    }
    uint32_t wd[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
    qa = na;
    qb = nb;
    if (wb < beg || wb + 8 > end) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (wb + i < beg || wb + i >= end) wd[i] = 0u;
    }
    float v[8];
    uint32_t big = 0, hm = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      big |= wd[i];
      hm |= (wd[i] >> 31) << i;
      v[i] = ut[((wd[i] & (kCountTab - 1)) << pshift) | ((wd[i] >> 16) & lrmask)];
    }
    if (__any_sync(0xffffffffu, (big & 0xfff0u) != 0u)) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const uint32_t cnt = wd[i] & 0xffffu;
        if (cnt >= (uint32_t)kCountTab) {
          const uint64_t r = r0 + ((wd[i] >> 16) & lrmask);
          v[i] = norm_count(cnt, X.isf[r]) * scaled_u(X, u, u_scale, scale, r);
        }
      }
    }
    // in-lane segmented sums: s[i] = sum since the last head at or before i
    float sl[8];
    sl[0] = v[0];
#pragma unroll
    for (int i = 1; i < 8; ++i) sl[i] = ((hm >> i) & 1u) ? v[i] : sl[i - 1] + v[i];
    const uint32_t F = __ballot_sync(0xffffffffu, hm != 0u);
    // cross-lane inclusive segmented scan of the lane tails
    float T = sl[7];
    uint32_t fa = hm != 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float Tp = __shfl_up_sync(0xffffffffu, T, d);
      const uint32_t fp = __shfl_up_sync(0xffffffffu, fa, d);
      if (lane >= d) {
        if (!fa) T = Tp + T;
        fa |= fp;
      }
    }
    if ((F & (lt | (1u << lane))) == 0u) T = carry + T;  // no head up to here
    float cin = __shfl_up_sync(0xffffffffu, T, 1);
    if (lane == 0) cin = carry;  // open sum entering this lane
    // heads in earlier lanes of this iteration
    const uint32_t h = __popc(hm);
    uint32_t hs = h;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, hs, d);
      if (lane >= d) hs += t;
    }
    const uint32_t kl = kb + hs - h;  // heads before this lane
    // a head closes the segment before it (the run's first head closes
    // nothing); each lane walks only its own heads, reading the running sum
    // before the head from its staging column
#pragma unroll
    for (int i = 0; i < 7; ++i) stg[i * kStageLd] = sl[i];
    for (uint32_t rem = hm; rem != 0u; rem &= rem - 1u) {
      const int i = __ffs(rem) - 1;
      const uint32_t pre = hm & ((1u << i) - 1u);
      const uint32_t k = kl + __popc(pre);
      if (k > 0) {
        float val = cin;
        if (i > 0) {
          const float sv = stg[(i - 1) * kStageLd];
          val = pre ? sv : cin + sv;
        }
        gsum[nz[i0 + k - 1]] = val;
      }
    }
    carry = __shfl_sync(0xffffffffu, T, 31);
    kb += __shfl_sync(0xffffffffu, hs, 31);
  }
  if (lane == 0 && kb > 0) gsum[nz[i0 + kb - 1]] = carry;
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < X.g; c += kRmatThreads)
    partT[(uint64_t)c * X.num_panels + p] = gsum[c];
}

// ---------------------------------------------------------------------------
// X.v, counts layout with row heads (genes < 32768): one CTA per row panel,
// the panel's CSR words as one flat stream, the same warp-segmented scan as
// X^T.u with rows as the segments. The panel's count table ([count][row],
// shared with X^T.u) arrives by bulk copy; each lane tracks the row of its
// words from the head flags.
struct RowSegLayout {
  uint32_t tab, w, rofs, nzr, rsum, misc, stage, total;
  __host__ __device__ RowSegLayout(uint32_t P, uint32_t g) {
    tab = 128;                             // mbarrier
    w = tab + r128(P * kCountTab * 4);     // count table [count][row]
    rofs = w + r128(g * 4);                // v / sd
    nzr = rofs + r128((P + 1) * 4);        // row offsets in the panel
    rsum = nzr + r128(P * 2);              // non-empty rows in order (u16)
    misc = rsum + r128(P * 4);             // per-row sums
    stage = misc + 128;                    // warp totals (above), then the
    total = stage + r128(stage_bytes(kSegWarps));  // lanes' running sums
  }
};

__global__ void __launch_bounds__(kSegThreads, 2)
k_spmv_seg(CsrView X, uint32_t pshift, const float* __restrict__ rtab_c,
           const float* __restrict__ v, const float* __restrict__ sd,
           float* __restrict__ y, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t P = 1u << pshift;
  const RowSegLayout L(P, X.g);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  const float* tab = reinterpret_cast<const float*>(smem + L.tab);
  float* wv = reinterpret_cast<float*>(smem + L.w);
  int32_t* rofs = reinterpret_cast<int32_t*>(smem + L.rofs);
  uint16_t* nzr = reinterpret_cast<uint16_t*>(smem + L.nzr);
  float* rsum = reinterpret_cast<float*>(smem + L.rsum);
  int32_t* wtot = reinterpret_cast<int32_t*>(smem + L.misc);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;

  const uint32_t p = blockIdx.x;
  const uint64_t r0 = (uint64_t)p << pshift;
  const uint32_t rows = (uint32_t)min_u64(P, X.n - r0);
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    fence_mbar_init();
    const uint32_t tb = P * kCountTab * 4;
    mbar_arrive_expect_tx(&bar[0], tb);
    bulk_g2s(smem + L.tab, rtab_c + (uint64_t)p * kCountTab * P, tb, &bar[0]);
  }
  for (uint32_t c = threadIdx.x; c < X.g; c += kSegThreads)
    wv[c] = sd ? v[c] / sd[c] : v[c];  // pca.pyx:461-462
  const int64_t pbase = X.rowptr[r0];
  for (uint32_t i = threadIdx.x; i <= P; i += kSegThreads)
    rofs[i] = (int32_t)(X.rowptr[r0 + min(i, rows)] - pbase);
  for (uint32_t i = threadIdx.x; i < P; i += kSegThreads) rsum[i] = 0.f;
  __syncthreads();

  // Non-empty rows of the panel, in order.
  uint32_t S = 0;
  for (uint32_t base = 0; base < rows; base += kSegThreads) {
    const uint32_t i = base + threadIdx.x;
    const bool f = i < rows && rofs[i + 1] > rofs[i];
    const uint32_t bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wtot[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, tot = 0;
#pragma unroll
    for (int j = 0; j < kSegWarps; ++j) {
      const uint32_t t = (uint32_t)wtot[j];
      before += j < wid ? t : 0u;
      tot += t;
    }
    if (f) nzr[S + before + __popc(bal & lanemask_lt())] = (uint16_t)i;
    S += tot;
    __syncthreads();
  }
  const uint32_t W = (uint32_t)rofs[rows];
  auto first_at = [&](uint64_t t) {  // first ordinal whose row starts >= t
    uint32_t lo = 0, hi = S;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if ((uint64_t)rofs[nzr[mid]] < t) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  const uint32_t i0 = first_at((uint64_t)W * wid / kSegWarps);
  const uint32_t i1 = wid == kSegWarps - 1 ? S : first_at((uint64_t)W * (wid + 1) / kSegWarps);
  const uint32_t s0 = i0 < S ? (uint32_t)rofs[nzr[i0]] : W;
  const uint32_t s1 = i1 < S ? (uint32_t)rofs[nzr[i1]] : W;
  const bool ok = __syncthreads_and(mbar_wait(&bar[0], 0, err));
  if (!ok) return;  // every thread waited (bounded) for the copy

  const int64_t beg = pbase + s0, end = pbase + s1;
  const uint32_t lt = lanemask_lt();
  float* stg = reinterpret_cast<float*>(smem + L.stage) + wid * 7 * kStageLd + lane;
  float carry = 0.f;
  uint32_t kb = 0;
  for (int64_t b = beg & ~7ll; b < end; b += 256) {
    const int64_t wb = b + 8 * lane;
    uint4 qa = make_uint4(0, 0, 0, 0), qb = qa;
    if (wb < end) {
      qa = ld_stream_u4(X.packed + wb);
      qb = ld_stream_u4(X.packed + wb + 4);
    }
    uint32_t wd[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
    if (wb < beg || wb + 8 > end) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (wb + i < beg || wb + i >= end) wd[i] = 0u;
    }
    uint32_t hm = 0, big = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      hm |= (wd[i] >> 31) << i;
      big |= wd[i];
    }
    // heads in earlier lanes of this iteration
    const uint32_t h = __popc(hm);
    uint32_t hs = h;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, hs, d);
      if (lane >= d) hs += t;
    }
    const uint32_t kl = kb + hs - h;  // heads before this lane
    // row of the open segment entering the lane (row 0 reads table slot 0
    // of a zeroed word before the run's first head)
    const uint32_t rin = kl > 0 ? nzr[i0 + kl - 1] : 0u;
    float sl[8];
    {
      uint32_t cur = rin, k = kl;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if ((hm >> i) & 1u) cur = nzr[i0 + k++];
        const float t = tab[((wd[i] & (kCountTab - 1)) << pshift) | cur];
        sl[i] = t * wv[(wd[i] >> 16) & 0x7fffu];
      }
    }
    if (__any_sync(0xffffffffu, (big & 0xfff0u) != 0u)) {
      uint32_t cur = rin, k = kl;
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        if ((hm >> i) & 1u) cur = nzr[i0 + k++];
        const uint32_t cnt = wd[i] & 0xffffu;
        if (cnt >= (uint32_t)kCountTab)
          sl[i] = norm_count(cnt, X.isf[r0 + cur]) * wv[(wd[i] >> 16) & 0x7fffu];
      }
    }
    // in-lane segmented sums
#pragma unroll
    for (int i = 1; i < 8; ++i) sl[i] = ((hm >> i) & 1u) ? sl[i] : sl[i - 1] + sl[i];
    const uint32_t F = __ballot_sync(0xffffffffu, hm != 0u);
    float T = sl[7];
    uint32_t fa = hm != 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const float Tp = __shfl_up_sync(0xffffffffu, T, d);
      const uint32_t fp = __shfl_up_sync(0xffffffffu, fa, d);
      if (lane >= d) {
        if (!fa) T = Tp + T;
        fa |= fp;
      }
    }
    if ((F & (lt | (1u << lane))) == 0u) T = carry + T;
    float cin = __shfl_up_sync(0xffffffffu, T, 1);
    if (lane == 0) cin = carry;
#pragma unroll
    for (int i = 0; i < 7; ++i) stg[i * kStageLd] = sl[i];
    for (uint32_t rem = hm; rem != 0u; rem &= rem - 1u) {
      const int i = __ffs(rem) - 1;
      const uint32_t pre = hm & ((1u << i) - 1u);
      const uint32_t k = kl + __popc(pre);
      if (k > 0) {
        float val = cin;
        if (i > 0) {
          const float sv = stg[(i - 1) * kStageLd];
          val = pre ? sv : cin + sv;
        }
        rsum[nzr[i0 + k - 1]] = val;
      }
    }
    carry = __shfl_sync(0xffffffffu, T, 31);
    kb += __shfl_sync(0xffffffffu, hs, 31);
  }
  if (lane == 0 && kb > 0) rsum[nzr[i0 + kb - 1]] = carry;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < rows; i += kSegThreads)
    y[r0 + i] = X.post ? rsum[i] * X.post[r0 + i] : rsum[i];
}

// Row heads (matrix creation): bit 31 of the first word of every non-empty
// CSR row (gene indices then fit in bits 16-30).
__global__ void k_mark_row_heads(const int64_t* __restrict__ rowptr, uint64_t n,
                                 uint32_t* __restrict__ packed) {
  const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (r < n && rowptr[r + 1] > rowptr[r]) packed[rowptr[r]] |= kHeadBit;
}

// Head flags (matrix creation): bit 31 of the first word of every non-empty
// (panel, gene) segment of the transposed copy.
__global__ void k_mark_heads(const int64_t* __restrict__ rowptr,
                             const int32_t* __restrict__ colptr, uint64_t n,
                             uint32_t g, uint32_t pshift, uint32_t num_panels,
                             uint32_t* __restrict__ packed) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= (uint64_t)num_panels * g) return;
  const uint64_t p = i / g;
  const uint32_t c = (uint32_t)(i % g);
  const int32_t* cp = colptr + p * (g + 1);
  if (cp[c + 1] > cp[c]) packed[rowptr[p << pshift] + cp[c]] |= kHeadBit;
}

// z[c] = (sum over panels in panel order of partT[c][p]) / sd[c]; one warp per
// gene, lanes stride the panels, fixed xor tree.
__device__ __forceinline__ void reduce_panels_body(const float* __restrict__ partT,
                                                   uint32_t num_panels, uint32_t g,
                                                   const float* __restrict__ sd,
                                                   float* __restrict__ z, uint32_t b) {
  const int lane = threadIdx.x & 31;
  const uint32_t c = b * 8 + (threadIdx.x >> 5);
  if (c >= g) return;
  const float* row = partT + (uint64_t)c * num_panels;
  float t = 0.f;
  for (uint32_t p = lane; p < num_panels; p += 32) t += row[p];
  t = warp_sum(t);
  if (lane == 0) z[c] = sd ? t / sd[c] : t;  // pca.pyx:510-511
}

__global__ void __launch_bounds__(256)
k_reduce_panels_t(const float* __restrict__ partT, uint32_t num_panels,
                  uint32_t g, const float* __restrict__ sd,
                  float* __restrict__ z) {
  reduce_panels_body(partT, num_panels, g, sd, z, blockIdx.x);
}

__global__ void __launch_bounds__(256)
k_reduce_panels_multi(const __grid_constant__ TaskList<ReducePanelsTask> L) {
  const uint32_t i = task_of(L.first, L.count, blockIdx.x);
  const ReducePanelsTask& t = L.t[i];
  reduce_panels_body(t.partT, t.num_panels, t.g, t.sd, t.z, blockIdx.x - L.first[i]);
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

// Row order for X.v (matrix creation): rows by descending count of 32-entry
// windows (the 8-lane groups' passes), stable, by a counting sort on the host.
// BGPU_KERNELS_NATURAL keeps the natural order.
int build_row_order(Matrix* m, cudaStream_t s, uint64_t* bytes_acc) {
  if ((m->kernels & BGPU_KERNELS_NATURAL) || m->n < 2 || m->n >= (uint64_t)INT32_MAX)
    return BGPU_OK;
  std::vector<int64_t> rp(m->n + 1);
  BGPU_CUDA(cudaMemcpyAsync(rp.data(), m->rowptr, (m->n + 1) * 8, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  constexpr uint64_t kCap = 4096;  // rows of >= 4096 windows share the top bucket
  std::vector<uint32_t> key(m->n);
  std::vector<uint64_t> cnt(kCap + 1, 0);
  for (uint64_t r = 0; r < m->n; ++r) {
    const uint64_t w = std::min<uint64_t>(kCap, (uint64_t)(rp[r + 1] - rp[r] + 31) / 32);
    key[r] = (uint32_t)(kCap - w);  // descending windows
    ++cnt[key[r]];
  }
  uint64_t run = 0;
  for (auto& c : cnt) { const uint64_t t = c; c = run; run += t; }
  std::vector<int32_t> order(m->n);
  for (uint64_t r = 0; r < m->n; ++r) order[cnt[key[r]]++] = (int32_t)r;
  BGPU_CUDA(cudaMallocAsync((void**)&m->row_order, m->n * 4, s));
  *bytes_acc += m->n * 4;
  BGPU_CUDA(cudaMemcpyAsync(m->row_order, order.data(), m->n * 4, cudaMemcpyHostToDevice, s));
  BGPU_CUDA(cudaStreamSynchronize(s));  // `order` is a host temporary
  return BGPU_OK;
}

bool stream_supported(const Matrix& m) {
  return m.mode == kCounts && m.P <= (uint32_t)kMaxPanelRows &&
         SegLayout(m.P, m.g).total <= 220 * 1024;
}

int build_stream_tiles(Matrix* m, const std::vector<int64_t>& panel_rowptr,
                       cudaStream_t s, uint64_t* bytes_acc) {
  (void)panel_rowptr;
  if (!stream_supported(*m)) return BGPU_OK;
  const uint64_t nr = m->n * kCountTab;
  const uint64_t nc = (uint64_t)m->num_panels * kCountTab * m->P;
  BGPU_CUDA(cudaMallocAsync((void**)&m->rtab_r, nr * 4, s));
  BGPU_CUDA(cudaMallocAsync((void**)&m->rtab_c, nc * 4, s));
  *bytes_acc += (nr + nc) * 4;
  BGPU_CUDA(cudaMemsetAsync(m->rtab_c, 0, nc * 4, s));
  k_count_tables<<<(unsigned)ceil_div(nr, 256), 256, 0, s>>>(
      m->isf, m->n, m->pshift, m->rtab_r, m->rtab_c);
  BGPU_CHECK_LAUNCH();
  const uint64_t segs = (uint64_t)m->num_panels * m->g;
  k_mark_heads<<<(unsigned)ceil_div(segs, 256), 256, 0, s>>>(
      m->rowptr, m->colptr, m->n, m->g, m->pshift, m->num_panels, m->csc_packed);
  BGPU_CHECK_LAUNCH();
  m->csr_heads = m->g <= 32768u && RowSegLayout(m->P, m->g).total <= 220 * 1024;
  if (m->csr_heads) {
    k_mark_row_heads<<<(unsigned)ceil_div(m->n, 256), 256, 0, s>>>(m->rowptr, m->n,
                                                                    m->csr_packed);
    BGPU_CHECK_LAUNCH();
  }
  BGPU_TRY(build_row_order(m, s, bytes_acc));
  m->stream_ok = true;
  // BGPU_KERNELS_WORDS32 keeps X^T.u on the 32-bit panel words
  if (!(m->kernels & BGPU_KERNELS_WORDS32)) BGPU_TRY(build_compact16(m, s, bytes_acc));
  return BGPU_OK;
}

int launch_matvec_stream(const Matrix& m, const float* v, const float* sd,
                         float* y, int* err, cudaStream_t s) {
  const CsrView X = csr_view(m);
  if (m.csr_heads && m.spmv_seg) {
    const size_t smem = RowSegLayout(m.P, m.g).total;
    BGPU_CUDA(allow_max_smem(k_spmv_seg));
    k_spmv_seg<<<m.num_panels, kSegThreads, smem, s>>>(X, m.pshift, m.rtab_c, v, sd,
                                                       y, err);
    BGPU_CHECK_LAUNCH();
    return BGPU_OK;
  }
  const size_t smem = ((size_t)((m.g + 3) & ~3u) + 32 * 2 * kTabSlot) * 4;
  if (smem > 48 * 1024)
    BGPU_CUDA(allow_max_smem(k_spmv_rows));
  // one 8-lane group per row at most (32 groups per CTA): a small matrix
  // launches a small grid and leaves the rest of the GPU to concurrent solves
  const uint64_t want = ceil_div(m.n, 32);
  const unsigned grid = (unsigned)std::max<uint64_t>(
      1, std::min<uint64_t>(want, (uint64_t)num_sms() * kSpmvRowsCtas));
  k_spmv_rows<<<grid, 256, smem, s>>>(X, m.row_order, v, sd, y);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_rmatvec_stream(const Matrix& m, const float* u, const float* u_scale,
                          float* u_out, float* partT, int* err, cudaStream_t s) {
  if (m.compact) return launch_rmatvec16(m, u, u_scale, u_out, partT, err, s);
  const CscView X = csc_view(m);
  const size_t smem = SegLayout(m.P, m.g).total;
  BGPU_CUDA(allow_max_smem(k_rmat_seg));
  k_rmat_seg<<<m.num_panels, kRmatThreads, smem, s>>>(X, u, u_scale, u_out, partT, err);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

uint32_t reduce_panels_ctas(const Matrix& m) { return (uint32_t)ceil_div(m.g, 8); }

int launch_reduce_panels_t(const Matrix& m, const float* partT, const float* sd,
                           float* z, cudaStream_t s) {
  k_reduce_panels_t<<<reduce_panels_ctas(m), 256, 0, s>>>(partT, m.num_panels, m.g, sd, z);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_reduce_panels_multi(const TaskList<ReducePanelsTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  k_reduce_panels_multi<<<L.grid(), 256, 0, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
