// Sliced-ELL layouts of the counts matrix and the two sparse products on them
// (X.v: brisc/pca.pyx:440-475, X^T.u: brisc/pca.pyx:478-511), for up to 4096
// genes with the normalisation fused into the load.
//
// Both products give every output element to ONE lane, which sums its
// entries sequentially in a fixed storage order: no scans, no atomics, no
// cross-lane combining. What makes that fast is the storage: the sums a warp
// computes are grouped 32 at a time by similar length, and a group's data is
// interleaved lane by lane (unit k of lane l at unit k*32 + l, 8 bytes = four
// 16-bit entries per unit), so every warp load is one coalesced 256-byte line.
//
// X.v ("rows"): the sums are the cell rows. Rows are ordered by length
// (units of 4 entries, longest first) and taken 32 at a time. Entry =
//   count << 12 | gene      (count < 16; 0 = padding or escaped)
// Each lane holds its row's 16-entry count table log1pf(c * isf) in a private
// shared-memory slot (stride 17: the 32 lanes of a warp hit 32 banks when
// their counts agree), w = v / sd is in shared memory. A count >= 16
// ("escape", 0.03 % of NB counts) is stored as 0 in the stream and kept in a
// per-row list (gene << 16 | count) that the lane adds after the stream.
//
// X^T.u ("panels"): the sums are (panel, gene) segments over panels of P <=
// 512 rows. A panel's segments are ordered by length and taken 32 at a time;
// a segment's entries keep the row order. Entry = a BYTE OFFSET into the
// CTA's shared memory:
//   (count * P + local_row) * 4     count < 16: the panel's table, laid out
//                                   [count][row] = log1pf(count * isf) * u
//   32768 + slot * 4                count >= 16: the slot-th escape value of
//                                   the panel, evaluated exactly per panel
// so the inner loop is: split the 32-bit word, load, add -- three
// instructions per entry whatever the count. Each CTA walks a fixed range of
// consecutive panels and adds each panel's segment sums into per-gene
// shared-memory totals in panel order; the per-CTA totals are reduced in CTA
// order by k_reduce_panels_t. The same kernel with u = 1 and FP64 sums gives
// the per-gene moments for the clipped standard deviation.
//
// Padding entries are 0: in X.v they read table slot 0 (= 0) times w[0]; in
// X^T.u byte offset 0 is table[0][0] = 0. Results depend only on the data and
// the layout, so repeated products are bit-identical.
#include <algorithm>
#include <cstring>
#include <vector>

#include "matrix.cuh"

namespace bgpu {

namespace {

constexpr int kSellThreads = 256;
constexpr int kSellWarps = kSellThreads / 32;
constexpr int kXvCtasPerSm = 6;
constexpr int kXtCtasPerSm = 4;
constexpr uint32_t kXvMaxGenes = 4096;      // 12-bit gene field
constexpr uint32_t kXvMaxUnits = 1024;      // rows of <= 4096 entries
constexpr uint32_t kXtMaxP = 512;           // (15 * P + P - 1) * 4 < 32768
constexpr uint32_t kXtTableBytes = 32768;   // table region; escapes follow
constexpr uint32_t kXtMaxEsc = 8192;        // escape slots: offsets < 65536
constexpr uint32_t kXtMaxUnits = kXtMaxP / 4;
constexpr uint32_t kTabStride = 17;         // per-lane X.v count table slot
constexpr uint32_t kNoGene = 0xffffu;

enum SellErr : int { kSellErrLong = 1, kSellErrEsc = 2 };

// ---------------------------------------------------------------------------
// X.v
// cta, ctas: the CTA's index and the CTAs of the launch (the warps stride
// the groups; each row's sum is one lane's whatever the grid)
__device__ __forceinline__ void xv_sell_body(const XvView& X, const float* __restrict__ v,
                                             const float* __restrict__ sd,
                                             float* __restrict__ y, uint32_t cta,
                                             uint32_t ctas) {
  extern __shared__ __align__(16) float sm[];
  float* w = sm;                                   // v / sd, g floats
  float* tabs = sm + ((X.g + 3) & ~3u);            // [warp][lane][kTabStride]
  for (uint32_t c = threadIdx.x; c < X.g; c += kSellThreads)
    w[c] = sd ? v[c] / sd[c] : v[c];  // pca.pyx:461-462
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* tb = tabs + (wid * 32 + lane) * kTabStride;
  const uint32_t nwarps = ctas * kSellWarps;
  const uint2 z2 = make_uint2(0u, 0u);
  for (uint32_t q = cta * kSellWarps + wid; q < X.groups; q += nwarps) {
    const uint64_t pos = (uint64_t)q * 32 + lane;
    const float f = X.isf[pos];  // 0 on the padding lanes of the last group
    tb[0] = 0.f;
#pragma unroll
    for (int c = 1; c < 16; ++c) tb[c] = norm_count((uint32_t)c, f);
    const uint2* src = X.data + X.grp[q] + lane;
    const uint32_t U = X.units[q];
    float acc = 0.f;
    // four units (16 entries) per step, the next four in flight meanwhile
    uint2 a0 = 0 < U ? ld_stream_u2(src) : z2;
    uint2 a1 = 1 < U ? ld_stream_u2(src + 32) : z2;
    uint2 a2 = 2 < U ? ld_stream_u2(src + 64) : z2;
    uint2 a3 = 3 < U ? ld_stream_u2(src + 96) : z2;
    for (uint32_t k = 0; k < U; k += 4) {
      const uint2* nx = src + (uint64_t)(k + 4) * 32;
      const uint2 b0 = k + 4 < U ? ld_stream_u2(nx) : z2;
      const uint2 b1 = k + 5 < U ? ld_stream_u2(nx + 32) : z2;
      const uint2 b2 = k + 6 < U ? ld_stream_u2(nx + 64) : z2;
      const uint2 b3 = k + 7 < U ? ld_stream_u2(nx + 96) : z2;
      const uint32_t wd[8] = {a0.x, a0.y, a1.x, a1.y, a2.x, a2.y, a3.x, a3.y};
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        acc = fmaf(tb[(wd[i] >> 12) & 15u], w[wd[i] & 0xfffu], acc);
        acc = fmaf(tb[wd[i] >> 28], w[(wd[i] >> 16) & 0xfffu], acc);
      }
      a0 = b0; a1 = b1; a2 = b2; a3 = b3;
    }
    const int32_t row = X.perm[pos];
    if (row >= 0) {
      const uint32_t ne = X.esc_n[pos];
      if (ne) {  // counts >= 16, after the stream, in the row's order
        const uint32_t* er = X.esc + X.esc_base[pos];
        for (uint32_t i = 0; i < ne; ++i) {
          const uint32_t e = er[i];
          acc = fmaf(norm_count(e & 0xffffu, f), w[e >> 16], acc);
        }
      }
      y[row] = X.post ? acc * X.post[pos] : acc;
    }
  }
}

__global__ void __launch_bounds__(kSellThreads, kXvCtasPerSm)
k_xv_sell(XvView X, const float* __restrict__ v, const float* __restrict__ sd,
          float* __restrict__ y) {
  xv_sell_body(X, v, sd, y, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kSellThreads, kXvCtasPerSm)
k_xv_sell_multi(const __grid_constant__ TaskList<XvTask> L) {
  const uint32_t i = task_of(L.first, L.count, blockIdx.x);
  const XvTask& t = L.t[i];
  xv_sell_body(t.X, t.v, t.sd, t.y, blockIdx.x - L.first[i], L.first[i + 1] - L.first[i]);
}

// ---------------------------------------------------------------------------
// X^T.u (kMom = false) and the per-gene moments (kMom = true: u = 1, value
// and squared value summed in FP64).
template <bool kMom>
struct XtAcc;
template <>
struct XtAcc<false> {
  float s = 0.f;
  __device__ __forceinline__ void add(float v) { s += v; }
};
template <>
struct XtAcc<true> {
  double s = 0.0, q = 0.0;
  __device__ __forceinline__ void add(float v) {
    s += (double)v;
    q += (double)v * (double)v;
  }
};

__host__ __device__ inline uint32_t xt_esc_floats(uint32_t esc_max) {
  return (esc_max + 3u) & ~3u;
}
__host__ __device__ inline size_t xt_smem_bytes(uint32_t P, uint32_t g,
                                                uint32_t esc_max, bool mom) {
  return kXtTableBytes + 4ull * xt_esc_floats(esc_max) + 4ull * ((P + 3) & ~3u) +
         (mom ? 16ull : 4ull) * g;
}

__device__ __forceinline__ float smem_at(const unsigned char* base, uint32_t off) {
  return *reinterpret_cast<const float*>(base + off);
}

// cta, ctas: the CTA's index and the CTAs of the launch (ctas is the row
// count of the gene-major partials)
template <bool kMom>
__device__ __forceinline__ void xt_sell_body(const XtView& X, const float* __restrict__ u,
                                             const float* __restrict__ u_scale,
                                             float* __restrict__ u_out,
                                             float* __restrict__ partT,
                                             double2* __restrict__ mom, uint32_t cta,
                                             uint32_t ctas) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* tab = reinterpret_cast<float*>(smem);  // [16][P]
  float* escv = reinterpret_cast<float*>(smem + kXtTableBytes);
  float* us = escv + xt_esc_floats(X.esc_max);
  float* gs = us + ((X.P + 3) & ~3u);           // per-gene totals (X^T.u)
  double2* gm = reinterpret_cast<double2*>(gs);  // per-gene moments
  for (uint32_t c = threadIdx.x; c < X.g; c += kSellThreads) {
    if constexpr (kMom) gm[c] = make_double2(0.0, 0.0);
    else gs[c] = 0.f;
  }
  const float scale = (!kMom && u_scale) ? *u_scale : 1.f;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t P = X.P;
  const uint32_t p0 = cta * X.ppc;
  const uint32_t p1 = min(X.panels, p0 + X.ppc);
  const uint2 z2 = make_uint2(0u, 0u);
  for (uint32_t p = p0; p < p1; ++p) {
    const uint64_t r0 = (uint64_t)p * P;
    const uint32_t rows = (uint32_t)min_u64(P, X.n - r0);
    __syncthreads();  // the previous panel's table is no longer read
    for (uint32_t i = threadIdx.x; i < P; i += kSellThreads) {
      float uu = 0.f, f = 0.f;
      if (i < rows) {
        f = X.isf[r0 + i];
        if constexpr (kMom) {
          uu = X.post ? X.post[r0 + i] : 1.f;
        } else {
          uu = u_scale ? u[r0 + i] * scale : u[r0 + i];
          if (u_out) u_out[r0 + i] = uu;
          if (X.post) uu *= X.post[r0 + i];
        }
      }
      us[i] = uu;
      tab[i] = 0.f;
#pragma unroll
      for (uint32_t c = 1; c < 16; ++c)
        tab[c * P + i] = i < rows ? norm_count(c, f) * uu : 0.f;
    }
    const uint32_t eb = X.esc_base[p], ne = X.esc_base[p + 1] - eb;
    if (ne) {
      __syncthreads();  // us[] is complete
      for (uint32_t t = threadIdx.x; t < ne; t += kSellThreads) {
        const uint32_t rec = X.esc[eb + t];
        const uint32_t lr = rec >> 16;
        escv[t] = norm_count(rec & 0xffffu, X.isf[r0 + lr]) * us[lr];
      }
    }
    __syncthreads();
    const uint32_t q1 = X.pgrp[p + 1];
    for (uint32_t q = X.pgrp[p] + wid; q < q1; q += kSellWarps) {
      const uint32_t gene = X.gene[(uint64_t)q * 32 + lane];
      const uint2* src = X.data + X.grp[q] + lane;
      const uint32_t U = X.units[q];
      XtAcc<kMom> acc;
      uint2 a0 = 0 < U ? ld_stream_u2(src) : z2;
      uint2 a1 = 1 < U ? ld_stream_u2(src + 32) : z2;
      uint2 a2 = 2 < U ? ld_stream_u2(src + 64) : z2;
      uint2 a3 = 3 < U ? ld_stream_u2(src + 96) : z2;
      for (uint32_t k = 0; k < U; k += 4) {
        const uint2* nx = src + (uint64_t)(k + 4) * 32;
        const uint2 b0 = k + 4 < U ? ld_stream_u2(nx) : z2;
        const uint2 b1 = k + 5 < U ? ld_stream_u2(nx + 32) : z2;
        const uint2 b2 = k + 6 < U ? ld_stream_u2(nx + 64) : z2;
        const uint2 b3 = k + 7 < U ? ld_stream_u2(nx + 96) : z2;
        const uint32_t wd[8] = {a0.x, a0.y, a1.x, a1.y, a2.x, a2.y, a3.x, a3.y};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          acc.add(smem_at(smem, wd[i] & 0xffffu));
          acc.add(smem_at(smem, wd[i] >> 16));
        }
        a0 = b0; a1 = b1; a2 = b2; a3 = b3;
      }
      if (gene != kNoGene) {  // one segment per gene and panel: no collisions
        if constexpr (kMom) {
          gm[gene].x += acc.s;
          gm[gene].y += acc.q;
        } else {
          gs[gene] += acc.s;
        }
      }
    }
  }
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < X.g; c += kSellThreads) {
    if constexpr (kMom) mom[(uint64_t)cta * X.g + c] = gm[c];
    else partT[(uint64_t)c * ctas + cta] = gs[c];
  }
}

template <bool kMom>
__global__ void __launch_bounds__(kSellThreads, kXtCtasPerSm)
k_xt_sell(XtView X, const float* __restrict__ u, const float* __restrict__ u_scale,
          float* __restrict__ u_out, float* __restrict__ partT,
          double2* __restrict__ mom) {
  xt_sell_body<kMom>(X, u, u_scale, u_out, partT, mom, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(kSellThreads, kXtCtasPerSm)
k_xt_sell_multi(const __grid_constant__ TaskList<XtTask> L) {
  const uint32_t i = task_of(L.first, L.count, blockIdx.x);
  const XtTask& t = L.t[i];
  xt_sell_body<false>(t.X, t.u, t.u_scale, t.u_out, t.partT, nullptr,
                      blockIdx.x - L.first[i], L.first[i + 1] - L.first[i]);
}

// ---------------------------------------------------------------------------
// Layout construction (matrix creation). The order of rows inside a length
// bucket and of segments inside a panel's length bucket come from atomics and
// may differ between builds; no sum depends on them (each sum is one lane's,
// over its entries in CSR / row order).

// Per row: units of 4 entries, escapes; histogram of units.
__global__ void k_xv_hist(const int64_t* __restrict__ rowptr,
                          const uint32_t* __restrict__ packed, uint64_t n,
                          uint16_t* __restrict__ row_units, uint16_t* __restrict__ row_esc,
                          uint32_t* __restrict__ hist, unsigned long long* __restrict__ esc_total,
                          int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t r = warp; r < n; r += nwarps) {
    const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
    uint32_t ne = 0;
    for (int64_t e = e0 + lane; e < e1; e += 32)
      ne += (packed[e] & 0xffffu) >= 16u ? 1u : 0u;
    ne = __reduce_add_sync(0xffffffffu, ne);
    if (lane == 0) {
      const uint64_t len = (uint64_t)(e1 - e0);
      uint32_t un = (uint32_t)((len + 3) / 4);
      if (un > kXvMaxUnits) {
        atomicOr(err, kSellErrLong);
        un = kXvMaxUnits;
      }
      row_units[r] = (uint16_t)un;
      row_esc[r] = (uint16_t)ne;
      atomicAdd(&hist[un], 1u);
      if (ne) atomicAdd(esc_total, (unsigned long long)ne);
    }
  }
}

// Row -> position (buckets of equal units, longest first), per-position isf,
// post and escape list.
__global__ void k_xv_place(const uint16_t* __restrict__ row_units,
                           const uint16_t* __restrict__ row_esc, uint64_t n,
                           uint32_t* __restrict__ cursor, const float* __restrict__ isf,
                           const float* __restrict__ post, int32_t* __restrict__ perm,
                           float* __restrict__ pisf, float* __restrict__ ppost,
                           uint16_t* __restrict__ pesc_n, uint32_t* __restrict__ pesc_base,
                           unsigned long long* __restrict__ esc_cursor) {
  const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const bool live = r < n;
  const uint32_t un = live ? row_units[r] : 0xffffffffu;
  // one atomic per distinct bucket in the warp
  const uint32_t peers = __match_any_sync(0xffffffffu, un);
  const int leader = __ffs(peers) - 1;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (live && lane == leader) base = atomicAdd(&cursor[un], (uint32_t)__popc(peers));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (!live) return;
  const uint32_t pos = base + __popc(peers & ((1u << lane) - 1u));
  perm[pos] = (int32_t)r;
  pisf[pos] = isf[r];
  if (ppost) ppost[pos] = post[r];
  const uint32_t ne = row_esc[r];
  pesc_n[pos] = (uint16_t)ne;
  pesc_base[pos] = ne ? (uint32_t)atomicAdd(esc_cursor, (unsigned long long)ne) : 0u;
}

// One warp per group of 32 positions: lane l writes its row's units.
__global__ void k_xv_fill(const int64_t* __restrict__ rowptr,
                          const uint32_t* __restrict__ packed,
                          const int32_t* __restrict__ perm, const uint32_t* __restrict__ grp,
                          const uint16_t* __restrict__ units,
                          const uint32_t* __restrict__ pesc_base, uint32_t groups,
                          uint2* __restrict__ data, uint32_t* __restrict__ esc) {
  const int lane = threadIdx.x & 31;
  const uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (q >= groups) return;
  const uint64_t pos = q * 32 + lane;
  const int32_t r = perm[pos];
  if (r < 0) return;
  const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
  uint32_t* er = esc + pesc_base[pos];
  uint32_t k_esc = 0;
  uint2* dst = data + grp[q] + lane;
  const uint32_t U = units[q];
  for (uint32_t k = 0; k < U; ++k) {
    uint32_t h[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int64_t e = e0 + 4 * (int64_t)k + s;
      if (e < e1) {
        const uint32_t wv = packed[e];
        const uint32_t gene = (wv >> 16) & 0xffffu, cnt = wv & 0xffffu;
        if (cnt < 16u) {
          h[s] = (cnt << 12) | gene;
        } else {
          er[k_esc++] = (gene << 16) | cnt;
        }
      }
    }
    dst[(uint64_t)k * 32] = make_uint2(h[0] | (h[1] << 16), h[2] | (h[3] << 16));
  }
}

// Per panel: segment lengths per gene (into seg_len[p][g]), escapes, the
// segments sorted by units (longest first) into order[p][slot], and the
// panel's group count and unit total.
__global__ void __launch_bounds__(1024)
k_xt_count(const int64_t* __restrict__ rowptr, const uint32_t* __restrict__ packed,
           uint64_t n, uint32_t g, uint32_t P, uint32_t* __restrict__ seg_len,
           uint16_t* __restrict__ order, uint32_t* __restrict__ panel_groups,
           uint32_t* __restrict__ panel_units, uint32_t* __restrict__ panel_esc,
           int* __restrict__ err) {
  extern __shared__ uint32_t cnt[];  // g counters, then kXtMaxUnits + 2 buckets
  uint32_t* bucket = cnt + g;
  __shared__ uint32_t nesc;
  const uint32_t p = blockIdx.x;
  const uint64_t r0 = (uint64_t)p * P;
  const uint64_t r1 = min_u64(n, r0 + P);
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) cnt[c] = 0;
  for (uint32_t b = threadIdx.x; b < kXtMaxUnits + 2; b += blockDim.x) bucket[b] = 0;
  if (threadIdx.x == 0) nesc = 0;
  __syncthreads();
  const int64_t e0 = rowptr[r0], e1 = rowptr[r1];
  uint32_t my_esc = 0;
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const uint32_t wv = packed[e];
    atomicAdd(&cnt[(wv >> 16) & 0xffffu], 1u);
    my_esc += (wv & 0xffffu) >= 16u ? 1u : 0u;
  }
  if (my_esc) atomicAdd(&nesc, my_esc);
  __syncthreads();
  // bucket histogram by units, descending: bucket index kXtMaxUnits - units
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) {
    const uint32_t len = cnt[c];
    seg_len[(uint64_t)p * g + c] = len;
    if (len == 0) continue;
    uint32_t un = (len + 3) / 4;
    if (un > kXtMaxUnits) {
      atomicOr(err, kSellErrLong);
      un = kXtMaxUnits;
    }
    atomicAdd(&bucket[kXtMaxUnits - un], 1u);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (uint32_t b = 0; b < kXtMaxUnits; ++b) {  // buckets of >= 1 unit
      const uint32_t t = bucket[b];
      bucket[b] = run;
      run += t;
    }
    bucket[kXtMaxUnits + 1] = run;  // segments
    if (nesc > kXtMaxEsc) atomicOr(err, kSellErrEsc);
  }
  __syncthreads();
  const uint32_t nseg = bucket[kXtMaxUnits + 1];
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) {
    const uint32_t len = cnt[c];
    if (len == 0) continue;
    const uint32_t un = min((len + 3) / 4, kXtMaxUnits);
    const uint32_t slot = atomicAdd(&bucket[kXtMaxUnits - un], 1u);
    order[(uint64_t)p * g + slot] = (uint16_t)c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t groups = (nseg + 31) / 32;
    uint32_t units = 0;
    for (uint32_t j = 0; j < groups; ++j) {
      const uint32_t c = order[(uint64_t)p * g + j * 32];
      units += 32u * min((cnt[c] + 3) / 4, kXtMaxUnits);
    }
    panel_groups[p] = groups;
    panel_units[p] = units;
    panel_esc[p] = nesc;
  }
}

// Per panel: group descriptors and the unit of lane 0 of each gene's segment.
__global__ void k_xt_struct(const uint32_t* __restrict__ seg_len,
                            const uint16_t* __restrict__ order, uint32_t g,
                            const uint32_t* __restrict__ pgrp,
                            const uint32_t* __restrict__ punit,
                            uint32_t* __restrict__ grp, uint16_t* __restrict__ units,
                            uint16_t* __restrict__ gene, uint32_t* __restrict__ seg_loc) {
  const uint32_t p = blockIdx.x;
  const uint32_t q0 = pgrp[p], groups = pgrp[p + 1] - q0;
  const uint32_t* len = seg_len + (uint64_t)p * g;
  const uint16_t* ord = order + (uint64_t)p * g;
  __shared__ uint32_t gbase[kXvMaxGenes / 32 + 1];  // unit base of each group
  if (threadIdx.x == 0) {
    uint32_t run = punit[p];
    for (uint32_t j = 0; j < groups; ++j) {
      gbase[j] = run;
      run += 32u * min((len[ord[j * 32]] + 3) / 4, kXtMaxUnits);
    }
  }
  __shared__ uint32_t total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  uint32_t mine = 0;
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) mine += len[c] ? 1u : 0u;
  if (mine) atomicAdd(&total, mine);
  __syncthreads();
  const uint32_t nseg = total;
  for (uint32_t j = threadIdx.x; j < groups; j += blockDim.x) {
    grp[q0 + j] = gbase[j];
    units[q0 + j] = (uint16_t)min((len[ord[j * 32]] + 3) / 4, kXtMaxUnits);
  }
  for (uint32_t s = threadIdx.x; s < groups * 32; s += blockDim.x) {
    const uint32_t j = s / 32, l = s % 32;
    if (s < nseg) {
      const uint32_t c = ord[s];
      gene[(uint64_t)(q0 + j) * 32 + l] = (uint16_t)c;
      seg_loc[(uint64_t)p * g + c] = gbase[j] + l;
    } else {
      gene[(uint64_t)(q0 + j) * 32 + l] = (uint16_t)kNoGene;
    }
  }
}

// Per panel (one CTA, 8 warps over contiguous row ranges): the rank of every
// entry inside its (panel, gene) segment in row order, then its 16-bit entry.
__global__ void __launch_bounds__(kSellThreads)
k_xt_scatter(const int64_t* __restrict__ rowptr, const uint32_t* __restrict__ packed,
             uint64_t n, uint32_t g, uint32_t P, const uint32_t* __restrict__ seg_loc,
             const uint32_t* __restrict__ esc_base, uint16_t* __restrict__ data16,
             uint32_t* __restrict__ esc) {
  extern __shared__ uint32_t wc[];  // [warp][g] running ranks
  __shared__ uint32_t esc_next;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t p = blockIdx.x;
  const uint64_t r0 = (uint64_t)p * P;
  const uint32_t rows = (uint32_t)min_u64(P, n - r0);
  const uint32_t per = (rows + kSellWarps - 1) / kSellWarps;
  const uint32_t ra = min(rows, wid * per), rb = min(rows, ra + per);
  uint32_t* my = wc + (uint64_t)wid * g;
  for (uint32_t c = threadIdx.x; c < kSellWarps * g; c += kSellThreads) wc[c] = 0;
  if (threadIdx.x == 0) esc_next = 0;
  __syncthreads();
  for (uint32_t r = ra; r < rb; ++r) {
    const int64_t e0 = rowptr[r0 + r], e1 = rowptr[r0 + r + 1];
    for (int64_t e = e0 + lane; e < e1; e += 32)
      atomicAdd(&my[(packed[e] >> 16) & 0xffffu], 1u);
  }
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < g; c += kSellThreads) {
    uint32_t run = 0;
    for (int w = 0; w < kSellWarps; ++w) {
      const uint32_t t = wc[(uint64_t)w * g + c];
      wc[(uint64_t)w * g + c] = run;
      run += t;
    }
  }
  __syncthreads();
  const uint32_t* loc = seg_loc + (uint64_t)p * g;
  const uint32_t eb = esc_base[p];
  for (uint32_t r = ra; r < rb; ++r) {
    const int64_t e0 = rowptr[r0 + r], e1 = rowptr[r0 + r + 1];
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      const uint32_t wv = packed[e];
      const uint32_t c = (wv >> 16) & 0xffffu, cnt = wv & 0xffffu;
      const uint32_t k = atomicAdd(&my[c], 1u);  // a row's genes are distinct
      const uint64_t d = ((uint64_t)loc[c] + (uint64_t)(k >> 2) * 32) * 4 + (k & 3u);
      uint32_t h;
      if (cnt < 16u) {
        h = (cnt * P + r) * 4u;
      } else {
        const uint32_t slot = atomicAdd(&esc_next, 1u);  // < kXtMaxEsc (checked)
        esc[eb + slot] = (r << 16) | cnt;
        h = kXtTableBytes + slot * 4u;
      }
      data16[d] = (uint16_t)h;
    }
    __syncwarp();
  }
}

}  // namespace

// ---------------------------------------------------------------------------
bool sell_supported(const Matrix& m) {
  return m.mode == kCounts && m.g <= kXvMaxGenes && m.n >= 1 &&
         m.n < (uint64_t)INT32_MAX;
}

// Panel rows and panels per CTA: one wave of kXtCtasPerSm CTAs per SM, each
// with ppc consecutive panels of P <= 512 rows (P a multiple of 32). A
// requested P (want_P) keeps the wave rule for the panels per CTA only.
static void xt_shape(uint64_t n, int sms, uint32_t want_P, uint32_t* P, uint32_t* ppc,
                     uint32_t* panels, uint32_t* ctas) {
  const uint64_t slots = (uint64_t)sms * kXtCtasPerSm;
  uint64_t k, p;
  if (want_P) {
    p = want_P;
    k = std::max<uint64_t>(1, ceil_div(ceil_div(n, p), slots));
  } else {
    k = std::max<uint64_t>(1, ceil_div(n, slots * kXtMaxP));
    p = ceil_div(n, slots * k);
    p = std::min<uint64_t>(kXtMaxP, std::max<uint64_t>(128, round_up(p, 32)));
  }
  *P = (uint32_t)p;
  *panels = (uint32_t)ceil_div(n, p);
  *ppc = (uint32_t)k;
  *ctas = (uint32_t)ceil_div(*panels, k);
}

int build_sell(Matrix* m, cudaStream_t s, bool* built) {
  *built = false;
  if (!sell_supported(*m)) return BGPU_OK;
  const uint64_t n = m->n;
  const uint32_t g = m->g;
  int* d_err = nullptr;
  uint32_t* hist = nullptr;
  unsigned long long* ctr = nullptr;  // [0] escapes total, [1] escape cursor
  uint16_t *row_units = nullptr, *row_esc = nullptr;
  uint32_t* seg_len = nullptr;
  uint16_t* order = nullptr;
  uint32_t *pg = nullptr, *pu = nullptr, *pe = nullptr, *seg_loc = nullptr;
  uint32_t* cursor = nullptr;
  struct Temps {  // build temporaries, released (stream-ordered) on return
    void* p[12] = {};
    cudaStream_t s;
    ~Temps() {
      for (void* q : p)
        if (q) cudaFreeAsync(q, s);
    }
  } tmp{{}, s};
  int ntmp = 0;
  auto raw_alloc = [&](void** p, size_t b) -> int {
    cudaError_t e = cudaMallocAsync(p, std::max<size_t>(b, 16), s);
    if (e != cudaSuccess) {
      *p = nullptr;
      set_error(std::string("cudaMalloc(") + std::to_string(b) + ") failed: " +
                cudaGetErrorString(e));
      return BGPU_ERR_ALLOC;
    }
    return BGPU_OK;
  };
  auto alloc = [&](void** p, size_t b) -> int {  // temporary
    BGPU_TRY(raw_alloc(p, b));
    tmp.p[ntmp++] = *p;
    return BGPU_OK;
  };
  auto palloc = [&](void** p, size_t b) -> int {  // persistent (matrix_free)
    BGPU_TRY(raw_alloc(p, b));
    m->bytes += std::max<size_t>(b, 16);
    return BGPU_OK;
  };

  // ---- X.v rows
  BGPU_TRY(alloc((void**)&d_err, 16));
  BGPU_TRY(alloc((void**)&hist, (kXvMaxUnits + 1) * 4));
  BGPU_TRY(alloc((void**)&ctr, 16));
  BGPU_TRY(alloc((void**)&row_units, n * 2));
  BGPU_TRY(alloc((void**)&row_esc, n * 2));
  BGPU_CUDA(cudaMemsetAsync(d_err, 0, 16, s));
  BGPU_CUDA(cudaMemsetAsync(hist, 0, (kXvMaxUnits + 1) * 4, s));
  BGPU_CUDA(cudaMemsetAsync(ctr, 0, 16, s));
  {
    const unsigned blocks = (unsigned)std::max<uint64_t>(
        1, std::min<uint64_t>(ceil_div(n, 8), (uint64_t)num_sms() * 16));
    k_xv_hist<<<blocks, 256, 0, s>>>(m->rowptr, m->csr_packed, n, row_units, row_esc,
                                     hist, ctr, d_err);
    BGPU_CHECK_LAUNCH();
  }
  std::vector<uint32_t> h_hist(kXvMaxUnits + 1);
  unsigned long long h_esc = 0;
  int h_err = 0;
  BGPU_CUDA(cudaMemcpyAsync(h_hist.data(), hist, h_hist.size() * 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaMemcpyAsync(&h_esc, ctr, 8, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  if (h_err) return BGPU_OK;  // rows too long for the layout: keep the panel layout
  const uint64_t groups = ceil_div(n, 32), npos = groups * 32;
  // bucket starts, longest first; the unit count of every position
  std::vector<uint32_t> start(kXvMaxUnits + 1);
  std::vector<uint32_t> gunits(groups), gbase(groups);
  {
    uint64_t run = 0;
    for (int u = (int)kXvMaxUnits; u >= 0; --u) {
      start[u] = (uint32_t)run;
      run += h_hist[u];
    }
    // position -> units: walk the buckets in descending order
    int u = (int)kXvMaxUnits;
    uint64_t bucket_end = h_hist[u];
    uint64_t ubase = 0;
    for (uint64_t q = 0; q < groups; ++q) {
      const uint64_t pos = q * 32;
      while (u > 0 && pos >= bucket_end) {
        --u;
        bucket_end += h_hist[u];
      }
      const uint32_t un = pos < n ? (uint32_t)u : 0u;
      gunits[q] = un;
      gbase[q] = (uint32_t)ubase;
      ubase += 32ull * un;
      if (ubase >= (1ull << 32)) return BGPU_OK;  // beyond 32-bit unit indices
    }
    m->xv.total_units = ubase;
  }
  m->xv.groups = (uint32_t)groups;
  m->xv.g = g;
  m->xv.n = n;
  BGPU_TRY(palloc((void**)&m->xv_perm, npos * 4));
  BGPU_TRY(palloc((void**)&m->xv_isf, npos * 4));
  if (m->post) BGPU_TRY(palloc((void**)&m->xv_post, npos * 4));
  BGPU_TRY(palloc((void**)&m->xv_esc_n, npos * 2));
  BGPU_TRY(palloc((void**)&m->xv_esc_base, npos * 4));
  BGPU_TRY(palloc((void**)&m->xv_esc, std::max<uint64_t>(h_esc, 1) * 4));
  BGPU_TRY(palloc((void**)&m->xv_grp, groups * 4));
  BGPU_TRY(palloc((void**)&m->xv_units, groups * 2));
  BGPU_TRY(palloc((void**)&m->xv_data, std::max<uint64_t>(m->xv.total_units, 1) * 8));
  BGPU_CUDA(cudaMemsetAsync(m->xv_perm, 0xff, npos * 4, s));
  BGPU_CUDA(cudaMemsetAsync(m->xv_isf, 0, npos * 4, s));
  if (m->xv_post) BGPU_CUDA(cudaMemsetAsync(m->xv_post, 0, npos * 4, s));
  BGPU_CUDA(cudaMemsetAsync(m->xv_esc_n, 0, npos * 2, s));
  BGPU_CUDA(cudaMemsetAsync(m->xv_esc_base, 0, npos * 4, s));
  BGPU_CUDA(cudaMemsetAsync(m->xv_data, 0, std::max<uint64_t>(m->xv.total_units, 1) * 8, s));
  BGPU_CUDA(cudaMemcpyAsync(m->xv_grp, gbase.data(), groups * 4, cudaMemcpyHostToDevice, s));
  {
    std::vector<uint16_t> u16(gunits.begin(), gunits.end());
    BGPU_CUDA(cudaMemcpyAsync(m->xv_units, u16.data(), groups * 2, cudaMemcpyHostToDevice, s));
    BGPU_TRY(alloc((void**)&cursor, (kXvMaxUnits + 1) * 4));
    BGPU_CUDA(cudaMemcpyAsync(cursor, start.data(), start.size() * 4, cudaMemcpyHostToDevice, s));
    k_xv_place<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(
        row_units, row_esc, n, cursor, m->isf, m->post, m->xv_perm, m->xv_isf, m->xv_post,
        m->xv_esc_n, m->xv_esc_base, ctr + 1);
    BGPU_CHECK_LAUNCH();
    k_xv_fill<<<(unsigned)ceil_div(groups * 32, 256), 256, 0, s>>>(
        m->rowptr, m->csr_packed, m->xv_perm, m->xv_grp, m->xv_units, m->xv_esc_base,
        (uint32_t)groups, m->xv_data, m->xv_esc);
    BGPU_CHECK_LAUNCH();
    BGPU_CUDA(cudaStreamSynchronize(s));  // host vectors above are temporaries
  }

  // ---- X^T.u panels
  uint32_t P, ppc, panels, ctas;
  xt_shape(n, num_sms(), m->sell_P, &P, &ppc, &panels, &ctas);
  BGPU_TRY(alloc((void**)&seg_len, (uint64_t)panels * g * 4));
  BGPU_TRY(alloc((void**)&order, (uint64_t)panels * g * 2));
  BGPU_TRY(alloc((void**)&pg, (uint64_t)panels * 4));
  BGPU_TRY(alloc((void**)&pu, (uint64_t)panels * 4));
  BGPU_TRY(alloc((void**)&pe, (uint64_t)panels * 4));
  {
    const size_t smem = ((size_t)g + kXtMaxUnits + 2) * 4;
    if (smem > 48 * 1024) BGPU_CUDA(allow_max_smem(k_xt_count));
    k_xt_count<<<panels, 1024, smem, s>>>(m->rowptr, m->csr_packed, n, g, P, seg_len,
                                          order, pg, pu, pe, d_err);
    BGPU_CHECK_LAUNCH();
  }
  std::vector<uint32_t> h_pg(panels), h_pu(panels), h_pe(panels);
  BGPU_CUDA(cudaMemcpyAsync(h_pg.data(), pg, panels * 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaMemcpyAsync(h_pu.data(), pu, panels * 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaMemcpyAsync(h_pe.data(), pe, panels * 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  if (h_err) return BGPU_OK;  // too many escapes or segments: keep the panel layout
  std::vector<uint32_t> pgrp(panels + 1), punit(panels), pesc(panels + 1);
  uint64_t ugroups = 0, uunits = 0, uesc = 0;
  uint32_t esc_max = 0;
  for (uint32_t p = 0; p < panels; ++p) {
    pgrp[p] = (uint32_t)ugroups;
    punit[p] = (uint32_t)uunits;
    pesc[p] = (uint32_t)uesc;
    ugroups += h_pg[p];
    uunits += h_pu[p];
    uesc += h_pe[p];
    esc_max = std::max(esc_max, h_pe[p]);
    if (uunits >= (1ull << 32) || uesc >= (1ull << 32)) return BGPU_OK;
  }
  pgrp[panels] = (uint32_t)ugroups;
  pesc[panels] = (uint32_t)uesc;
  m->xt.P = P;
  m->xt.ppc = ppc;
  m->xt.panels = panels;
  m->xt.ctas = ctas;
  m->xt.g = g;
  m->xt.n = n;
  m->xt.esc_max = esc_max;
  m->xt.total_units = uunits;
  m->xt.groups = (uint32_t)ugroups;
  if (xt_smem_bytes(P, g, esc_max, true) > (size_t)device_smem_optin()) return BGPU_OK;
  BGPU_TRY(palloc((void**)&m->xt_pgrp, (panels + 1) * 4ull));
  BGPU_TRY(palloc((void**)&m->xt_esc_base, (panels + 1) * 4ull));
  BGPU_TRY(palloc((void**)&m->xt_esc, std::max<uint64_t>(uesc, 1) * 4));
  BGPU_TRY(palloc((void**)&m->xt_grp, std::max<uint64_t>(ugroups, 1) * 4));
  BGPU_TRY(palloc((void**)&m->xt_units, std::max<uint64_t>(ugroups, 1) * 2));
  BGPU_TRY(palloc((void**)&m->xt_gene, std::max<uint64_t>(ugroups, 1) * 64));
  BGPU_TRY(palloc((void**)&m->xt_data, std::max<uint64_t>(uunits, 1) * 8));
  BGPU_TRY(alloc((void**)&seg_loc, (uint64_t)panels * g * 4));
  BGPU_CUDA(cudaMemsetAsync(m->xt_data, 0, std::max<uint64_t>(uunits, 1) * 8, s));
  BGPU_CUDA(cudaMemcpyAsync(m->xt_pgrp, pgrp.data(), (panels + 1) * 4ull,
                            cudaMemcpyHostToDevice, s));
  BGPU_CUDA(cudaMemcpyAsync(m->xt_esc_base, pesc.data(), (panels + 1) * 4ull,
                            cudaMemcpyHostToDevice, s));
  BGPU_CUDA(cudaMemcpyAsync(pu, punit.data(), panels * 4ull, cudaMemcpyHostToDevice, s));
  k_xt_struct<<<panels, 256, 0, s>>>(seg_len, order, g, m->xt_pgrp, pu, m->xt_grp,
                                     m->xt_units, m->xt_gene, seg_loc);
  BGPU_CHECK_LAUNCH();
  {
    const size_t smem = (size_t)kSellWarps * g * 4;
    if (smem > 48 * 1024) BGPU_CUDA(allow_max_smem(k_xt_scatter));
    k_xt_scatter<<<panels, kSellThreads, smem, s>>>(m->rowptr, m->csr_packed, n, g, P,
                                                     seg_loc, m->xt_esc_base,
                                                     reinterpret_cast<uint16_t*>(m->xt_data),
                                                     m->xt_esc);
    BGPU_CHECK_LAUNCH();
  }
  BGPU_CUDA(cudaStreamSynchronize(s));  // host vectors above are temporaries
  m->num_panels = ctas;  // rows of the per-CTA partials
  m->sell = true;
  *built = true;
  return BGPU_OK;
}

XvView xv_view(const Matrix& m) {
  XvView v = m.xv;
  v.data = m.xv_data;
  v.grp = m.xv_grp;
  v.units = m.xv_units;
  v.perm = m.xv_perm;
  v.isf = m.xv_isf;
  v.post = m.xv_post;
  v.esc_n = m.xv_esc_n;
  v.esc_base = m.xv_esc_base;
  v.esc = m.xv_esc;
  return v;
}

XtView xt_view(const Matrix& m) {
  XtView v = m.xt;
  v.data = m.xt_data;
  v.grp = m.xt_grp;
  v.units = m.xt_units;
  v.gene = m.xt_gene;
  v.pgrp = m.xt_pgrp;
  v.esc_base = m.xt_esc_base;
  v.esc = m.xt_esc;
  v.isf = m.isf;
  v.post = m.post;
  return v;
}

static size_t xv_smem_bytes(uint32_t g) {
  return (((size_t)g + 3) / 4 * 4 + (size_t)kSellThreads * kTabStride) * 4;
}

uint32_t xv_sell_ctas(const Matrix& m) {
  const uint64_t want = ceil_div(m.xv.groups, kSellWarps);
  return (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>(want, (uint64_t)num_sms() * kXvCtasPerSm));
}

uint32_t xt_sell_ctas(const Matrix& m) { return m.xt.panels ? m.xt.ctas : 1u; }

int launch_xv_sell(const Matrix& m, const float* v, const float* sd, float* y,
                   cudaStream_t s) {
  const XvView X = xv_view(m);
  const size_t smem = xv_smem_bytes(m.g);
  if (smem > 48 * 1024) BGPU_CUDA(allow_max_smem(k_xv_sell));
  k_xv_sell<<<xv_sell_ctas(m), kSellThreads, smem, s>>>(X, v, sd, y);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_xv_sell_multi(const TaskList<XvTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  uint32_t g = 0;
  for (uint32_t i = 0; i < L.count; ++i) g = std::max(g, L.t[i].X.g);
  const size_t smem = xv_smem_bytes(g);
  if (smem > 48 * 1024) BGPU_CUDA(allow_max_smem(k_xv_sell_multi));
  k_xv_sell_multi<<<L.grid(), kSellThreads, smem, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_xt_sell_multi(const TaskList<XtTask>& L, cudaStream_t s) {
  if (L.count == 0) return BGPU_OK;
  size_t smem = 0;
  for (uint32_t i = 0; i < L.count; ++i) {
    const XtView& X = L.t[i].X;
    smem = std::max(smem, xt_smem_bytes(X.P, X.g, X.esc_max, false));
  }
  BGPU_CUDA(allow_max_smem(k_xt_sell_multi));
  k_xt_sell_multi<<<L.grid(), kSellThreads, smem, s>>>(L);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_xt_sell(const Matrix& m, const float* u, const float* u_scale, float* u_out,
                   float* partT, cudaStream_t s) {
  const XtView X = xt_view(m);
  const size_t smem = xt_smem_bytes(X.P, X.g, X.esc_max, false);
  BGPU_CUDA(allow_max_smem(k_xt_sell<false>));
  k_xt_sell<false><<<X.panels ? m.xt.ctas : 1, kSellThreads, smem, s>>>(
      X, u, u_scale, u_out, partT, nullptr);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

int launch_xt_moments(const Matrix& m, double* partials, cudaStream_t s) {
  const XtView X = xt_view(m);
  const size_t smem = xt_smem_bytes(X.P, X.g, X.esc_max, true);
  BGPU_CUDA(allow_max_smem(k_xt_sell<true>));
  k_xt_sell<true><<<m.xt.ctas, kSellThreads, smem, s>>>(X, nullptr, nullptr, nullptr,
                                                        nullptr, (double2*)partials);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
