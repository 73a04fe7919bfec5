// X^T.u (brisc/pca.pyx:478-511) on a compact 16-bit copy of the transposed
// panels (counts mode, genes <= 2048, row panels of 1024 rows): half the
// bytes of the 32-bit packed words and twice the entries per 16-byte load.
//
//   csc16 entry:  head << 15 | row << 5 | code   (head: first entry of a
//                 (panel, gene) segment; row: local row in the panel, 10 bits)
//   code: the count for counts 0..15; 16 (bit 4) marks a count >= 16, whose
//         exact value the 32-bit packed copy keeps. An iteration's escape
//         shows in the OR of its words (bit 4 of each half), and its escaped
//         entries are then valued from the 32-bit copy.
//
// The kernel is the warp-segmented panel stream of the 32-bit one with 16
// entries per lane per iteration (512 per warp), software-pipelined. (On the
// CSR side the 16-bit unpacking costs more instructions than the bytes save,
// so X.v stays on 32-bit words.) Sums keep a fixed order, so products are
// bit-identical from run to run.
#include <algorithm>

#include "matrix.cuh"
#include "tma.cuh"

namespace bgpu {
namespace {

constexpr uint32_t kEsc = 0x00100010u;  // escape bit of both 16-bit halves
constexpr int kTab16 = 16;
__host__ __device__ constexpr uint32_t r128b(uint32_t b) { return (b + 127u) & ~127u; }

// ---------------------------------------------------------------------------
constexpr int kR16Threads = 384;
constexpr int kR16Warps = kR16Threads / 32;
constexpr int kR16Rows = 1024;  // panel rows the 10-bit row field allows

constexpr int kStageLd = 33;  // per-warp [position][lane] staging, padded

struct Seg16Layout {
  uint32_t tab, cps, nz, misc, stage, total;
  __host__ __device__ Seg16Layout(uint32_t P, uint32_t g) {
    tab = 128;                              // mbarrier
    cps = tab + r128b(P * kTab16 * 4);      // table scaled by u: [count][row]
    nz = cps + r128b((g + 1) * 4);          // gene offsets, then per-gene sums
    misc = nz + r128b(g * 2);               // non-empty genes in order (u16)
    stage = misc + 128;                     // warp totals (above), then the
    total = stage + r128b(kR16Warps * 15 * kStageLd * 4);  // lanes' running sums
  }
};

__device__ __forceinline__ uint32_t lanemask_lt16() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ float scaled_u16(const CscView& X, const float* u,
                                            const float* u_scale, float scale, uint64_t r) {
  const float uu = u_scale ? u[r] * scale : u[r];
  return X.post ? uu * X.post[r] : uu;
}

__global__ void __launch_bounds__(kR16Threads, 2)
k_rmat_seg16(CscView X, const uint16_t* __restrict__ e16, const float* __restrict__ u,
             const float* __restrict__ u_scale, float* __restrict__ u_out,
             float* __restrict__ partT, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  const uint32_t P = 1u << X.pshift;
  const Seg16Layout L(P, X.g);
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
    const uint32_t tb = P * kTab16 * 4;
    mbar_arrive_expect_tx(&bar[0], tb);
    bulk_g2s(smem + L.tab, X.rtab + (uint64_t)p * kTab16 * P, tb, &bar[0]);
  }
  const float scale = u_scale ? *u_scale : 1.f;
  constexpr int kPer = (kR16Rows + kR16Threads - 1) / kR16Threads;
  float usr[kPer];
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const uint32_t i = threadIdx.x + k * kR16Threads;
    float us = 0.f;
    if (i < rows) {
      if (u_out) u_out[r0 + i] = u_scale ? u[r0 + i] * scale : u[r0 + i];
      us = scaled_u16(X, u, u_scale, scale, r0 + i);
    }
    usr[k] = us;
  }
  const int32_t* cp = X.colptr + (uint64_t)p * (X.g + 1);
  for (uint32_t c = threadIdx.x; c <= X.g; c += kR16Threads) cps[c] = cp[c];
  __syncthreads();

  // Non-empty genes of the panel, in gene order.
  uint32_t S = 0;
  for (uint32_t base = 0; base < X.g; base += kR16Threads) {
    const uint32_t c = base + threadIdx.x;
    const bool f = c < X.g && cps[c + 1] > cps[c];
    const uint32_t bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) wtot[wid] = __popc(bal);
    __syncthreads();
    uint32_t before = 0, tot = 0;
#pragma unroll
    for (int j = 0; j < kR16Warps; ++j) {
      const uint32_t t = (uint32_t)wtot[j];
      before += j < wid ? t : 0u;
      tot += t;
    }
    if (f) nz[S + before + __popc(bal & lanemask_lt16())] = (uint16_t)c;
    S += tot;
    __syncthreads();
  }
  const uint32_t W = (uint32_t)cps[X.g];

  const bool ok = __syncthreads_and(mbar_wait(&bar[0], 0, err));
  if (!ok) return;  // every thread waited (bounded) for the copy
#pragma unroll
  for (int k = 0; k < kPer; ++k) {
    const uint32_t i = threadIdx.x + k * kR16Threads;
    if (i < P)
#pragma unroll
      for (int c = 1; c < kTab16; ++c) ut[c * P + i] *= usr[k];
  }

  auto first_at = [&](uint64_t t) {  // first ordinal whose segment starts >= t
    uint32_t lo = 0, hi = S;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if ((uint64_t)cps[nz[mid]] < t) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  const uint32_t i0 = first_at((uint64_t)W * wid / kR16Warps);
  const uint32_t i1 = wid == kR16Warps - 1 ? S : first_at((uint64_t)W * (wid + 1) / kR16Warps);
  const uint32_t s0 = i0 < S ? (uint32_t)cps[nz[i0]] : W;
  const uint32_t s1 = i1 < S ? (uint32_t)cps[nz[i1]] : W;
  __syncthreads();  // cps is no longer read: its space holds the gene sums
  for (uint32_t c = threadIdx.x; c < X.g; c += kR16Threads) gsum[c] = 0.f;
  __syncthreads();

  const int64_t pbase = X.rowptr[r0];
  const int64_t beg = pbase + s0, end = pbase + s1;
  const uint32_t pshift = X.pshift;
  const uint32_t lt = lanemask_lt16();
  float* stg = reinterpret_cast<float*>(smem + L.stage) + wid * 15 * kStageLd + lane;
  float carry = 0.f;
  uint32_t kb = 0;
  const uint4 z4 = make_uint4(0, 0, 0, 0);
  uint4 qa = z4, qb = z4;
  {
    const int64_t wb0 = (beg & ~7ll) + 16 * lane;
    if (wb0 < end) {
      qa = ld_stream_u4(e16 + wb0);
      qb = ld_stream_u4(e16 + wb0 + 8);
    }
  }
  for (int64_t b = beg & ~7ll; b < end; b += 512) {
    const int64_t wb = b + 16 * lane;
    uint4 na = z4, nb = z4;  // next iteration's 32 bytes, in flight meanwhile
    if (wb + 512 < end) {
      na = ld_stream_u4(e16 + wb + 512);
      nb = ld_stream_u4(e16 + wb + 520);
    }
    uint32_t wd[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
    qa = na;
    qb = nb;
    if (wb < beg || wb + 16 > end) {
#pragma unroll
      for (int i = 0; i < 16; ++i)
        if (wb + i < beg || wb + i >= end) wd[i >> 1] &= (i & 1) ? 0x0000FFFFu : 0xFFFF0000u;
    }
    float sl[16];
    uint32_t big = 0, hm = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint32_t e = (i & 1) ? (wd[i >> 1] >> 16) : (wd[i >> 1] & 0xffffu);
      hm |= (e >> 15) << i;
      sl[i] = ut[((e & 15u) << pshift) | ((e >> 5) & 1023u)];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) big |= wd[i];
    if (__any_sync(0xffffffffu, (big & kEsc) != 0u)) {
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint32_t e = (i & 1) ? (wd[i >> 1] >> 16) : (wd[i >> 1] & 0xffffu);
        if (e & 16u) {
          const uint32_t cnt = X.packed[wb + i] & 0xffffu;
          const uint64_t r = r0 + ((e >> 5) & 1023u);
          sl[i] = norm_count(cnt, X.isf[r]) * scaled_u16(X, u, u_scale, scale, r);
        }
      }
    }
    // in-lane segmented sums
#pragma unroll
    for (int i = 1; i < 16; ++i) sl[i] = ((hm >> i) & 1u) ? sl[i] : sl[i - 1] + sl[i];
    const uint32_t F = __ballot_sync(0xffffffffu, hm != 0u);
    float T = sl[15];
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
    const uint32_t h = __popc(hm);
    uint32_t hs = h;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, hs, d);
      if (lane >= d) hs += t;
    }
    const uint32_t kl = kb + hs - h;
    // a head closes the segment before it (the run's first head closes
    // nothing); each lane walks only its own heads, reading the running sum
    // before the head from its staging column
#pragma unroll
    for (int i = 0; i < 15; ++i) stg[i * kStageLd] = sl[i];
    __syncwarp();
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
    __syncwarp();
    carry = __shfl_sync(0xffffffffu, T, 31);
    kb += __shfl_sync(0xffffffffu, hs, 31);
  }
  if (lane == 0 && kb > 0) gsum[nz[i0 + kb - 1]] = carry;
  __syncthreads();
  for (uint32_t c = threadIdx.x; c < X.g; c += kR16Threads)
    partT[(uint64_t)c * X.num_panels + p] = gsum[c];
}

__global__ void k_compact16(const uint32_t* __restrict__ csc32, uint64_t nnz,
                            uint16_t* __restrict__ csc16) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= nnz) return;
  const uint32_t b = csc32[i];
  const uint32_t cb = b & 0xffffu;
  csc16[i] = (uint16_t)(((b >> 31) << 15) | (((b >> 16) & 0x3ffu) << 5) |
                        (cb < 16u ? cb : 16u));
}

}  // namespace

bool compact16_supported(const Matrix& m) {
  return m.stream_ok && m.g <= 2048 && m.P <= (uint32_t)kR16Rows &&
         Seg16Layout(m.P, m.g).total <= 220 * 1024;
}

int build_compact16(Matrix* m, cudaStream_t s, uint64_t* bytes_acc) {
  if (!compact16_supported(*m)) return BGPU_OK;
  const uint64_t n16 = round_up(m->nnz, 16) + 32;
  BGPU_CUDA(cudaMallocAsync((void**)&m->csc16, n16 * 2, s));
  *bytes_acc += n16 * 2;
  BGPU_CUDA(cudaMemsetAsync(m->csc16, 0, n16 * 2, s));
  if (m->nnz) {
    k_compact16<<<(unsigned)ceil_div(m->nnz, 256), 256, 0, s>>>(m->csc_packed, m->nnz,
                                                                 m->csc16);
    BGPU_CHECK_LAUNCH();
  }
  m->compact = true;
  return BGPU_OK;
}

int launch_rmatvec16(const Matrix& m, const float* u, const float* u_scale,
                     float* u_out, float* partT, int* err, cudaStream_t s) {
  const CscView X = csc_view(m);
  const size_t smem = Seg16Layout(m.P, m.g).total;
  BGPU_CUDA(allow_max_smem(k_rmat_seg16));
  k_rmat_seg16<<<m.num_panels, kR16Threads, smem, s>>>(X, m.csc16, u, u_scale, u_out,
                                                       partT, err);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

}  // namespace bgpu
