// Restart rotation U <- U . Ub[:, :kc] (brisc/pca.pyx:1210-1215, the
// reference's matmul_nn_f_out of pca.pyx:578-616) on the 5th-generation tensor
// cores: tcgen05.mma with operands in shared memory and the accumulator in
// tensor memory (TMEM).
//
// Precision: 3 x BF16 split products accumulated in FP32. Each FP32 operand
// is split x = x1 + x2 + x3 with x1 = bf16(x), x2 = bf16(x - x1), x3 =
// bf16(x - x1 - x2) (round to nearest; both differences are exact in FP32),
// which carries 24 significant bits. Six kind::f16 MMAs per K step form
// x1y1 + x1y2 + x2y1 + x1y3 + x2y2 + x3y1; the dropped terms are below 2^-24
// relative per product and unbiased. The tensor pipe carries the arithmetic:
// the rotation's ~25 flop/byte would need ~170 TFLOP/s of FP32 to keep up
// with HBM.
//
// The tensor core's FP32 accumulation does not round to nearest: measured on
// GB300, a 100-term rotation of unit columns comes out 5e-7 to 8e-7 short in
// relative norm (4-6 ulp, always toward zero), where an FP32 FMA loop is
// unbiased. The restart applies the rotation to the same converged Ritz
// vectors every restart, so that shrinkage compounds (5e-5 relative
// singular-value error after the 69 restarts of the 1M-cell solve, 2.8e-7
// with an FP32 FMA rotation). Two measures keep the bias off the result:
//  - pivoted delta: an output column i whose rotation column is dominated by
//    one entry (|Ub[p, i]| >= 1/2; a converged Ritz vector's column is e_p up
//    to small mixing) is computed as U . (Ub[:, i] - sign e_p) on the tensor
//    cores plus sign U[:, p], added in the epilogue in FP32 (one
//    round-to-nearest add). The biased part then scales with the mixing,
//    not with the vector; a column that is exactly e_p is copied exactly;
//  - the five small cross products of every K step are accumulated first and
//    the x1y1 products last, so the small terms are not truncated against
//    large partial sums.
// The MMAs and the epilogue adds run in a fixed order: the result is the
// same on every run.
//
// Shape: persistent CTAs (one per SM, 512 threads) walk 128-row tiles of U.
// Ub's three parts are staged once per CTA; each tile of U is loaded with
// coalesced 32-byte row runs into registers, split and written in the
// canonical no-swizzle K-major layout (8-row x 16-byte core matrices of 8
// BF16, K-direction core stride LBO = 128 B, 8-row stride SBO = Kp/8 * 128
// B); one elected thread issues 6 * Kp/16 MMAs of M=128, N=Np, K=16 into one
// of two TMEM accumulators and commits them to that accumulator's mbarrier.
// While they run, the next tile's loads are in flight and all 16 warps drain
// the previous tile's accumulator (tcgen05.ld, 32 lanes x 8 columns per
// load) and store C column-major (128-byte runs per column).
//
// Subspaces beyond one staging (K > 112: the 10M-cell solve's m = 200) run
// in k_gemm_tc_pipe, which keeps B resident and streams A in K chunks of 16
// to 32 through a warp-specialised pipeline (producer warps: cp.async ring,
// split, stage; one MMA lane; epilogue warps), the small cross products and
// x1y1 in separate accumulators added in FP32 in the epilogue; output columns
// in chunks of 128.
//
// Every mbarrier wait is bounded (about 1 s of SM clock): on timeout the
// kernel records kDevErrTimeout, stops, frees its TMEM and returns.
#include <algorithm>

#include <cuda_bf16.h>

#include "dense.cuh"
#include "tma.cuh"

namespace bgpu {
namespace {

constexpr int kTcThreads = 512;
constexpr int kTcRows = 128;  // M of one MMA / rows per tile
constexpr uint32_t kTcChunkK = 112;  // K per staging (A and B halves in smem)
// the per-task packing of k_gemm_tc: <= 16 k groups, offsets below 2^16
static_assert(kTcChunkK <= 128, "k_gemm_tc packs k groups and offsets in 16 bits");
constexpr uint32_t kTcChunkN = 128;  // output columns per staging

struct TcLayout {  // three BF16 parts of the A tile and of B
  uint32_t a[3], b[3], total;
  __host__ __device__ TcLayout(uint32_t Kp, uint32_t Np) {
    a[0] = 1024;  // mbarrier + TMEM address slot live below
    for (int i = 1; i < 3; ++i) a[i] = a[i - 1] + kTcRows * Kp * 2;
    b[0] = a[2] + kTcRows * Kp * 2;
    for (int i = 1; i < 3; ++i) b[i] = b[i - 1] + Np * Kp * 2;
    total = b[2] + Np * Kp * 2;
  }
};

// Shared-memory matrix descriptor (tcgen05): start address, leading (K) and
// stride (8-row) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo,
                                              uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b,
                                         uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
      ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
      ::"r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// Split 8 floats into three BF16 parts (round to nearest at each stage; the
// differences are exact in FP32), packed 8 per 16 bytes in k order.
__device__ __forceinline__ void split8(const float (&x)[8], uint4 (&p)[3]) {
  uint32_t w[3][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float2 r = make_float2(x[2 * i], x[2 * i + 1]);
#pragma unroll
    for (int part = 0; part < 3; ++part) {
      const __nv_bfloat162 h = __float22bfloat162_rn(r);
      const float2 f = __bfloat1622float2(h);
      r = make_float2(r.x - f.x, r.y - f.y);
      w[part][i] = *reinterpret_cast<const uint32_t*>(&h);
    }
  }
#pragma unroll
  for (int part = 0; part < 3; ++part)
    p[part] = make_uint4(w[part][0], w[part][1], w[part][2], w[part][3]);
}

// Byte offset of element (row, 8*kg) in the core-matrix layout (16 bytes
// hold k = 8kg..8kg+7 of one row).
__device__ __forceinline__ uint32_t core_off(uint32_t row, uint32_t kg, uint32_t kq) {
  return ((row >> 3) * kq + kg) * 128u + (row & 7u) * 16u;
}

// 16 columns of two accumulators (lane = row), one wait for all 32 values.
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float (&va)[16],
                                            float (&vb)[16]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
      "%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
        "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
        "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(ta)
      : "memory");
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
      "%12,%13,%14,%15}, [%16];"
      : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(tb)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    va[i] = __uint_as_float(r[i]);
    vb[i] = __uint_as_float(r[16 + i]);
  }
}

// 16-byte asynchronous copy global -> shared, src_bytes (0-16) read and the
// rest zero-filled; both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)),
               "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}


// Tasks per thread when a tile's A values are staged in registers: one task
// is 8 consecutive k of one row (128 rows x Kp/8 tasks, Kp <= 112).
constexpr int kTcTasks = (kTcRows * 14 + kTcThreads - 1) / kTcThreads;

// Pivots of the delta form: for column i of Bm (K x ncols, ldb), p = the
// row of its largest |entry| (lowest row on ties); when |Bm[p, i]| >= 1/2,
// piv[i] = +-(p + 1) (the entry's sign) and D[:, i] = Bm[:, i] - sign e_p
// (exact in FP32), else piv[i] = 0 and D[:, i] = Bm[:, i]. D has ld = K.
// One warp per column.
__global__ void __launch_bounds__(256)
k_rot_pivots(const float* __restrict__ Bm, uint64_t ldb, uint32_t K, uint32_t ncols,
             float* __restrict__ D, int* __restrict__ piv) {
  const int lane = threadIdx.x & 31;
  const uint32_t col = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (col >= ncols) return;
  const float* b = Bm + (uint64_t)col * ldb;
  float best = -1.f;
  uint32_t arg = 0;
  for (uint32_t r = lane; r < K; r += 32) {
    const float a = fabsf(b[r]);
    if (a > best) { best = a; arg = r; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ob = __shfl_xor_sync(0xffffffffu, best, o);
    const uint32_t oa = __shfl_xor_sync(0xffffffffu, arg, o);
    if (ob > best || (ob == best && oa < arg)) { best = ob; arg = oa; }
  }
  const bool use = best >= 0.5f;
  const float sgn = b[arg] < 0.f ? -1.f : 1.f;
  for (uint32_t r = lane; r < K; r += 32)
    D[(uint64_t)col * K + r] = (use && r == arg) ? b[r] - sgn : b[r];
  if (lane == 0) piv[col] = use ? (sgn > 0.f ? (int)arg + 1 : -((int)arg + 1)) : 0;
}

// C = A . Bm, plus sign Apiv[:, p] for the columns with a pivot (piv may be
// null).
__global__ void __launch_bounds__(kTcThreads, 1)
k_gemm_tc(const float* __restrict__ A, uint64_t lda, uint64_t rows, uint32_t K,
          const float* __restrict__ Bm, uint64_t ldb, uint32_t ncols,
          float* __restrict__ C, uint64_t ldc, uint32_t Kp, uint32_t Np,
          uint32_t tmem_cols, int accumulate, const float* __restrict__ Apiv,
          const int* __restrict__ piv, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);  // two: one per accumulator
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 64);
  __shared__ int stop;
  __shared__ int spiv[kTcChunkN];  // pivot of each output column (0: none)
  __shared__ long long spoff[kTcChunkN];  // its source column's offset (-1: none)
  const TcLayout L(Kp, Np);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint32_t kq = Kp / 8;  // 16-byte K groups (8 BF16) per row
  const uint32_t ntask = kTcRows * kq;

  if (wid == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(tslot)), "r"(2u * tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(bars, 1);
    mbar_init(bars + 1, 1);
    fence_mbar_init();
    stop = 0;
  }
  for (uint32_t c = tid; c < kTcChunkN; c += kTcThreads) {
    const int pv = (piv && c < ncols) ? piv[c] : 0;
    spiv[c] = pv;
    spoff[c] = pv == 0 ? -1ll : (long long)(pv > 0 ? pv - 1 : -pv - 1) * (long long)lda;
  }
  // B operand (N x K, K-major): row n of it is column n of Bm.
  for (uint32_t t = tid; t < Np * kq; t += kTcThreads) {
    const uint32_t n = t / kq, kg = t % kq;
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t k = kg * 8 + j;
      x[j] = (n < ncols && k < K) ? Bm[(uint64_t)n * ldb + k] : 0.f;
    }
    uint4 p[3];
    split8(x, p);
#pragma unroll
    for (int part = 0; part < 3; ++part)
      *reinterpret_cast<uint4*>(smem + L.b[part] + core_off(n, kg, kq)) = p[part];
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = idesc_bf16(kTcRows, Np);
  const uint32_t sbo = kq * 128u;
  const uint32_t base = smem_u32(smem);

  // A tile values of one tile, in registers: task = (row group, k group, row
  // in group); 8 lanes read 8 consecutive rows of one column (32-byte runs).
  // A task's k group, row and destination are the same for every tile:
  // computed once and packed (bits 0-15 shared-memory offset, 16-19 k group,
  // 20-23 valid k count, 24-30 row in the tile; no task: 0xFFFFFFFF).
  float xa[kTcTasks][8];
  uint32_t t_meta[kTcTasks];
#pragma unroll
  for (int i = 0; i < kTcTasks; ++i) {
    const uint32_t t = tid + i * kTcThreads;
    const uint32_t rr = t & 7u, kg = (t >> 3) % kq, rg = (t >> 3) / kq;
    const uint32_t nk = kg * 8 >= K ? 0u : min(8u, K - kg * 8);
    t_meta[i] = t < ntask ? core_off(rg * 8 + rr, kg, kq) | (kg << 16) | (nk << 20) |
                                ((rg * 8 + rr) << 24)
                          : 0xFFFFFFFFu;
  }
  auto load_tile = [&](uint64_t row0) {
    const bool full = row0 + kTcRows <= rows;
#pragma unroll
    for (int i = 0; i < kTcTasks; ++i) {
      const uint32_t meta = t_meta[i];
      const uint32_t nk = meta == 0xFFFFFFFFu ? 0u : (meta >> 20) & 15u;
      const uint32_t row = (meta >> 24) & 127u;
      const float* src = A + (uint64_t)(((meta >> 16) & 15u) * 8u) * lda + row0 + row;
      const bool rok = full || row0 + row < rows;
#pragma unroll
      for (int j = 0; j < 8; ++j)
        xa[i][j] = (rok && (uint32_t)j < nk) ? src[(uint64_t)j * lda] : 0.f;
    }
  };

  const uint64_t ntiles = (rows + kTcRows - 1) / kTcRows;
  // Two accumulators: the MMAs of tile i run while the epilogue of tile
  // i - 1 drains the other one and the loads of tile i + 1 are in flight.
  // Iteration it waits for the MMAs of it - 1 (which frees the shared A
  // tile and completes that accumulator), stages and issues tile it, then
  // drains tile it - 1.
  const uint32_t q = wid & 3u, h = wid >> 2;
  const uint32_t quarter = Np / 4;  // columns per epilogue warp (<= 32)
  float pa[32];                     // signed pivot values of this thread's row
  auto prefetch_pivots = [&](uint64_t row0) {
    const uint64_t gr = row0 + q * 32 + lane;
    const bool rok = gr < rows;
    const float* ap = Apiv + gr;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const uint32_t c = h * quarter + j;  // < 128: spoff / spiv cover it
      const long long off = spoff[c];
      float a = 0.f;
      if ((uint32_t)j < quarter && off >= 0 && rok) {
        a = ap[off];
        if (spiv[c] < 0) a = -a;
      }
      pa[j] = a;
    }
  };
  // Epilogue: warp w reads TMEM lanes 32*(w%4).. (tile rows) and the columns
  // of quarter w/4; lane = row.
  auto epilogue = [&](uint64_t row0, uint32_t acc) {
    const uint64_t gr = row0 + q * 32 + lane;
    float* cp = C + (uint64_t)(h * quarter) * ldc + gr;  // column h * quarter
#pragma unroll
    for (uint32_t g8 = 0; g8 < 4; ++g8) {
      const uint32_t c0 = h * quarter + g8 * 8;
      if (g8 * 8 >= quarter) break;
      float v[8];
      tmem_ld8(acc + ((q * 32u) << 16) + c0, v);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (gr < rows && c0 + j < ncols) {
          const float val = v[j] + pa[g8 * 8 + j];  // pivot column, FP32 add
          *cp = accumulate ? *cp + val : val;  // K chunks add in order
        }
        cp += ldc;
      }
    }
  };
  uint32_t phases = 0u;  // bit b: the phase accumulator b's barrier waits for
  int pend = -1;  // accumulator whose MMAs are committed and not yet waited for
  uint64_t tile = blockIdx.x, prev = 0;
  if (tile < ntiles) load_tile(tile * kTcRows);
  for (uint32_t it = 0;; ++it) {
    const bool has_cur = tile < ntiles;
    if (it > 0) {  // the MMAs of tile `prev`
      const uint32_t pb = (it - 1) & 1u;
      const bool ok = mbar_wait(bars + pb, (phases >> pb) & 1u, err);
      if (__syncthreads_or(!ok)) {
        if (tid == 0) stop = 1;
        break;
      }
      phases ^= 1u << pb;
      pend = -1;
      tc_fence_after();
    }
    if (has_cur) {
#pragma unroll
      for (int i = 0; i < kTcTasks; ++i) {
        if (t_meta[i] != 0xFFFFFFFFu) {
          const uint32_t off = t_meta[i] & 0xFFFFu;
          uint4 p[3];
          split8(xa[i], p);
#pragma unroll
          for (int part = 0; part < 3; ++part)
            *reinterpret_cast<uint4*>(smem + L.a[part] + off) = p[part];
        }
      }
      fence_proxy_async_smem();  // generic-proxy writes -> tensor-core reads
      tc_fence_before();
      __syncthreads();
      const uint32_t acc = tmem + (it & 1u) * tmem_cols;
      if (tid == 0) {
        tc_fence_after();
        for (uint32_t ks = 0; ks < Kp / 16; ++ks) {
          const uint32_t off = ks * 256u;  // two 16-byte K groups per K=16 step
          uint64_t da[3], db[3];
#pragma unroll
          for (int part = 0; part < 3; ++part) {
            da[part] = smem_desc(base + L.a[part] + off, 128u, sbo);
            db[part] = smem_desc(base + L.b[part] + off, 128u, sbo);
          }
          // the small cross products first: x1y3 + x2y2 + x3y1 + x1y2 + x2y1
          mma_bf16(acc, da[0], db[2], idesc, ks > 0 ? 1u : 0u);
          mma_bf16(acc, da[1], db[1], idesc, 1u);
          mma_bf16(acc, da[2], db[0], idesc, 1u);
          mma_bf16(acc, da[0], db[1], idesc, 1u);
          mma_bf16(acc, da[1], db[0], idesc, 1u);
        }
        for (uint32_t ks = 0; ks < Kp / 16; ++ks) {  // then x1y1
          const uint32_t off = ks * 256u;
          mma_bf16(acc, smem_desc(base + L.a[0] + off, 128u, sbo),
                   smem_desc(base + L.b[0] + off, 128u, sbo), idesc, 1u);
        }
        mma_commit(bars + (it & 1u));
      }
      pend = (int)(it & 1u);
      // the next tile's loads fly while these MMAs run
      if (tile + gridDim.x < ntiles) load_tile((tile + gridDim.x) * kTcRows);
    }
    if (it > 0) epilogue(prev * kTcRows, tmem + ((it - 1) & 1u) * tmem_cols);
    if (!has_cur) break;
    prefetch_pivots(tile * kTcRows);  // for this tile's epilogue
    tc_fence_before();  // the epilogue's TMEM reads before the next barrier
    prev = tile;
    tile += gridDim.x;
  }
  __syncthreads();
  if (stop && pend >= 0) {
    // a committed group may still be outstanding: one more bounded wait
    // before the TMEM goes back
    (void)mbar_wait(bars + pend, (phases >> pend) & 1u, nullptr);
  }
  tc_fence_after();
  if (wid == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(2u * tmem_cols)
                 : "memory");
  }
}


// ---------------------------------------------------------------------------
// The pipelined rotation (K > 112).
constexpr int kTpRows = 128;          // M of one MMA / rows per tile
constexpr int kTpProducerWarps = 8;   // load, split and stage tiles of U
constexpr int kTpMmaWarp = kTpProducerWarps;  // one lane issues the MMAs
constexpr int kTpEpilogueWarps = 4;   // drain TMEM, one per 32-lane quarter
constexpr int kTpThreads = 32 * (kTpProducerWarps + 1 + kTpEpilogueWarps);
constexpr int kTpProducerThreads = 32 * kTpProducerWarps;
constexpr int kTpTasks = 2;           // 8-value split tasks per producer thread and chunk
constexpr uint32_t kTpChunkN = 128;   // output columns per launch: four accumulators
constexpr uint32_t kTpMaxKc = 32;     // K per staged chunk of a tile
constexpr int kTpRing = 4;            // FP32 chunks in flight (cp.async ring)
constexpr uint32_t kTpMaxK = 1024;
constexpr size_t kTpSmem = 227 * 1024;
static_assert(kTpRows * kTpMaxKc / 8 <= kTpTasks * kTpProducerThreads,
              "a chunk's split tasks fit the producer threads");

// Shared memory: barriers and the TMEM slot, B's three BF16 parts (resident),
// two buffers of the A chunk's three BF16 parts (K-major core matrices, read
// by the MMAs), and a ring of FP32 A chunks ([k][row], filled by cp.async).
struct TpLayout {
  uint32_t b[3], a[2][3], f[kTpRing], total;
  __host__ __device__ TpLayout(uint32_t Kp, uint32_t Np, uint32_t KC) {
    uint32_t o = 1024;
    for (int i = 0; i < 3; ++i) {
      b[i] = o;
      o += Np * Kp * 2;
    }
    for (int st = 0; st < 2; ++st)
      for (int i = 0; i < 3; ++i) {
        a[st][i] = o;
        o += kTpRows * KC * 2;
      }
    for (int r = 0; r < kTpRing; ++r) {
      f[r] = o;
      o += kTpRows * KC * 4;
    }
    total = o;
  }
};

// The producer warps' own barrier (named barrier 1).
__device__ __forceinline__ void producers_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kTpProducerThreads) : "memory");
}

// Bounded wait for phase `parity` of `bar` that gives up when another role has
// raised *stop; a timeout (~2^31 SM cycles) records the error word and
// raises *stop.
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity, volatile int* stop,
                                        int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  while (true) {
    if (*stop) return false;
    if (mbar_try_wait(bar, parity)) return true;
    if (clock64() - t0 > (2LL << 30)) {
      atomicOr(err, kDevErrTimeout);
      *stop = 1;
      return false;
    }
  }
}

// C = A . Bm, plus sign Apiv[:, p] for the columns with a pivot (piv may be
// null). Warp-specialised and pipelined: producer warps load a K chunk of a
// 128-row tile of A, split it and stage it in one of two shared buffers; the
// MMA lane issues that chunk's MMAs (the five small cross products into one
// accumulator, x1y1 into another) and commits; epilogue warps add the two
// accumulators and the pivot column in FP32 and store C, while the next
// tile's MMAs run into the other accumulator pair. mbarriers: a_full
// (producers -> MMA), a_empty (MMA commit -> producers), acc_full (MMA commit
// -> epilogue), acc_empty (epilogue -> MMA). Waits are bounded; a timeout
// records the error word, raises a stop flag every waiting role polls, and
// the MMA lane waits (bounded) for its last commit before TMEM is freed.
__global__ void __launch_bounds__(kTpThreads, 1)
k_gemm_tc_pipe(const float* __restrict__ A, uint64_t lda, uint64_t rows, uint32_t K,
          const float* __restrict__ Bm, uint64_t ldb, uint32_t ncols,
          float* __restrict__ C, uint64_t ldc, uint32_t Kp, uint32_t Np, uint32_t KC,
          uint32_t tmem_cols, int accumulate, const float* __restrict__ Apiv,
          const int* __restrict__ piv, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  uint64_t* a_full = bars;         // [2], one arrive per producer warp
  uint64_t* a_empty = bars + 2;    // [2], MMA commit
  uint64_t* acc_full = bars + 4;   // [2], MMA commit
  uint64_t* acc_empty = bars + 6;  // [2], one arrive per epilogue warp
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 128);
  __shared__ volatile int stop;
  __shared__ int spiv[kTpChunkN];         // pivot of each output column (0: none)
  __shared__ long long spoff[kTpChunkN];  // its source column's offset (-1: none)
  const TpLayout L(Kp, Np, KC);
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const uint32_t kq = Kp / 8;  // B's 16-byte K groups per row
  const uint32_t nch = (Kp + KC - 1) / KC;

  if (wid == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 ::"r"(smem_u32(tslot)), "r"(4u * tmem_cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int b = 0; b < 2; ++b) {
      mbar_init(a_full + b, kTpProducerWarps);
      mbar_init(a_empty + b, 1);
      mbar_init(acc_full + b, 1);
      mbar_init(acc_empty + b, kTpEpilogueWarps);
    }
    fence_mbar_init();
    stop = 0;
  }
  for (uint32_t c = tid; c < kTpChunkN; c += kTpThreads) {
    const int pv = (piv && c < ncols) ? piv[c] : 0;
    spiv[c] = pv;
    spoff[c] = pv == 0 ? -1ll : (long long)(pv > 0 ? pv - 1 : -pv - 1) * (long long)lda;
  }
  // B operand (N x K, K-major): row n of it is column n of Bm.
  for (uint32_t t = tid; t < Np * kq; t += kTpThreads) {
    const uint32_t n = t / kq, kg = t % kq;
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t k = kg * 8 + j;
      x[j] = (n < ncols && k < K) ? Bm[(uint64_t)n * ldb + k] : 0.f;
    }
    uint4 p[3];
    split8(x, p);
#pragma unroll
    for (int part = 0; part < 3; ++part)
      *reinterpret_cast<uint4*>(smem + L.b[part] + core_off(n, kg, kq)) = p[part];
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint64_t ntiles = (rows + kTpRows - 1) / kTpRows;
  const uint64_t my_tiles =
      blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

  auto wait = [&](uint64_t* bar, uint32_t parity) -> bool {
    return tc_wait(bar, parity, &stop, err);
  };

  if (wid < kTpProducerWarps) {
    // ---- producers: stage s = (tile ti, chunk c), BF16 buffer s & 1 --------
    // Each chunk (KC columns of 128 rows of A) is copied with cp.async into
    // ring slot s % kTpRing, kTpRing - 1 chunks ahead; then split from there
    // (task = 8 consecutive k of one row) into the BF16 buffer. Decisions that
    // end the loop are taken by thread 0 and shared through the producers'
    // barrier, so every producer thread reaches every barrier.
    __shared__ int pgo;
    // a warp's 32 lanes take 32 consecutive rows of one k group: their reads
    // of the ring ([k][row]) fall on 32 different banks
    const uint32_t wf = KC / 8, wl = (Kp - (nch - 1) * KC) / 8;
    uint32_t mf[kTpTasks], ml[kTpTasks];  // row | k group << 8 | 1 << 16 (0: none)
#pragma unroll
    for (int i = 0; i < kTpTasks; ++i) {
      const uint32_t t = tid + i * kTpProducerThreads;
      mf[i] = t < kTpRows * wf ? (((t >> 5) / wf) * 32 + (t & 31u)) |
                                     (((t >> 5) % wf) << 8) | (1u << 16)
                               : 0u;
      ml[i] = t < kTpRows * wl ? (((t >> 5) / wl) * 32 + (t & 31u)) |
                                     (((t >> 5) % wl) << 8) | (1u << 16)
                               : 0u;
    }
    const uint64_t S = my_tiles * nch;
    auto issue = [&](uint64_t st) {  // ring slot st % kTpRing <- chunk st
      const uint64_t ti = st / nch;
      const uint32_t c = (uint32_t)(st % nch);
      const uint64_t row0 = (blockIdx.x + ti * gridDim.x) * kTpRows;
      float* ring = reinterpret_cast<float*>(smem + L.f[st % kTpRing]);
      const uint32_t w = min(KC, Kp - c * KC);
      for (uint32_t e = tid; e < w * 32u; e += kTpProducerThreads) {
        const uint32_t kl = e >> 5, r4 = (e & 31u) * 4u;
        const uint32_t k = c * KC + kl;
        const uint64_t gr = row0 + r4;
        const uint32_t nb = (k < K && gr < rows) ? (uint32_t)min_u64(16, (rows - gr) * 4) : 0u;
        cp_async16(ring + kl * kTpRows + r4, nb ? A + (uint64_t)k * lda + gr : A, nb);
      }
    };
    for (int s0 = 0; s0 < kTpRing - 1; ++s0) {
      if ((uint64_t)s0 < S) issue(s0);
      cp_async_commit();
    }
    for (uint64_t st = 0; st < S; ++st) {
      if (st + kTpRing - 1 < S) issue(st + kTpRing - 1);
      cp_async_commit();
      cp_async_wait<kTpRing - 1>();  // this thread's copies of chunk st landed
      const uint32_t b = (uint32_t)(st & 1u);
      if (tid == 0)
        pgo = (st < 2 || wait(a_empty + b, (uint32_t)(((st >> 1) - 1) & 1u))) ? 1 : 0;
      producers_sync();  // every copy of chunk st visible; BF16 buffer b free
      if (!pgo) break;
      const uint32_t c = (uint32_t)(st % nch);
      const bool last = c == nch - 1;
      const uint32_t wq = last ? wl : wf;
      const float* ring = reinterpret_cast<const float*>(smem + L.f[st % kTpRing]);
#pragma unroll
      for (int i = 0; i < kTpTasks; ++i) {
        const uint32_t m = last ? ml[i] : mf[i];
        if (m) {
          const uint32_t row = m & 255u, kg = (m >> 8) & 255u;
          float x[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) x[j] = ring[(kg * 8 + j) * kTpRows + row];
          uint4 p[3];
          split8(x, p);
          const uint32_t off = core_off(row, kg, wq);
#pragma unroll
          for (int part = 0; part < 3; ++part)
            *reinterpret_cast<uint4*>(smem + L.a[b][part] + off) = p[part];
        }
      }
      fence_proxy_async_smem();  // generic-proxy writes -> tensor-core reads
      __syncwarp();
      if (lane == 0) mbar_arrive(a_full + b);
      producers_sync();  // ring slot st % kTpRing is read: it may be refilled
    }
    asm volatile("cp.async.wait_all;" ::: "memory");  // no copy outlives the CTA
  } else if (wid == kTpMmaWarp) {
    // ---- MMA lane --------------------------------------------------------------
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16(kTpRows, Np);
      const uint32_t sbo_b = kq * 128u;
      const uint32_t base = smem_u32(smem);
      uint64_t* last_bar = nullptr;
      uint32_t last_par = 0;
      uint64_t st = 0;
      bool ok = true;
      for (uint64_t i = 0; i < my_tiles && ok; ++i) {
        const uint32_t ab = (uint32_t)(i & 1u);
        const uint32_t acc_s = tmem + 2u * ab * tmem_cols, acc_b = acc_s + tmem_cols;
        if (i >= 2 && !wait(acc_empty + ab, (uint32_t)(((i >> 1) - 1) & 1u))) break;
        for (uint32_t c = 0; c < nch; ++c, ++st) {
          const uint32_t b = (uint32_t)(st & 1u);
          if (!wait(a_full + b, (uint32_t)((st >> 1) & 1u))) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t k0 = c * KC, w = min(KC, Kp - k0), sbo_a = (w / 8) * 128u;
          for (uint32_t ks = 0; ks < w / 16; ++ks) {
            const uint32_t offa = ks * 256u, offb = (k0 / 16 + ks) * 256u;
            uint64_t da[3], db[3];
#pragma unroll
            for (int part = 0; part < 3; ++part) {
              da[part] = smem_desc(base + L.a[b][part] + offa, 128u, sbo_a);
              db[part] = smem_desc(base + L.b[part] + offb, 128u, sbo_b);
            }
            const uint32_t acc0 = (c == 0 && ks == 0) ? 0u : 1u;
            // the small cross products: x1y3 + x2y2 + x3y1 + x1y2 + x2y1
            mma_bf16(acc_s, da[0], db[2], idesc, acc0);
            mma_bf16(acc_s, da[1], db[1], idesc, 1u);
            mma_bf16(acc_s, da[2], db[0], idesc, 1u);
            mma_bf16(acc_s, da[0], db[1], idesc, 1u);
            mma_bf16(acc_s, da[1], db[0], idesc, 1u);
            mma_bf16(acc_b, da[0], db[0], idesc, acc0);  // x1y1
          }
          mma_commit(a_empty + b);  // the buffer is free once these complete
          last_bar = a_empty + b;
          last_par = (uint32_t)((st >> 1) & 1u);
          if (c == nch - 1) mma_commit(acc_full + ab);
        }
      }
      // every committed MMA completes before TMEM is freed
      if (last_bar) (void)mbar_wait(last_bar, last_par, nullptr);
    }
  } else {
    // ---- epilogue: warp quarter q reads TMEM lanes 32q.. (tile rows) ----------
    const uint32_t q = (uint32_t)wid & 3u;
    float pa[32], pb[32];
    auto pivots = [&](uint64_t row0, uint32_t c0, float (&pv)[32]) {
      const uint64_t gr = row0 + q * 32 + lane;
      const bool rok = gr < rows;
      const float* ap = Apiv + gr;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const uint32_t col = c0 + j;  // < Np <= 128: spoff / spiv cover it
        const long long off = col < ncols ? spoff[col] : -1ll;
        float a = 0.f;
        if (off >= 0 && rok) {
          a = ap[off];
          if (spiv[col] < 0) a = -a;
        }
        pv[j] = a;
      }
    };
    for (uint64_t i = 0; i < my_tiles; ++i) {
      const uint64_t row0 = (blockIdx.x + i * gridDim.x) * kTpRows;
      const uint64_t gr = row0 + q * 32 + lane;
      const uint32_t ab = (uint32_t)(i & 1u);
      pivots(row0, 0, pa);  // in flight while the MMAs finish
      // lane 0 waits and the warp follows its answer (tcgen05.ld needs every lane)
      const int ok = __shfl_sync(0xffffffffu,
                                 lane == 0 ? (int)wait(acc_full + ab, (uint32_t)((i >> 1) & 1u))
                                           : 0,
                                 0);
      if (!ok) break;
      tc_fence_after();
      const uint32_t t_s = tmem + 2u * ab * tmem_cols + ((q * 32u) << 16);
      const uint32_t t_b = t_s + tmem_cols;
      for (uint32_t g = 0; g < Np; g += 32) {
        if (g + 32 < Np) pivots(row0, g + 32, pb);  // the next group's loads fly
#pragma unroll
        for (uint32_t u = 0; u < 32; u += 16) {
          if (g + u < Np) {  // Np is a multiple of 32
            float vs[16], vb[16];
            tmem_ld16x2(t_s + g + u, t_b + g + u, vs, vb);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const uint32_t col = g + u + j;
              if (gr < rows && col < ncols) {
                const float val = (vs[j] + vb[j]) + pa[u + j];  // FP32, round to nearest
                float* cp = C + (uint64_t)col * ldc + gr;
                *cp = accumulate ? *cp + val : val;  // K chunks add in order
              }
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) pa[j] = pb[j];
      }
      tc_fence_before();  // the TMEM reads before the accumulators are reused
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_empty + ab);
    }
  }
  __syncthreads();
  tc_fence_after();
  if (wid == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 ::"r"(tmem), "r"(4u * tmem_cols)
                 : "memory");
  }
}

}  // namespace

bool gemm_tc_supported(uint32_t K, uint32_t ncols) {
  // one staging: the whole K (A tile and B in shared memory) and at most 128
  // output columns (the epilogue's four 32-column quarters)
  if (K == 0 || ncols == 0 || K > kTcChunkK || ncols > kTcChunkN) return false;
  const uint32_t Kp = (K + 15) & ~15u, Np = (ncols + 31) & ~31u;
  return TcLayout(Kp, Np).total <= 227 * 1024;
}

static int launch_tc_chunk(const float* A, uint64_t lda, uint64_t rows, uint32_t K,
                           const float* Bm, uint64_t ldb, uint32_t ncols, float* C,
                           uint64_t ldc, int accumulate, const float* Apiv,
                           const int* piv, int* err, cudaStream_t s) {
  const uint32_t Kp = (K + 15) & ~15u, Np = (ncols + 31) & ~31u;
  uint32_t tcols = 32;
  while (tcols < Np) tcols <<= 1;
  BGPU_REQUIRE(2 * tcols <= 512, BGPU_ERR_UNSUPPORTED,
               "tensor-core rotation: two accumulators must fit the 512 TMEM columns");
  // at least 120 KB so that one CTA (and one TMEM allocation) runs per SM
  const size_t smem = std::max<size_t>(TcLayout(Kp, Np).total, 120 * 1024);
  BGPU_CUDA(allow_max_smem(k_gemm_tc));
  const uint64_t ntiles = (rows + kTcRows - 1) / kTcRows;
  const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)num_sms());
  k_gemm_tc<<<grid, kTcThreads, smem, s>>>(A, lda, rows, K, Bm, ldb, ncols, C, ldc,
                                           Kp, Np, tcols, accumulate, Apiv, piv, err);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

// The widest K chunk (a multiple of 16, at most 32) whose layout fits one
// CTA's shared memory with B resident; 0 when none does.
static uint32_t tp_chunk_k(uint32_t Kp, uint32_t Np) {
  for (uint32_t kc = kTpMaxKc; kc >= 16; kc -= 16) {
    const uint32_t k = std::min(kc, Kp);
    if (TpLayout(Kp, Np, k).total <= kTpSmem) return k;
  }
  return 0;
}

static int launch_tp_chunk(const float* A, uint64_t lda, uint64_t rows, uint32_t K,
                           const float* Bm, uint64_t ldb, uint32_t ncols, float* C,
                           uint64_t ldc, int accumulate, const float* Apiv,
                           const int* piv, int* err, cudaStream_t s) {
  const uint32_t Kp = (K + 15) & ~15u, Np = (ncols + 31) & ~31u;
  const uint32_t KC = tp_chunk_k(Kp, Np);
  BGPU_REQUIRE(KC > 0 && ncols <= kTpChunkN, BGPU_ERR_UNSUPPORTED,
               "tensor-core rotation: operands do not fit shared memory");
  uint32_t tcols = 32;
  while (tcols < Np) tcols <<= 1;
  // at least 120 KB so that one CTA (and one TMEM allocation) runs per SM
  const size_t smem = std::max<size_t>(TpLayout(Kp, Np, KC).total, 120 * 1024);
  BGPU_CUDA(allow_max_smem(k_gemm_tc_pipe));
  const uint64_t ntiles = (rows + kTpRows - 1) / kTpRows;
  const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)num_sms());
  k_gemm_tc_pipe<<<grid, kTpThreads, smem, s>>>(A, lda, rows, K, Bm, ldb, ncols, C, ldc,
                                           Kp, Np, KC, tcols, accumulate, Apiv, piv, err);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

// One staging when the whole K and all output columns fit (K <= 112,
// ncols <= 256: the 1M-cell solve's m = 100); otherwise the pipelined kernel,
// output columns in chunks of <= 128 each reading all of K with B resident,
// and a K that does not fit even with 16-wide A chunks (beyond ~230) as K
// chunks of <= 128 added into C in chunk order (fixed, so the result is the
// same on every run), the first adding the pivot columns. The pipelined
// kernel stages A with cp.async: A's columns must start 16-byte aligned.
int launch_gemm_tc(const float* A, uint64_t lda, uint64_t rows, uint32_t K,
                   const float* Bm, uint64_t ldb, uint32_t ncols, float* C,
                   uint64_t ldc, float* dwork, int* piv, int* err, cudaStream_t s) {
  if (rows == 0 || ncols == 0) return BGPU_OK;
  BGPU_REQUIRE(K >= 1 && ncols <= K && K <= kTpMaxK, BGPU_ERR_UNSUPPORTED,
               "tensor-core rotation needs 1 <= ncols <= K <= 1024");
  BGPU_REQUIRE(dwork && piv, BGPU_ERR_INVALID, "tensor-core rotation needs its scratch");
  k_rot_pivots<<<(unsigned)ceil_div((uint64_t)ncols * 32, 256), 256, 0, s>>>(
      Bm, ldb, K, ncols, dwork, piv);
  BGPU_CHECK_LAUNCH();
  if (gemm_tc_supported(K, ncols))
    return launch_tc_chunk(A, lda, rows, K, dwork, K, ncols, C, ldc, 0, A, piv, err, s);
  BGPU_REQUIRE(((uintptr_t)A & 15u) == 0 && (lda & 3u) == 0, BGPU_ERR_UNSUPPORTED,
               "tensor-core rotation needs 16-byte aligned columns of A when K > 112");
  const uint32_t kchunk =
      tp_chunk_k((K + 15) & ~15u, (std::min(ncols, kTpChunkN) + 31) & ~31u) ? K : 128u;
  for (uint32_t n0 = 0; n0 < ncols; n0 += kTpChunkN) {
    const uint32_t nc = std::min(kTpChunkN, ncols - n0);
    for (uint32_t k0 = 0; k0 < K; k0 += kchunk) {
      const uint32_t kk = std::min(kchunk, K - k0);
      BGPU_TRY(launch_tp_chunk(A + (uint64_t)k0 * lda, lda, rows, kk,
                               dwork + (uint64_t)n0 * K + k0, K, nc,
                               C + (uint64_t)n0 * ldc, ldc, k0 > 0 ? 1 : 0, A,
                               k0 == 0 ? piv + n0 : nullptr, err, s));
    }
  }
  return BGPU_OK;
}

}  // namespace bgpu
