// Per-gene statistics for highly-variable-gene selection, the inputs of
// brisc's HVG step (brisc/hvg.pyx): gene means, variances and nonzero counts
// of the raw counts (gene_mean_and_variance_csr/_csc, hvg.pyx:9-252), and the
// per-gene sums and squared sums of counts clipped at a per-gene value
// (clipped_sum_csr/_csc, hvg.pyx:255-530).
//
// Exactness: every count is cast to uint64 as the reference casts it
// (`<unsigned long long> data[i]`), and the sums, squared sums and counts are
// integer sums, so their totals do not depend on the order of accumulation:
// shared-memory and global 64-bit atomics give the reference's integers
// exactly. The float outputs then follow the reference's expressions with
// every rounding written out (no contraction left to the compiler):
//   mean = float(sum) * inv_num_cells
//   var  = float(double(inv_num_pairs) * (double(n) * double(sumsq) -
//                                         double(sum) * double(sum)))
//   batch_counts_sum         = fma(float(out), clip, float(sum))
//   squared_batch_counts_sum = fma(float(out), clip * clip, float(sumsq))
// The last two are the forms the reference's -Ofast build computes (an FMA,
// and clip * clip associated first); the oracle's tests pin them against the
// compiled reference.
//
// Indices are checked: a gene or cell index outside its range, or an indptr
// that is not a valid range, sets an error word and the entry is skipped
// (the reference does not check; here the call returns BGPU_ERR_INVALID).
#include <algorithm>

#include "common.cuh"

namespace bgpu {
namespace {

enum : int { kMeanVar = 0, kClipped = 1 };

constexpr int kHvgThreads = 512;
// Genes whose three 64-bit accumulators fit one CTA's shared memory (96 KB,
// two CTAs per SM); larger gene counts accumulate in global memory.
constexpr uint32_t kHvgSmemGenes = 4096;

// `<unsigned long long> x` of the reference, per stored value type. Signed
// integers wrap modulo 2^64; floating values are truncated toward zero
// (counts are non-negative).
__device__ __forceinline__ unsigned long long as_u64(uint16_t x) { return x; }
__device__ __forceinline__ unsigned long long as_u64(uint32_t x) { return x; }
__device__ __forceinline__ unsigned long long as_u64(int32_t x) {
  return (unsigned long long)(long long)x;
}
__device__ __forceinline__ unsigned long long as_u64(int64_t x) {
  return (unsigned long long)x;
}
__device__ __forceinline__ unsigned long long as_u64(uint64_t x) { return x; }
__device__ __forceinline__ unsigned long long as_u64(float x) {
  return __float2ull_rz(x);
}
__device__ __forceinline__ unsigned long long as_u64(double x) {
  return __double2ull_rz(x);
}

// acc = [sum | sumsq | count] x g. kMeanVar: count = stored entries.
// kClipped: values above clip[gene] only count (hvg.pyx:298-303); the
// comparison converts the integer to float, as C's `value > clip_val[gene]`.
template <int MODE>
__device__ __forceinline__ void accumulate(unsigned long long* acc, uint32_t g,
                                           uint32_t gene, unsigned long long v,
                                           const float* __restrict__ clip) {
  if (MODE == kClipped && __ull2float_rn(v) > clip[gene]) {
    atomicAdd(acc + 2ull * g + gene, 1ull);
    return;
  }
  atomicAdd(acc + gene, v);
  atomicAdd(acc + (uint64_t)g + gene, v * v);
  if (MODE == kMeanVar) atomicAdd(acc + 2ull * g + gene, 1ull);
}

// CSR input. cells == nullptr: every stored entry in [e0, e1) (flat,
// grid-stride). cells != nullptr: warp per listed cell, lanes over its row.
// use_smem: per-CTA accumulators in shared memory, added to `acc` at the end.
template <typename V, typename I, int MODE>
__global__ void __launch_bounds__(kHvgThreads)
k_hvg_csr(const V* __restrict__ data, const I* __restrict__ indices,
          const I* __restrict__ indptr, uint64_t nnz, uint64_t num_rows,
          uint64_t e0, uint64_t e1, const int64_t* __restrict__ cells,
          uint64_t num_listed, uint32_t g, const float* __restrict__ clip,
          unsigned long long* __restrict__ acc, int use_smem,
          int* __restrict__ err) {
  extern __shared__ unsigned long long sacc[];
  if (use_smem) {
    for (uint32_t i = threadIdx.x; i < 3 * g; i += blockDim.x) sacc[i] = 0ull;
    __syncthreads();
  }
  unsigned long long* a = use_smem ? sacc : acc;
  auto entry = [&](uint64_t i) {
    const long long gene = (long long)indices[i];
    if (gene < 0 || gene >= (long long)g) {
      *err = 1;
      return;
    }
    accumulate<MODE>(a, g, (uint32_t)gene, as_u64(data[i]), clip);
  };
  if (cells == nullptr) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = e0 + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < e1;
         i += stride)
      entry(i);
  } else {
    const int lane = threadIdx.x & 31;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t j = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
         j < num_listed; j += nwarps) {
      const long long cell = cells[j];
      if (cell < 0 || (uint64_t)cell >= num_rows) {
        if (lane == 0) *err = 1;
        continue;
      }
      const long long b = (long long)indptr[cell], e = (long long)indptr[cell + 1];
      if (b < 0 || e < b || (uint64_t)e > nnz) {
        if (lane == 0) *err = 1;
        continue;
      }
      for (uint64_t i = (uint64_t)b + lane; i < (uint64_t)e; i += 32) entry(i);
    }
  }
  if (use_smem) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 3 * g; i += blockDim.x)
      if (sacc[i]) atomicAdd(acc + i, sacc[i]);
  }
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// CSC input: warp per gene, lanes over its entries, the cell mask applied
// when given; integer warp sums written straight to acc (no atomics).
template <typename V, typename I, int MODE>
__global__ void __launch_bounds__(kHvgThreads)
k_hvg_csc(const V* __restrict__ data, const I* __restrict__ indices,
          const I* __restrict__ indptr, uint64_t nnz, uint32_t g,
          const int8_t* __restrict__ mask, uint64_t mask_len,
          const float* __restrict__ clip, unsigned long long* __restrict__ acc,
          int* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t gene = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; gene < g;
       gene += nwarps) {
    const long long b = (long long)indptr[gene], e = (long long)indptr[gene + 1];
    unsigned long long s = 0, s2 = 0, c = 0;
    if (b < 0 || e < b || (uint64_t)e > nnz) {
      if (lane == 0) *err = 1;
    } else {
      const float cv = MODE == kClipped ? clip[gene] : 0.f;
      for (uint64_t i = (uint64_t)b + lane; i < (uint64_t)e; i += 32) {
        if (mask) {
          const long long cell = (long long)indices[i];
          if (cell < 0 || (uint64_t)cell >= mask_len) {
            *err = 1;
            continue;
          }
          if (!mask[cell]) continue;
        }
        const unsigned long long v = as_u64(data[i]);
        if (MODE == kClipped && __ull2float_rn(v) > cv) {
          ++c;
          continue;
        }
        s += v;
        s2 += v * v;
        if (MODE == kMeanVar) ++c;
      }
    }
    s = warp_sum_u64(s);
    s2 = warp_sum_u64(s2);
    c = warp_sum_u64(c);
    if (lane == 0) {
      acc[gene] = s;
      acc[(uint64_t)g + gene] = s2;
      acc[2ull * g + gene] = c;
    }
  }
}

// hvg.pyx:66-70 / :246-250, every rounding explicit.
__global__ void k_hvg_mean_var(const unsigned long long* __restrict__ acc, uint32_t g,
                               uint64_t num_cells, float inv_num_cells,
                               float inv_num_pairs, float* __restrict__ mean,
                               float* __restrict__ var,
                               uint32_t* __restrict__ nonzero_count) {
  const uint32_t gene = blockIdx.x * blockDim.x + threadIdx.x;
  if (gene >= g) return;
  const unsigned long long s = acc[gene], s2 = acc[(uint64_t)g + gene];
  mean[gene] = __fmul_rn(__ull2float_rn(s), inv_num_cells);
  const double sd = __ull2double_rn(s);
  const double d = __dsub_rn(__dmul_rn(__ull2double_rn(num_cells), __ull2double_rn(s2)),
                             __dmul_rn(sd, sd));
  var[gene] = __double2float_rn(__dmul_rn((double)inv_num_pairs, d));
  nonzero_count[gene] = (uint32_t)acc[2ull * g + gene];
}

// hvg.pyx:320-325 / :393-399: the reference's -Ofast build computes these as
// fused multiply-adds, with clip * clip rounded first.
__global__ void k_hvg_clipped(const unsigned long long* __restrict__ acc, uint32_t g,
                              const float* __restrict__ clip,
                              float* __restrict__ batch_counts_sum,
                              float* __restrict__ squared_batch_counts_sum) {
  const uint32_t gene = blockIdx.x * blockDim.x + threadIdx.x;
  if (gene >= g) return;
  const float out = __ull2float_rn(acc[2ull * g + gene]), c = clip[gene];
  batch_counts_sum[gene] = __fmaf_rn(out, c, __ull2float_rn(acc[gene]));
  squared_batch_counts_sum[gene] =
      __fmaf_rn(out, __fmul_rn(c, c), __ull2float_rn(acc[(uint64_t)g + gene]));
}

}  // namespace
}  // namespace bgpu

namespace bgpu {
namespace {

struct Scratch {  // stream-ordered device buffer, freed on the same stream
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~Scratch() { if (p) cudaFreeAsync(p, s); }
  int alloc(size_t bytes, cudaStream_t stream) {
    s = stream;
    cudaError_t e = cudaMallocAsync(&p, std::max<size_t>(bytes, 16), stream);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error(std::string("cudaMalloc(") + std::to_string(bytes) +
                ") failed: " + cudaGetErrorString(e));
      return BGPU_ERR_ALLOC;
    }
    return BGPU_OK;
  }
};

size_t hvg_value_size(int t) {
  switch (t) {
    case BGPU_VALUE_U16: return 2;
    case BGPU_VALUE_U32: case BGPU_VALUE_I32: case BGPU_VALUE_F32: return 4;
    case BGPU_VALUE_I64: case BGPU_VALUE_U64: case BGPU_VALUE_F64: return 8;
    default: return 0;
  }
}

// `p` on the device: the caller's pointer, or a stream-ordered copy of the
// host array.
int stage(const void* src, size_t bytes, bool on_device, Scratch& buf,
          const void** out, cudaStream_t s) {
  if (on_device || src == nullptr) {
    *out = src;
    return BGPU_OK;
  }
  BGPU_TRY(buf.alloc(bytes, s));
  BGPU_CUDA(cudaMemcpyAsync(buf.p, src, bytes, cudaMemcpyHostToDevice, s));
  *out = buf.p;
  return BGPU_OK;
}

struct HvgArgs {
  const void* data;
  const void* indices;
  const void* indptr;
  const int64_t* cells;
  uint64_t num_listed;
  const int8_t* mask;
  uint64_t mask_len;
  uint64_t e0, e1;  // CSR flat range
  uint32_t g;       // genes accumulated
  const float* clip;
  unsigned long long* acc;
  int* err;
};

template <typename V, typename I, int MODE>
int launch_hvg_typed(const bgpu_hvg_input& in, const HvgArgs& a, cudaStream_t s) {
  const V* data = static_cast<const V*>(a.data);
  const I* idx = static_cast<const I*>(a.indices);
  const I* ptr = static_cast<const I*>(a.indptr);
  if (in.is_csr) {
    const bool smem = a.g <= kHvgSmemGenes;
    const size_t sm = smem ? 3ull * a.g * sizeof(unsigned long long) : 0;
    if (sm > 48 * 1024) BGPU_CUDA((allow_max_smem(k_hvg_csr<V, I, MODE>)));
    const uint64_t work = a.cells ? a.num_listed * 32 : a.e1 - a.e0;
    const uint64_t want = std::max<uint64_t>(1, (work + kHvgThreads - 1) / kHvgThreads);
    const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)num_sms() * 2);
    k_hvg_csr<V, I, MODE><<<grid, kHvgThreads, sm, s>>>(
        data, idx, ptr, in.nnz, in.num_major, a.e0, a.e1, a.cells, a.num_listed,
        a.g, a.clip, a.acc, smem ? 1 : 0, a.err);
  } else {
    const uint64_t want = std::max<uint64_t>(1, ((uint64_t)a.g * 32 + kHvgThreads - 1) /
                                                    kHvgThreads);
    const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)num_sms() * 4);
    k_hvg_csc<V, I, MODE><<<grid, kHvgThreads, 0, s>>>(
        data, idx, ptr, in.nnz, a.g, a.mask, a.mask_len, a.clip, a.acc, a.err);
  }
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

template <typename I, int MODE>
int launch_hvg_index(const bgpu_hvg_input& in, const HvgArgs& a, cudaStream_t s) {
  switch (in.value_type) {
    case BGPU_VALUE_U16: return launch_hvg_typed<uint16_t, I, MODE>(in, a, s);
    case BGPU_VALUE_U32: return launch_hvg_typed<uint32_t, I, MODE>(in, a, s);
    case BGPU_VALUE_I32: return launch_hvg_typed<int32_t, I, MODE>(in, a, s);
    case BGPU_VALUE_F32: return launch_hvg_typed<float, I, MODE>(in, a, s);
    case BGPU_VALUE_I64: return launch_hvg_typed<int64_t, I, MODE>(in, a, s);
    case BGPU_VALUE_U64: return launch_hvg_typed<uint64_t, I, MODE>(in, a, s);
    case BGPU_VALUE_F64: return launch_hvg_typed<double, I, MODE>(in, a, s);
  }
  set_error("unknown value_type");
  return BGPU_ERR_INVALID;
}

int64_t read_index(const void* p, int index_type, uint64_t i) {
  return index_type == BGPU_INDEX_I64 ? static_cast<const int64_t*>(p)[i]
                                      : static_cast<const int32_t*>(p)[i];
}

// Stages the inputs, accumulates the integer sums into acc (3 x g) and checks
// the kernels' error word. num_cells: as the reference's argument. For CSR
// without a cell list, mean/variance sums every stored entry
// (hvg.pyx:43-52) and the clipped sums every entry of rows [0, num_cells)
// (hvg.pyx:292-303); with a list, mean/variance takes its first num_cells
// cells (hvg.pyx:56-63) and the clipped sums all of them (hvg.pyx:305-314).
template <int MODE>
int hvg_accumulate(const bgpu_hvg_input* in, uint64_t num_cells, uint32_t g,
                   const float* clip_dev, Scratch& acc, cudaStream_t s) {
  const size_t vsz = hvg_value_size(in->value_type);
  BGPU_REQUIRE(vsz != 0, BGPU_ERR_INVALID, "unknown value_type");
  BGPU_REQUIRE(in->index_type == BGPU_INDEX_I32 || in->index_type == BGPU_INDEX_I64,
               BGPU_ERR_INVALID, "unknown index_type");
  BGPU_REQUIRE(in->nnz == 0 || (in->data && in->indices), BGPU_ERR_INVALID,
               "data and indices are required");
  const size_t isz = in->index_type == BGPU_INDEX_I64 ? 8 : 4;
  const bool dev = in->on_device != 0;
  BGPU_REQUIRE(in->indptr, BGPU_ERR_INVALID, "indptr is required");
  BGPU_REQUIRE(!in->is_csr || in->cell_mask == nullptr, BGPU_ERR_INVALID,
               "a CSR input takes cell_indices, not cell_mask");
  BGPU_REQUIRE(in->is_csr || in->cell_indices == nullptr, BGPU_ERR_INVALID,
               "a CSC input takes cell_mask, not cell_indices");
  if (!in->is_csr)
    BGPU_REQUIRE(g <= in->num_major, BGPU_ERR_INVALID,
                 "indptr has fewer genes than num_genes");

  HvgArgs a{};
  a.g = g;
  a.clip = clip_dev;
  uint64_t listed = 0;
  if (in->is_csr && in->cell_indices) {
    listed = MODE == kMeanVar ? num_cells : in->num_cell_indices;
    BGPU_REQUIRE(listed <= in->num_cell_indices, BGPU_ERR_INVALID,
                 "cell_indices holds fewer than num_cells cells");
  } else if (in->is_csr) {
    if (MODE == kMeanVar) {
      a.e0 = 0;
      a.e1 = in->nnz;
    } else {
      BGPU_REQUIRE(num_cells <= in->num_major, BGPU_ERR_INVALID,
                   "num_cells exceeds the rows of indptr");
      int64_t b = 0, e = 0;
      if (dev) {
        int64_t two[2] = {0, 0};
        const char* base = static_cast<const char*>(in->indptr);
        BGPU_CUDA(cudaMemcpyAsync(&two[0], base, isz, cudaMemcpyDeviceToHost, s));
        BGPU_CUDA(cudaMemcpyAsync(&two[1], base + num_cells * isz, isz,
                                  cudaMemcpyDeviceToHost, s));
        BGPU_CUDA(cudaStreamSynchronize(s));
        if (isz == 4) {  // the low words hold the int32 values (little endian)
          b = (int32_t)(uint32_t)two[0];
          e = (int32_t)(uint32_t)two[1];
        } else {
          b = two[0];
          e = two[1];
        }
      } else {
        b = read_index(in->indptr, in->index_type, 0);
        e = read_index(in->indptr, in->index_type, num_cells);
      }
      BGPU_REQUIRE(b >= 0 && e >= b && (uint64_t)e <= in->nnz, BGPU_ERR_INVALID,
                   "indptr is not a valid range");
      a.e0 = (uint64_t)b;
      a.e1 = (uint64_t)e;
    }
  }

  Scratch d_data, d_idx, d_ptr, d_cells, d_mask, d_err;
  BGPU_TRY(stage(in->data, in->nnz * vsz, dev, d_data, &a.data, s));
  BGPU_TRY(stage(in->indices, in->nnz * isz, dev, d_idx, &a.indices, s));
  BGPU_TRY(stage(in->indptr, (in->num_major + 1) * isz, dev, d_ptr, &a.indptr, s));
  const void* cells = nullptr;
  if (in->is_csr && in->cell_indices)
    BGPU_TRY(stage(in->cell_indices, listed * sizeof(int64_t), dev, d_cells, &cells, s));
  a.cells = static_cast<const int64_t*>(cells);
  a.num_listed = listed;
  const void* mask = nullptr;
  if (!in->is_csr && in->cell_mask)
    BGPU_TRY(stage(in->cell_mask, in->cell_mask_len, dev, d_mask, &mask, s));
  a.mask = static_cast<const int8_t*>(mask);
  a.mask_len = in->cell_mask_len;

  BGPU_TRY(acc.alloc(3ull * std::max<uint32_t>(g, 1) * sizeof(unsigned long long), s));
  BGPU_TRY(d_err.alloc(sizeof(int), s));
  a.acc = static_cast<unsigned long long*>(acc.p);
  a.err = static_cast<int*>(d_err.p);
  BGPU_CUDA(cudaMemsetAsync(acc.p, 0, 3ull * std::max<uint32_t>(g, 1) * 8, s));
  BGPU_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(int), s));
  if (g > 0 && (in->is_csr ? (a.cells ? listed > 0 : a.e1 > a.e0) : true)) {
    if (in->index_type == BGPU_INDEX_I64)
      BGPU_TRY((launch_hvg_index<int64_t, MODE>(*in, a, s)));
    else
      BGPU_TRY((launch_hvg_index<int32_t, MODE>(*in, a, s)));
  }
  int herr = 0;
  BGPU_CUDA(cudaMemcpyAsync(&herr, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  BGPU_REQUIRE(herr == 0, BGPU_ERR_INVALID,
               "a gene or cell index, or an indptr range, is out of bounds");
  return BGPU_OK;
}

}  // namespace
}  // namespace bgpu

using namespace bgpu;

extern "C" int bgpu_gene_mean_var(const bgpu_hvg_input* in, uint64_t num_cells,
                                  float* mean, float* var, uint32_t* nonzero_count,
                                  void* stream) {
  BGPU_REQUIRE(in && mean && var && nonzero_count, BGPU_ERR_INVALID,
               "bad gene mean/variance arguments");
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t g = in->num_genes;
  Scratch acc;
  BGPU_TRY(hvg_accumulate<kMeanVar>(in, num_cells, g, nullptr, acc, s));
  // float inv_num_cells = 1.0 / num_cells; inv_num_pairs_of_cells =
  // 1.0 / (num_cells * (num_cells - 1)), an integer product (hvg.pyx:24-25)
  const float inv_n = (float)(1.0 / (double)num_cells);
  const float inv_p = (float)(1.0 / (double)(num_cells * (num_cells - 1)));
  const bool dev = in->on_device != 0;
  Scratch o_mean, o_var, o_nz;
  float* dm = mean;
  float* dv = var;
  uint32_t* dn = nonzero_count;
  if (!dev) {
    BGPU_TRY(o_mean.alloc(g * 4ull, s));
    BGPU_TRY(o_var.alloc(g * 4ull, s));
    BGPU_TRY(o_nz.alloc(g * 4ull, s));
    dm = static_cast<float*>(o_mean.p);
    dv = static_cast<float*>(o_var.p);
    dn = static_cast<uint32_t*>(o_nz.p);
  }
  if (g > 0) {
    k_hvg_mean_var<<<(g + 255) / 256, 256, 0, s>>>(
        static_cast<const unsigned long long*>(acc.p), g, num_cells, inv_n, inv_p, dm,
        dv, dn);
    BGPU_CHECK_LAUNCH();
  }
  if (!dev && g > 0) {
    BGPU_CUDA(cudaMemcpyAsync(mean, dm, g * 4ull, cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaMemcpyAsync(var, dv, g * 4ull, cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaMemcpyAsync(nonzero_count, dn, g * 4ull, cudaMemcpyDeviceToHost, s));
  }
  BGPU_CUDA(cudaStreamSynchronize(s));
  return BGPU_OK;
}

extern "C" int bgpu_clipped_sum(const bgpu_hvg_input* in, uint64_t num_cells,
                                const float* clip_val, float* batch_counts_sum,
                                float* squared_batch_counts_sum, void* stream) {
  BGPU_REQUIRE(in && clip_val && batch_counts_sum && squared_batch_counts_sum,
               BGPU_ERR_INVALID, "bad clipped-sum arguments");
  cudaStream_t s = (cudaStream_t)stream;
  // genes: num_genes (CSR, num_dataset_genes) or the columns of indptr (CSC,
  // hvg.pyx:414)
  BGPU_REQUIRE(in->is_csr || in->num_major <= 0xFFFFFFFFull, BGPU_ERR_INVALID,
               "too many genes");
  const uint32_t g = in->is_csr ? in->num_genes : (uint32_t)in->num_major;
  const bool dev = in->on_device != 0;
  Scratch d_clip, o_b, o_s;
  const void* clip = nullptr;
  BGPU_TRY(stage(clip_val, g * 4ull, dev, d_clip, &clip, s));
  Scratch acc;
  BGPU_TRY(hvg_accumulate<kClipped>(in, num_cells, g, static_cast<const float*>(clip),
                                    acc, s));
  float* db = batch_counts_sum;
  float* ds = squared_batch_counts_sum;
  if (!dev) {
    BGPU_TRY(o_b.alloc(g * 4ull, s));
    BGPU_TRY(o_s.alloc(g * 4ull, s));
    db = static_cast<float*>(o_b.p);
    ds = static_cast<float*>(o_s.p);
  }
  if (g > 0) {
    k_hvg_clipped<<<(g + 255) / 256, 256, 0, s>>>(
        static_cast<const unsigned long long*>(acc.p), g, static_cast<const float*>(clip),
        db, ds);
    BGPU_CHECK_LAUNCH();
  }
  if (!dev && g > 0) {
    BGPU_CUDA(cudaMemcpyAsync(batch_counts_sum, db, g * 4ull, cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaMemcpyAsync(squared_batch_counts_sum, ds, g * 4ull,
                              cudaMemcpyDeviceToHost, s));
  }
  BGPU_CUDA(cudaStreamSynchronize(s));
  return BGPU_OK;
}
