// Device layout construction: packed CSR, row-panel transposed copy, size
// factors, materialised normalisation and the stable CSR -> CSC transpose.
//
// The transpose follows the counting-sort structure of the reference's
// csr_tocsc (brisc/cysparse.pyx:1179-1295: per-worker column counts -> prefix
// sum -> stable scatter that keeps rows ascending inside each column), with the
// workers being fixed 256-row sub-blocks so the output never depends on the
// launch configuration.
#include <algorithm>
#include <vector>

#include "matrix.cuh"

namespace bgpu {

namespace {

constexpr int kSubRows = 256;  // rows per transpose sub-block (one warp each)

enum ErrBits : int {
  kErrIndex = 1,     // gene index outside [0, num_genes)
  kErrCount = 2,     // count not an integer in [0, 65535]
  kErrIndptr = 4,    // indptr decreasing or not ending at nnz
};

// Temporaries of the layout build: stream-ordered (no device-wide waits).
struct DevBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  ~DevBuf() { if (p) cudaFreeAsync(p, s); }
  int alloc(size_t bytes, cudaStream_t stream) {
    if (bytes == 0) bytes = 16;
    s = stream;
    cudaError_t e = cudaMallocAsync(&p, bytes, stream);
    if (e != cudaSuccess) {
      p = nullptr;
      set_error(std::string("cudaMalloc(") + std::to_string(bytes) +
                ") failed: " + cudaGetErrorString(e));
      return BGPU_ERR_ALLOC;
    }
    return BGPU_OK;
  }
};

// Persistent matrix arrays: stream-ordered on the matrix's creation stream
// (released on the same stream by matrix_free), so creating and destroying
// matrices never waits for other streams' work.
template <typename T>
int dev_alloc(T** out, size_t count, uint64_t* bytes_acc, cudaStream_t s) {
  size_t b = std::max<size_t>(count * sizeof(T), 16);
  cudaError_t e = cudaMallocAsync((void**)out, b, s);
  if (e != cudaSuccess) {
    *out = nullptr;
    set_error(std::string("cudaMalloc(") + std::to_string(b) +
              ") failed: " + cudaGetErrorString(e));
    return BGPU_ERR_ALLOC;
  }
  if (bytes_acc) *bytes_acc += b;
  return BGPU_OK;
}

size_t index_size(int t) { return t == BGPU_INDEX_I64 ? 8 : 4; }
size_t value_size(int t) { return t == BGPU_VALUE_U16 ? 2 : 4; }

// ---------------------------------------------------------------------------
// indptr -> int64 rowptr, with monotonicity check
template <typename I>
__global__ void k_rowptr(const I* __restrict__ indptr, int64_t* __restrict__ rowptr,
                         uint64_t n, uint64_t nnz, int* err) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  int64_t v = (int64_t)indptr[i];
  rowptr[i] = v;
  if (i == 0 && v != 0) atomicOr(err, kErrIndptr);
  if (i == n && v != (int64_t)nnz) atomicOr(err, kErrIndptr);
  if (i < n && (int64_t)indptr[i + 1] < v) atomicOr(err, kErrIndptr);
}

template <typename V>
__device__ __forceinline__ bool count_of(V x, uint32_t* c) {
  if constexpr (std::is_same<V, float>::value) {
    if (!(x >= 0.f && x <= 65535.f) || x != floorf(x)) return false;
    *c = (uint32_t)x;
    return true;
  } else if constexpr (std::is_same<V, int32_t>::value) {
    if (x < 0 || x > 65535) return false;
    *c = (uint32_t)x;
    return true;
  } else {
    if ((uint32_t)x > 65535u) return false;
    *c = (uint32_t)x;
    return true;
  }
}

// Pack CSR entries: one warp per row, grid-stride over rows.
template <typename I, typename V, bool kFloatMode>
__global__ void k_pack_csr(const int64_t* __restrict__ rowptr,
                           const I* __restrict__ indices,
                           const V* __restrict__ values, uint64_t n, uint32_t g,
                           uint32_t* __restrict__ packed, float* __restrict__ fval,
                           uint16_t* __restrict__ fcol, int* err) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  int e_local = 0;
  for (uint64_t r = warp; r < n; r += nwarps) {
    int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      int64_t c = (int64_t)indices[e];
      if (c < 0 || c >= (int64_t)g) { e_local |= kErrIndex; c = 0; }
      if constexpr (kFloatMode) {
        fval[e] = (float)values[e];
        fcol[e] = (uint16_t)c;
      } else {
        uint32_t cnt;
        if (!count_of(values[e], &cnt)) { e_local |= kErrCount; cnt = 0; }
        packed[e] = ((uint32_t)c << 16) | cnt;
      }
    }
  }
  if (e_local) atomicOr(err, e_local);
}

// Per-sub-block gene counts (integer atomics: order-independent).
template <typename C>
__global__ void k_sub_hist(const int64_t* __restrict__ rowptr,
                           const uint32_t* __restrict__ packed,
                           const uint16_t* __restrict__ fcol, uint64_t n,
                           uint32_t g, uint32_t num_sub, C* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const uint64_t s = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (s >= num_sub) return;
  uint64_t r0 = s * kSubRows, r1 = min_u64(n, r0 + kSubRows);
  int64_t e0 = rowptr[r0], e1 = rowptr[r1];
  C* my = cnt + s * (uint64_t)g;
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    uint32_t c = packed ? (packed[e] >> 16) : (uint32_t)fcol[e];
    atomicAdd(my + c, (C)1);
  }
}

// rowptr at every panel boundary (num_panels + 1 entries).
__global__ void k_panel_bounds(const int64_t* __restrict__ rowptr, uint64_t n,
                               uint32_t pshift, uint32_t num_panels,
                               int64_t* __restrict__ out) {
  uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > num_panels) return;
  uint64_t r = min_u64((uint64_t)p << pshift, n);
  out[p] = rowptr[r];
}

// Panel scan: per panel p (sub-blocks [s0, s1)), write
//   colptr[p][c] = sum_{c' < c} total(c')  (relative to the panel start)
// and turn cnt[s][c] into the first destination of sub-block s in gene c.
// base_off is added to every destination (0 for the panel layout; for the
// global CSC a single "panel" spans every sub-block).
template <typename C>
__global__ void k_panel_scan(C* __restrict__ cnt, C* __restrict__ colptr,
                             uint32_t g, uint32_t num_sub,
                             uint32_t subs_per_panel) {
  const uint32_t p = blockIdx.x;
  const uint32_t s0 = p * subs_per_panel;
  const uint32_t s1 = min(num_sub, s0 + subs_per_panel);
  C* cp = colptr + (uint64_t)p * (g + 1);
  // A: totals
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) {
    C t = 0;
    for (uint32_t s = s0; s < s1; ++s) t += cnt[(uint64_t)s * g + c];
    cp[c] = t;
  }
  __syncthreads();
  // B: exclusive scan over g + 1 entries, 1024 at a time with a carry
  __shared__ C warp_tot[32];
  __shared__ C carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint32_t base = 0; base <= g; base += blockDim.x) {
    uint32_t c = base + threadIdx.x;
    C v = (c < g) ? cp[c] : 0;
    C x = v;  // inclusive warp scan
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      C y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int nw = blockDim.x >> 5;
      C t = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        C y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < nw) warp_tot[lane] = t;
    }
    __syncthreads();
    C excl = carry + x - v + (wid > 0 ? warp_tot[wid - 1] : 0);
    C block_total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    if (c <= g) cp[c] = excl;
    if (threadIdx.x == 0) carry += block_total;
    __syncthreads();
  }
  // C: per-sub-block start offsets
  for (uint32_t c = threadIdx.x; c < g; c += blockDim.x) {
    C run = cp[c];
    for (uint32_t s = s0; s < s1; ++s) {
      C t = cnt[(uint64_t)s * g + c];
      cnt[(uint64_t)s * g + c] = run;
      run += t;
    }
  }
}

// Stable scatter: one warp per sub-block walks its rows in order; the lanes
// share a row's entries (distinct genes), so each gene's destination counter
// advances in row order. Destinations are panel-relative offsets plus the
// panel's first element.
template <typename C, int kOut>
__global__ void k_sub_scatter(const int64_t* __restrict__ rowptr,
                              const uint32_t* __restrict__ packed,
                              const float* __restrict__ fval,
                              const uint16_t* __restrict__ fcol, uint64_t n,
                              uint32_t g, uint32_t num_sub, uint32_t pshift,
                              C* __restrict__ cnt,
                              // kOut == 0: panel layout (packed counts)
                              uint32_t* __restrict__ out_packed,
                              // kOut == 1: panel layout (float values)
                              float* __restrict__ out_val,
                              uint16_t* __restrict__ out_row) {
  const int lane = threadIdx.x & 31;
  const uint64_t s = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (s >= num_sub) return;
  uint64_t r0 = s * kSubRows, r1 = min_u64(n, r0 + kSubRows);
  C* pos = cnt + s * (uint64_t)g;
  const uint64_t p = r0 >> pshift;
  const int64_t pbase = rowptr[p << pshift];
  for (uint64_t r = r0; r < r1; ++r) {
    int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
    const uint32_t lr = (uint32_t)(r - (p << pshift));
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      uint32_t c = packed ? (packed[e] >> 16) : (uint32_t)fcol[e];
      C slot = atomicAdd(pos + c, (C)1);
      int64_t dst = pbase + (int64_t)slot;
      if constexpr (kOut == 0) {
        out_packed[dst] = (lr << 16) | (packed[e] & 0xffffu);
      } else {
        out_val[dst] = fval[e];
        out_row[dst] = (uint16_t)lr;
      }
    }
    __syncwarp();
  }
}

__global__ void k_copy_float(const float* __restrict__ a, float* __restrict__ b,
                             uint64_t n) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

int grid_for(uint64_t work, int block, int cap = 1 << 20) {
  uint64_t g = ceil_div(work, (uint64_t)block);
  return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, (uint64_t)cap));
}

template <typename I>
int build_rowptr(Matrix* m, const void* indptr, int* d_err, cudaStream_t s) {
  k_rowptr<I><<<grid_for(m->n + 1, 256), 256, 0, s>>>(
      (const I*)indptr, m->rowptr, m->n, m->nnz, d_err);
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

template <typename I, typename V>
int pack_typed(Matrix* m, const void* idx, const void* val, int* d_err,
               cudaStream_t s) {
  int blocks = std::min<uint64_t>(ceil_div(m->n, 8), (uint64_t)num_sms() * 16);
  blocks = std::max(blocks, 1);
  if (m->mode == kFloat) {
    k_pack_csr<I, V, true><<<blocks, 256, 0, s>>>(
        m->rowptr, (const I*)idx, (const V*)val, m->n, m->g, nullptr,
        m->csr_val, m->csr_col, d_err);
  } else {
    k_pack_csr<I, V, false><<<blocks, 256, 0, s>>>(
        m->rowptr, (const I*)idx, (const V*)val, m->n, m->g, m->csr_packed,
        nullptr, nullptr, d_err);
  }
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

template <typename I>
int pack_by_value(Matrix* m, int vt, const void* idx, const void* val,
                  int* d_err, cudaStream_t s) {
  switch (vt) {
    case BGPU_VALUE_U16: return pack_typed<I, uint16_t>(m, idx, val, d_err, s);
    case BGPU_VALUE_U32: return pack_typed<I, uint32_t>(m, idx, val, d_err, s);
    case BGPU_VALUE_I32: return pack_typed<I, int32_t>(m, idx, val, d_err, s);
    default: return pack_typed<I, float>(m, idx, val, d_err, s);
  }
}

uint32_t choose_pshift(uint64_t n, uint32_t requested) {
  if (requested) {
    uint32_t p = 0;
    while ((1u << p) < requested) ++p;
    return p;
  }
  // 1024-row panels: the streaming X^T.u stages u and an 8-count table per
  // panel row in shared memory (36 KB), keeps two CTAs per SM, and a panel's
  // local row fits the 16-bit field of the packed entry.
  (void)n;
  return 10;
}

}  // namespace

int matrix_build(Matrix* m, const bgpu_matrix_desc* d, cudaStream_t s) {
  BGPU_REQUIRE(d != nullptr, BGPU_ERR_INVALID, "desc is NULL");
  BGPU_REQUIRE(d->num_cells >= 1 && d->num_genes >= 1, BGPU_ERR_INVALID,
               "num_cells and num_genes must be positive");
  BGPU_REQUIRE(d->num_genes <= 65536, BGPU_ERR_UNSUPPORTED,
               "num_genes must be <= 65536 (16-bit gene index layout)");
  BGPU_REQUIRE(d->index_type == BGPU_INDEX_I32 || d->index_type == BGPU_INDEX_I64,
               BGPU_ERR_INVALID, "index_type must be BGPU_INDEX_I32 or _I64");
  BGPU_REQUIRE(d->value_type >= BGPU_VALUE_U16 && d->value_type <= BGPU_VALUE_F32,
               BGPU_ERR_INVALID, "unknown value_type");
  BGPU_REQUIRE(d->norm_method >= BGPU_NORM_NONE && d->norm_method <= BGPU_NORM_PFLOG1PPF,
               BGPU_ERR_INVALID, "unknown norm_method");
  BGPU_REQUIRE(d->indptr && (d->nnz == 0 || (d->indices && d->values)),
               BGPU_ERR_INVALID, "indptr/indices/values must not be NULL");
  BGPU_REQUIRE((d->kernels & ~63u) == 0, BGPU_ERR_INVALID, "unknown BGPU_KERNELS_* bits");
  m->kernels = d->kernels;
  if (d->norm_method == BGPU_NORM_NONE) {
    BGPU_REQUIRE(d->value_type == BGPU_VALUE_F32, BGPU_ERR_INVALID,
                 "pre-normalised input (BGPU_NORM_NONE) must be float32");
  } else {
    BGPU_REQUIRE(d->inv_size_factors != nullptr, BGPU_ERR_INVALID,
                 "fused normalisation needs per-cell inverse size factors");
    BGPU_REQUIRE(d->norm_method != BGPU_NORM_PFLOG1PPF || d->post_factors,
                 BGPU_ERR_INVALID, "PFlog1pPF needs per-cell post factors");
  }
  if (d->panel_rows) {
    BGPU_REQUIRE((d->panel_rows & (d->panel_rows - 1)) == 0 &&
                     d->panel_rows >= 1024 && d->panel_rows <= 65536,
                 BGPU_ERR_INVALID,
                 "panel_rows must be a power of two in [1024, 65536]");
  }
  BGPU_REQUIRE(d->sell_panel_rows == 0 || (d->sell_panel_rows % 32 == 0 &&
                                          d->sell_panel_rows >= 128 &&
                                          d->sell_panel_rows <= 512),
               BGPU_ERR_INVALID, "sell_panel_rows must be 0 or a multiple of 32 in [128, 512]");
  m->sell_P = d->sell_panel_rows;
  BGPU_CUDA(cudaGetDevice(&m->device));
  m->stream = s;

  m->n = d->num_cells;
  m->g = d->num_genes;
  m->nnz = d->nnz;
  m->mode = d->norm_method == BGPU_NORM_NONE ? kFloat : kCounts;
  m->norm_method = d->norm_method;
  m->nnz_alloc = round_up(m->nnz, 4) + 4;
  m->pshift = choose_pshift(m->n, d->panel_rows);
  m->P = 1u << m->pshift;
  m->num_panels = (uint32_t)ceil_div(m->n, m->P);

  // Stage host inputs on the device.
  const size_t isz = index_size(d->index_type), vsz = value_size(d->value_type);
  DevBuf t_indptr, t_idx, t_val, t_isf, t_post, t_err;
  const void *indptr = d->indptr, *idx = d->indices, *val = d->values;
  const float *isf = d->inv_size_factors, *post = d->post_factors;
  if (!d->on_device) {
    // Host-side checks the device path does on the GPU.
    int64_t first, last;
    if (d->index_type == BGPU_INDEX_I64) {
      first = ((const int64_t*)indptr)[0];
      last = ((const int64_t*)indptr)[m->n];
    } else {
      first = ((const int32_t*)indptr)[0];
      last = ((const int32_t*)indptr)[m->n];
    }
    BGPU_REQUIRE(first == 0 && last == (int64_t)m->nnz, BGPU_ERR_INVALID,
                 "indptr must start at 0 and end at nnz");
    BGPU_TRY(t_indptr.alloc((m->n + 1) * isz, s));
    BGPU_CUDA(cudaMemcpyAsync(t_indptr.p, indptr, (m->n + 1) * isz,
                              cudaMemcpyHostToDevice, s));
    indptr = t_indptr.p;
    BGPU_TRY(t_idx.alloc(m->nnz * isz, s));
    BGPU_TRY(t_val.alloc(m->nnz * vsz, s));
    if (m->nnz) {
      BGPU_CUDA(cudaMemcpyAsync(t_idx.p, idx, m->nnz * isz,
                                cudaMemcpyHostToDevice, s));
      BGPU_CUDA(cudaMemcpyAsync(t_val.p, val, m->nnz * vsz,
                                cudaMemcpyHostToDevice, s));
    }
    idx = t_idx.p;
    val = t_val.p;
    if (isf) {
      BGPU_TRY(t_isf.alloc(m->n * 4, s));
      BGPU_CUDA(cudaMemcpyAsync(t_isf.p, isf, m->n * 4, cudaMemcpyHostToDevice, s));
      isf = (const float*)t_isf.p;
    }
    if (post && m->norm_method == BGPU_NORM_PFLOG1PPF) {
      BGPU_TRY(t_post.alloc(m->n * 4, s));
      BGPU_CUDA(cudaMemcpyAsync(t_post.p, post, m->n * 4, cudaMemcpyHostToDevice, s));
      post = (const float*)t_post.p;
    }
  }
  BGPU_TRY(t_err.alloc(sizeof(int), s));
  int* d_err = (int*)t_err.p;
  BGPU_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), s));

  // Persistent arrays.
  // rowptr, isf and post carry 4 padding entries: the streaming X.v copies
  // 16-byte-aligned slices of them that may end past the last row.
  BGPU_TRY(dev_alloc(&m->rowptr, m->n + 5, &m->bytes, s));
  BGPU_CUDA(cudaMemsetAsync(m->rowptr, 0, (m->n + 5) * 8, s));
  if (m->mode == kFloat) {
    BGPU_TRY(dev_alloc(&m->csr_val, m->nnz_alloc, &m->bytes, s));
    BGPU_TRY(dev_alloc(&m->csr_col, m->nnz_alloc, &m->bytes, s));
    BGPU_TRY(dev_alloc(&m->csc_val, m->nnz_alloc, &m->bytes, s));
    BGPU_TRY(dev_alloc(&m->csc_row, m->nnz_alloc, &m->bytes, s));
    BGPU_CUDA(cudaMemsetAsync(m->csr_val, 0, m->nnz_alloc * 4, s));
    BGPU_CUDA(cudaMemsetAsync(m->csr_col, 0, m->nnz_alloc * 2, s));
    BGPU_CUDA(cudaMemsetAsync(m->csc_val, 0, m->nnz_alloc * 4, s));
    BGPU_CUDA(cudaMemsetAsync(m->csc_row, 0, m->nnz_alloc * 2, s));
  } else {
    BGPU_TRY(dev_alloc(&m->csr_packed, m->nnz_alloc, &m->bytes, s));
    BGPU_TRY(dev_alloc(&m->csc_packed, m->nnz_alloc, &m->bytes, s));
    BGPU_CUDA(cudaMemsetAsync(m->csr_packed, 0, m->nnz_alloc * 4, s));
    BGPU_CUDA(cudaMemsetAsync(m->csc_packed, 0, m->nnz_alloc * 4, s));
    BGPU_TRY(dev_alloc(&m->isf, m->n + 4, &m->bytes, s));
    BGPU_CUDA(cudaMemsetAsync(m->isf, 0, (m->n + 4) * 4, s));
    k_copy_float<<<grid_for(m->n, 256), 256, 0, s>>>(isf, m->isf, m->n);
    BGPU_CHECK_LAUNCH();
    if (m->norm_method == BGPU_NORM_PFLOG1PPF) {
      BGPU_TRY(dev_alloc(&m->post, m->n + 4, &m->bytes, s));
      BGPU_CUDA(cudaMemsetAsync(m->post, 0, (m->n + 4) * 4, s));
      k_copy_float<<<grid_for(m->n, 256), 256, 0, s>>>(post, m->post, m->n);
      BGPU_CHECK_LAUNCH();
    }
  }
  // indptr is validated (and the stream synchronised) before any kernel
  // reads entries through it.
  if (d->index_type == BGPU_INDEX_I64)
    BGPU_TRY(build_rowptr<int64_t>(m, indptr, d_err, s));
  else
    BGPU_TRY(build_rowptr<int32_t>(m, indptr, d_err, s));
  {
    int herr = 0;
    BGPU_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaStreamSynchronize(s));
    BGPU_REQUIRE(!(herr & kErrIndptr), BGPU_ERR_INVALID,
                 "indptr must start at 0, be non-decreasing and end at nnz");
  }
  if (d->index_type == BGPU_INDEX_I64)
    BGPU_TRY(pack_by_value<int64_t>(m, d->value_type, idx, val, d_err, s));
  else
    BGPU_TRY(pack_by_value<int32_t>(m, d->value_type, idx, val, d_err, s));

  // Panel-relative offsets fit in int32 if every panel holds < 2^31 entries.
  std::vector<int64_t> panel_rp;
  {
    std::vector<int64_t> rp(m->num_panels + 1);
    DevBuf t_rp;
    BGPU_TRY(t_rp.alloc(rp.size() * 8, s));
    k_panel_bounds<<<grid_for(rp.size(), 256), 256, 0, s>>>(
        m->rowptr, m->n, m->pshift, m->num_panels, (int64_t*)t_rp.p);
    BGPU_CHECK_LAUNCH();
    BGPU_CUDA(cudaMemcpyAsync(rp.data(), t_rp.p, rp.size() * 8,
                              cudaMemcpyDeviceToHost, s));
    int herr = 0;
    BGPU_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaStreamSynchronize(s));
    if (herr & kErrIndptr) {
      set_error("indptr must start at 0, be non-decreasing and end at nnz");
      return BGPU_ERR_INVALID;
    }
    if (herr & kErrIndex) {
      set_error("a gene index is outside [0, num_genes)");
      return BGPU_ERR_INVALID;
    }
    if (herr & kErrCount) {
      set_error("fused normalisation needs integer counts in [0, 65535]");
      return BGPU_ERR_UNSUPPORTED;
    }
    for (uint32_t p = 0; p < m->num_panels; ++p)
      BGPU_REQUIRE(rp[p + 1] - rp[p] < (int64_t)INT32_MAX, BGPU_ERR_UNSUPPORTED,
                   "a row panel holds >= 2^31 entries; use a smaller panel_rows");
    panel_rp.swap(rp);
  }

  // Sliced-ELL layout for both products where it applies (counts, <= 4096
  // genes); the packed CSR words were only its source then.
  if (m->mode == kCounts && !(m->kernels & BGPU_KERNELS_PANELS)) {
    bool built = false;
    BGPU_TRY(build_sell(m, s, &built));
    if (built) {
      BGPU_CUDA(cudaFreeAsync(m->csr_packed, s));
      m->csr_packed = nullptr;
      m->bytes -= std::max<size_t>(m->nnz_alloc * 4, 16);
      BGPU_CUDA(cudaStreamSynchronize(s));  // temporaries are freed on return
      return BGPU_OK;
    }
  }

  // Transposed copy.
  BGPU_TRY(dev_alloc(&m->colptr, (size_t)m->num_panels * (m->g + 1), &m->bytes, s));
  const uint32_t num_sub = (uint32_t)ceil_div(m->n, kSubRows);
  const uint32_t subs_per_panel = m->P / kSubRows;
  DevBuf t_cnt;
  BGPU_TRY(t_cnt.alloc((size_t)num_sub * m->g * sizeof(int32_t), s));
  int32_t* cnt = (int32_t*)t_cnt.p;
  BGPU_CUDA(cudaMemsetAsync(cnt, 0, (size_t)num_sub * m->g * sizeof(int32_t), s));
  const int wblocks = (int)ceil_div(num_sub, 8);
  k_sub_hist<int32_t><<<wblocks, 256, 0, s>>>(m->rowptr, m->csr_packed, m->csr_col,
                                              m->n, m->g, num_sub, cnt);
  BGPU_CHECK_LAUNCH();
  k_panel_scan<int32_t><<<m->num_panels, 1024, 0, s>>>(cnt, m->colptr, m->g,
                                                       num_sub, subs_per_panel);
  BGPU_CHECK_LAUNCH();
  if (m->mode == kFloat) {
    k_sub_scatter<int32_t, 1><<<wblocks, 256, 0, s>>>(
        m->rowptr, nullptr, m->csr_val, m->csr_col, m->n, m->g, num_sub,
        m->pshift, cnt, nullptr, m->csc_val, m->csc_row);
  } else {
    k_sub_scatter<int32_t, 0><<<wblocks, 256, 0, s>>>(
        m->rowptr, m->csr_packed, nullptr, nullptr, m->n, m->g, num_sub,
        m->pshift, cnt, m->csc_packed, nullptr, nullptr);
  }
  BGPU_CHECK_LAUNCH();
  BGPU_TRY(build_stream_tiles(m, panel_rp, s, &m->bytes));
  BGPU_CUDA(cudaStreamSynchronize(s));  // temporaries are freed on return
  return BGPU_OK;
}

// ===========================================================================
// Row subsets: the layout of X[rows, :] built from a full matrix (its own
// per-gene centring and scaling follow, since the solver computes them from
// the matrix it is given). Device inputs are gathered on the GPU (one warp
// per selected row); host inputs on the host.
namespace {

template <typename I>
__global__ void k_row_lengths(const I* __restrict__ indptr, const int64_t* __restrict__ rows,
                              uint64_t nr, uint64_t n, int64_t* __restrict__ len,
                              int* __restrict__ err) {
  const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= nr) return;
  const int64_t r = rows[i];
  if (r < 0 || (uint64_t)r >= n) {
    atomicOr(err, kErrIndptr);
    len[i] = 0;
    return;
  }
  len[i] = (int64_t)indptr[r + 1] - (int64_t)indptr[r];
}

template <typename I, typename V>
__global__ void k_gather_rows(const I* __restrict__ indptr, const I* __restrict__ indices,
                              const V* __restrict__ values, const int64_t* __restrict__ rows,
                              uint64_t nr, const int64_t* __restrict__ sub_ptr,
                              I* __restrict__ out_idx, V* __restrict__ out_val,
                              const float* __restrict__ isf, const float* __restrict__ post,
                              float* __restrict__ out_isf, float* __restrict__ out_post) {
  const int lane = threadIdx.x & 31;
  const uint64_t w = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nw = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t i = w; i < nr; i += nw) {
    const int64_t r = rows[i];
    const int64_t src = (int64_t)indptr[r], dst = sub_ptr[i];
    const int64_t len = sub_ptr[i + 1] - dst;
    for (int64_t e = lane; e < len; e += 32) {
      out_idx[dst + e] = indices[src + e];
      out_val[dst + e] = values[src + e];
    }
    if (lane == 0) {
      if (isf) out_isf[i] = isf[r];
      if (post) out_post[i] = post[r];
    }
  }
}

template <typename I, typename V>
int gather_device(const bgpu_matrix_desc* d, const int64_t* rows, uint64_t nr,
                  Matrix* m, cudaStream_t s) {
  DevBuf t_len, t_err, t_ptr, t_ptr_i, t_idx, t_val, t_isf, t_post;
  BGPU_TRY(t_len.alloc(nr * 8, s));
  BGPU_TRY(t_err.alloc(4, s));
  BGPU_CUDA(cudaMemsetAsync(t_err.p, 0, 4, s));
  k_row_lengths<I><<<grid_for(nr, 256), 256, 0, s>>>(
      (const I*)d->indptr, rows, nr, d->num_cells, (int64_t*)t_len.p, (int*)t_err.p);
  BGPU_CHECK_LAUNCH();
  std::vector<int64_t> ptr(nr + 1, 0);
  int herr = 0;
  BGPU_CUDA(cudaMemcpyAsync(ptr.data() + 1, t_len.p, nr * 8, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaMemcpyAsync(&herr, t_err.p, 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  BGPU_REQUIRE(herr == 0, BGPU_ERR_INVALID, "a selected row is outside [0, num_cells)");
  for (uint64_t i = 0; i < nr; ++i) ptr[i + 1] += ptr[i];
  const uint64_t nnz = (uint64_t)ptr[nr];
  BGPU_TRY(t_ptr.alloc((nr + 1) * 8, s));
  BGPU_CUDA(cudaMemcpyAsync(t_ptr.p, ptr.data(), (nr + 1) * 8, cudaMemcpyHostToDevice, s));
  BGPU_TRY(t_idx.alloc(nnz * sizeof(I), s));
  BGPU_TRY(t_val.alloc(nnz * sizeof(V), s));
  BGPU_TRY(t_isf.alloc(nr * 4, s));
  if (d->post_factors) BGPU_TRY(t_post.alloc(nr * 4, s));
  const int blocks = std::max(1, (int)std::min<uint64_t>(ceil_div(nr, 8), (uint64_t)num_sms() * 16));
  k_gather_rows<I, V><<<blocks, 256, 0, s>>>(
      (const I*)d->indptr, (const I*)d->indices, (const V*)d->values, rows, nr,
      (const int64_t*)t_ptr.p, (I*)t_idx.p, (V*)t_val.p, d->inv_size_factors,
      d->post_factors, (float*)t_isf.p, (float*)t_post.p);
  BGPU_CHECK_LAUNCH();
  const void* sub_indptr = t_ptr.p;
  std::vector<int32_t> ptr32;
  if (sizeof(I) == 4) {
    ptr32.assign(ptr.begin(), ptr.end());
    BGPU_TRY(t_ptr_i.alloc((nr + 1) * 4, s));
    BGPU_CUDA(cudaMemcpyAsync(t_ptr_i.p, ptr32.data(), (nr + 1) * 4,
                              cudaMemcpyHostToDevice, s));
    sub_indptr = t_ptr_i.p;
  }
  bgpu_matrix_desc sub = *d;
  sub.indptr = sub_indptr;
  sub.indices = t_idx.p;
  sub.values = t_val.p;
  sub.on_device = 1;
  sub.num_cells = nr;
  sub.nnz = nnz;
  sub.inv_size_factors = d->inv_size_factors ? (const float*)t_isf.p : nullptr;
  sub.post_factors = d->post_factors ? (const float*)t_post.p : nullptr;
  return matrix_build(m, &sub, s);  // synchronises before the temporaries go
}

template <typename I, typename V>
int gather_host(const bgpu_matrix_desc* d, const int64_t* rows, uint64_t nr,
                Matrix* m, cudaStream_t s) {
  const I* ip = (const I*)d->indptr;
  const I* ix = (const I*)d->indices;
  const V* vv = (const V*)d->values;
  std::vector<I> ptr(nr + 1, 0);
  for (uint64_t i = 0; i < nr; ++i) {
    const int64_t r = rows[i];
    BGPU_REQUIRE(r >= 0 && (uint64_t)r < d->num_cells, BGPU_ERR_INVALID,
                 "a selected row is outside [0, num_cells)");
    ptr[i + 1] = ptr[i] + (ip[r + 1] - ip[r]);
  }
  const uint64_t nnz = (uint64_t)ptr[nr];
  std::vector<I> idx(nnz);
  std::vector<V> val(nnz);
  std::vector<float> isf(d->inv_size_factors ? nr : 0), post(d->post_factors ? nr : 0);
  for (uint64_t i = 0; i < nr; ++i) {
    const int64_t r = rows[i];
    std::copy(ix + ip[r], ix + ip[r + 1], idx.begin() + ptr[i]);
    std::copy(vv + ip[r], vv + ip[r + 1], val.begin() + ptr[i]);
    if (d->inv_size_factors) isf[i] = d->inv_size_factors[r];
    if (d->post_factors) post[i] = d->post_factors[r];
  }
  bgpu_matrix_desc sub = *d;
  sub.indptr = ptr.data();
  sub.indices = idx.data();
  sub.values = val.data();
  sub.num_cells = nr;
  sub.nnz = nnz;
  sub.inv_size_factors = d->inv_size_factors ? isf.data() : nullptr;
  sub.post_factors = d->post_factors ? post.data() : nullptr;
  return matrix_build(m, &sub, s);
}

template <typename I>
int gather_by_value(const bgpu_matrix_desc* d, const int64_t* rows, uint64_t nr,
                    Matrix* m, cudaStream_t s) {
  const bool dev = d->on_device != 0;
  if (d->value_type == BGPU_VALUE_U16)
    return dev ? gather_device<I, uint16_t>(d, rows, nr, m, s)
               : gather_host<I, uint16_t>(d, rows, nr, m, s);
  return dev ? gather_device<I, uint32_t>(d, rows, nr, m, s)
             : gather_host<I, uint32_t>(d, rows, nr, m, s);
}

}  // namespace

int matrix_build_rows(Matrix* m, const bgpu_matrix_desc* d, const int64_t* rows,
                      uint64_t nr, cudaStream_t s) {
  BGPU_REQUIRE(d != nullptr && rows != nullptr && nr >= 1, BGPU_ERR_INVALID,
               "desc and a non-empty row list are required");
  BGPU_REQUIRE(d->indptr && (d->nnz == 0 || (d->indices && d->values)),
               BGPU_ERR_INVALID, "indptr/indices/values must not be NULL");
  BGPU_REQUIRE(d->index_type == BGPU_INDEX_I32 || d->index_type == BGPU_INDEX_I64,
               BGPU_ERR_INVALID, "index_type must be BGPU_INDEX_I32 or _I64");
  BGPU_REQUIRE(d->value_type >= BGPU_VALUE_U16 && d->value_type <= BGPU_VALUE_F32,
               BGPU_ERR_INVALID, "unknown value_type");
  return d->index_type == BGPU_INDEX_I64 ? gather_by_value<int64_t>(d, rows, nr, m, s)
                                         : gather_by_value<int32_t>(d, rows, nr, m, s);
}

void matrix_free(Matrix* m) {
  void* ptrs[] = {m->rowptr,  m->csr_packed,  m->csr_val,   m->csr_col,
                  m->colptr,  m->csc_packed,  m->csc_val,   m->csc_row,
                  m->isf,     m->post,        m->sd,        m->rtab_r,
                  m->rtab_c,  m->csc16,       m->row_order, m->xv_data,
                  m->xv_grp,  m->xv_units,    m->xv_perm,   m->xv_isf,
                  m->xv_post, m->xv_esc_n,    m->xv_esc_base, m->xv_esc,
                  m->xt_data, m->xt_grp,      m->xt_units,  m->xt_gene,
                  m->xt_pgrp, m->xt_esc_base, m->xt_esc};
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, m->stream);
  *m = Matrix();
}

// ===========================================================================
// Size factors (brisc/normalize.pyx:9-268) and materialised normalisation.
namespace {

// indptr[0] == 0 and non-decreasing (device-pointer entry points check this
// before reading values through indptr).
template <typename I>
__global__ void k_check_indptr(const I* __restrict__ indptr, uint64_t n,
                               int* err) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i > n) return;
  const int64_t v = (int64_t)indptr[i];
  if ((i == 0 && v != 0) || (i < n && (int64_t)indptr[i + 1] < v))
    atomicOr(err, kErrIndptr);
}

template <typename I>
int check_indptr(const void* indptr, uint64_t n, cudaStream_t s) {
  DevBuf e;
  BGPU_TRY(e.alloc(sizeof(int), s));
  BGPU_CUDA(cudaMemsetAsync(e.p, 0, sizeof(int), s));
  k_check_indptr<I><<<grid_for(n + 1, 256), 256, 0, s>>>((const I*)indptr, n,
                                                         (int*)e.p);
  BGPU_CHECK_LAUNCH();
  int herr = 0;
  BGPU_CUDA(cudaMemcpyAsync(&herr, e.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  BGPU_REQUIRE(herr == 0, BGPU_ERR_INVALID,
               "indptr must start at 0 and be non-decreasing");
  return BGPU_OK;
}

int check_indptr_any(const void* indptr, int index_type, uint64_t n,
                     cudaStream_t s) {
  return index_type == BGPU_INDEX_I64 ? check_indptr<int64_t>(indptr, n, s)
                                      : check_indptr<int32_t>(indptr, n, s);
}

template <typename V>
__device__ __forceinline__ unsigned long long as_u64(V x) {
  // `<unsigned long long> data[j]` (normalize.pyx:45): truncation toward zero.
  return (unsigned long long)x;
}

template <typename I, typename V>
__global__ void k_row_sums(const I* __restrict__ indptr, const V* __restrict__ values,
                           uint64_t n, const uint8_t* __restrict__ qc,
                           unsigned long long* __restrict__ row_sums,
                           unsigned long long* __restrict__ totals /*[2]*/) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  unsigned long long tot = 0, nqc = 0;
  for (uint64_t r = warp; r < n; r += nwarps) {
    int64_t e0 = (int64_t)indptr[r], e1 = (int64_t)indptr[r + 1];
    unsigned long long s = 0;
    for (int64_t e = e0 + lane; e < e1; e += 32) s += as_u64(values[e]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      row_sums[r] = s;
      if (!qc || qc[r]) { tot += s; nqc += 1; }
    }
  }
  if (lane == 0 && (tot || nqc)) {
    atomicAdd(&totals[0], tot);  // integer: order-independent
    atomicAdd(&totals[1], nqc);
  }
}

__global__ void k_isf(const unsigned long long* __restrict__ row_sums, uint64_t n,
                      int method, const unsigned long long* __restrict__ totals,
                      float* __restrict__ isf) {
  uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  float nf;
  if (method == 0) {
    nf = 10000.f;  // normalize.pyx:55
  } else {
    // normalize.pyx:78: `<float> total_sum / num_QCed_cells`
    nf = (float)totals[0] / (float)totals[1];
  }
  isf[i] = nf / (float)row_sums[i];  // normalize.pyx:87
}

// Method 2, step 3a: new_row_sums[i] = sum_j log1p(data[j] * isf[i]) in float.
template <typename I, typename V>
__global__ void k_new_row_sums(const I* __restrict__ indptr, const V* __restrict__ values,
                               uint64_t n, const float* __restrict__ isf,
                               float* __restrict__ nrs) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t r = warp; r < n; r += nwarps) {
    int64_t e0 = (int64_t)indptr[r], e1 = (int64_t)indptr[r + 1];
    const float f = isf[r];
    float s = 0.f;
    for (int64_t e = e0 + lane; e < e1; e += 32) s += log1pf((float)values[e] * f);
    s = warp_sum(s);
    if (lane == 0) nrs[r] = s;
  }
}

// Fixed-order float total over QC cells: 1024-cell blocks, then blocks in order.
__global__ void k_block_float_sum(const float* __restrict__ x, uint64_t n,
                                  const uint8_t* __restrict__ qc,
                                  float* __restrict__ partial) {
  __shared__ float sh[32];
  uint64_t base = blockIdx.x * 1024ull;
  float v = 0.f;
  uint64_t i = base + threadIdx.x;
  if (i < n && (!qc || qc[i])) v = x[i];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    float t = sh[threadIdx.x];
    t = warp_sum(t);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

__global__ void k_post(const float* __restrict__ partial, uint32_t nblocks,
                       const unsigned long long* __restrict__ totals,
                       const float* __restrict__ nrs, uint64_t n,
                       float* __restrict__ post) {
  __shared__ float nf2;
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (uint32_t b = 0; b < nblocks; ++b) t += partial[b];
    nf2 = t / (float)totals[1];  // normalize.pyx:255-256
  }
  __syncthreads();
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
       i += (uint64_t)gridDim.x * blockDim.x)
    post[i] = nf2 / nrs[i];  // normalize.pyx:263-264
}

template <typename I, typename V>
__global__ void k_normalize(const I* __restrict__ indptr, const V* __restrict__ values,
                            uint64_t n, const float* __restrict__ isf,
                            const float* __restrict__ post, float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = (gridDim.x * (uint64_t)blockDim.x) >> 5;
  for (uint64_t r = warp; r < n; r += nwarps) {
    int64_t e0 = (int64_t)indptr[r], e1 = (int64_t)indptr[r + 1];
    const float f = isf[r];
    const float q = post ? post[r] : 1.f;
    for (int64_t e = e0 + lane; e < e1; e += 32) {
      float v = log1pf((float)values[e] * f);
      out[e] = post ? v * q : v;
    }
  }
}

template <typename I, typename V>
int size_factors_typed(const void* indptr, const void* values, uint64_t n,
                       int method, const uint8_t* qc, float* isf, float* post,
                       uint64_t* row_sums_out, cudaStream_t s) {
  DevBuf t_rs, t_tot, t_nrs, t_part;
  unsigned long long* rs = (unsigned long long*)row_sums_out;
  if (!rs) {
    BGPU_TRY(t_rs.alloc(n * 8, s));
    rs = (unsigned long long*)t_rs.p;
  }
  BGPU_TRY(t_tot.alloc(16, s));
  unsigned long long* tot = (unsigned long long*)t_tot.p;
  BGPU_CUDA(cudaMemsetAsync(tot, 0, 16, s));
  int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(n, 8),
                                                            (uint64_t)num_sms() * 16));
  k_row_sums<I, V><<<blocks, 256, 0, s>>>((const I*)indptr, (const V*)values, n,
                                          qc, rs, tot);
  BGPU_CHECK_LAUNCH();
  k_isf<<<grid_for(n, 256), 256, 0, s>>>(rs, n, method, tot, isf);
  BGPU_CHECK_LAUNCH();
  if (method == 2) {
    BGPU_TRY(t_nrs.alloc(n * 4, s));
    float* nrs = (float*)t_nrs.p;
    k_new_row_sums<I, V><<<blocks, 256, 0, s>>>((const I*)indptr,
                                                (const V*)values, n, isf, nrs);
    BGPU_CHECK_LAUNCH();
    uint32_t nb = (uint32_t)ceil_div(n, 1024);
    BGPU_TRY(t_part.alloc(nb * 4, s));
    k_block_float_sum<<<nb, 1024, 0, s>>>(nrs, n, qc, (float*)t_part.p);
    BGPU_CHECK_LAUNCH();
    k_post<<<grid_for(n, 256, 4096), 256, 0, s>>>((const float*)t_part.p, nb,
                                                  tot, nrs, n, post);
    BGPU_CHECK_LAUNCH();
  }
  BGPU_CUDA(cudaStreamSynchronize(s));
  return BGPU_OK;
}

template <typename I>
int size_factors_by_value(const void* indptr, int vt, const void* values,
                          uint64_t n, int method, const uint8_t* qc, float* isf,
                          float* post, uint64_t* rs, cudaStream_t s) {
  switch (vt) {
    case BGPU_VALUE_U16:
      return size_factors_typed<I, uint16_t>(indptr, values, n, method, qc, isf, post, rs, s);
    case BGPU_VALUE_U32:
      return size_factors_typed<I, uint32_t>(indptr, values, n, method, qc, isf, post, rs, s);
    case BGPU_VALUE_I32:
      return size_factors_typed<I, int32_t>(indptr, values, n, method, qc, isf, post, rs, s);
    default:
      return size_factors_typed<I, float>(indptr, values, n, method, qc, isf, post, rs, s);
  }
}

template <typename I>
int normalize_by_value(const void* indptr, int vt, const void* values,
                       uint64_t n, const float* isf, const float* post,
                       float* out, cudaStream_t s) {
  int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>(ceil_div(n, 8),
                                                            (uint64_t)num_sms() * 16));
  switch (vt) {
    case BGPU_VALUE_U16:
      k_normalize<I, uint16_t><<<blocks, 256, 0, s>>>((const I*)indptr, (const uint16_t*)values, n, isf, post, out);
      break;
    case BGPU_VALUE_U32:
      k_normalize<I, uint32_t><<<blocks, 256, 0, s>>>((const I*)indptr, (const uint32_t*)values, n, isf, post, out);
      break;
    case BGPU_VALUE_I32:
      k_normalize<I, int32_t><<<blocks, 256, 0, s>>>((const I*)indptr, (const int32_t*)values, n, isf, post, out);
      break;
    default:
      k_normalize<I, float><<<blocks, 256, 0, s>>>((const I*)indptr, (const float*)values, n, isf, post, out);
  }
  BGPU_CHECK_LAUNCH();
  return BGPU_OK;
}

// ---------------------------------------------------------------------------
// Global stable CSR -> CSC (the reference's output format).
template <typename I>
__global__ void k_global_hist(const I* __restrict__ Ap, const I* __restrict__ Aj,
                              uint64_t n, uint32_t g, uint32_t num_sub,
                              long long* __restrict__ cnt, int* err) {
  const int lane = threadIdx.x & 31;
  const uint64_t s = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (s >= num_sub) return;
  uint64_t r0 = s * kSubRows, r1 = min_u64(n, r0 + kSubRows);
  long long* my = cnt + s * (uint64_t)g;
  for (int64_t e = (int64_t)Ap[r0] + lane; e < (int64_t)Ap[r1]; e += 32) {
    int64_t c = (int64_t)Aj[e];
    if (c < 0 || c >= (int64_t)g) { atomicOr(err, kErrIndex); continue; }
    atomicAdd((unsigned long long*)(my + c), 1ull);
  }
}

template <typename I>
__global__ void k_global_scatter(const I* __restrict__ Ap, const I* __restrict__ Aj,
                                 const uint32_t* __restrict__ Ax, uint64_t n,
                                 uint32_t g, uint32_t num_sub,
                                 long long* __restrict__ cnt, I* __restrict__ Bi,
                                 uint32_t* __restrict__ Bx) {
  const int lane = threadIdx.x & 31;
  const uint64_t s = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
  if (s >= num_sub) return;
  uint64_t r0 = s * kSubRows, r1 = min_u64(n, r0 + kSubRows);
  long long* pos = cnt + s * (uint64_t)g;
  for (uint64_t r = r0; r < r1; ++r) {
    for (int64_t e = (int64_t)Ap[r] + lane; e < (int64_t)Ap[r + 1]; e += 32) {
      int64_t c = (int64_t)Aj[e];
      if (c < 0 || c >= (int64_t)g) continue;
      long long slot = (long long)atomicAdd((unsigned long long*)(pos + c), 1ull);
      Bi[slot] = (I)r;
      Bx[slot] = Ax[e];
    }
    __syncwarp();
  }
}

template <typename I>
__global__ void k_store_bp(const long long* __restrict__ cp, I* __restrict__ Bp,
                           uint32_t g) {
  uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c <= g) Bp[c] = (I)cp[c];
}

template <typename I>
int csr_tocsc_typed(uint64_t n, uint32_t g, const void* Ap, const void* Aj,
                    const void* Ax, void* Bp, void* Bi, void* Bx, cudaStream_t s) {
  const uint32_t num_sub = (uint32_t)ceil_div(n, kSubRows);
  DevBuf t_cnt, t_cp, t_err;
  BGPU_TRY(t_cnt.alloc((size_t)num_sub * g * 8, s));
  BGPU_TRY(t_cp.alloc((size_t)(g + 1) * 8, s));
  BGPU_TRY(t_err.alloc(4, s));
  long long* cnt = (long long*)t_cnt.p;
  BGPU_CUDA(cudaMemsetAsync(cnt, 0, (size_t)num_sub * g * 8, s));
  BGPU_CUDA(cudaMemsetAsync(t_err.p, 0, 4, s));
  const int wblocks = (int)ceil_div(num_sub, 8);
  k_global_hist<I><<<wblocks, 256, 0, s>>>((const I*)Ap, (const I*)Aj, n, g,
                                           num_sub, cnt, (int*)t_err.p);
  BGPU_CHECK_LAUNCH();
  k_panel_scan<long long><<<1, 1024, 0, s>>>(cnt, (long long*)t_cp.p, g, num_sub,
                                             num_sub);
  BGPU_CHECK_LAUNCH();
  k_global_scatter<I><<<wblocks, 256, 0, s>>>((const I*)Ap, (const I*)Aj,
                                              (const uint32_t*)Ax, n, g, num_sub,
                                              cnt, (I*)Bi, (uint32_t*)Bx);
  BGPU_CHECK_LAUNCH();
  k_store_bp<I><<<grid_for(g + 1, 256), 256, 0, s>>>((const long long*)t_cp.p,
                                                     (I*)Bp, g);
  BGPU_CHECK_LAUNCH();
  int herr = 0;
  BGPU_CUDA(cudaMemcpyAsync(&herr, t_err.p, 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  BGPU_REQUIRE(herr == 0, BGPU_ERR_INVALID, "a column index is outside [0, n_col)");
  return BGPU_OK;
}

}  // namespace
}  // namespace bgpu

using namespace bgpu;

extern "C" int bgpu_size_factors(const void* indptr, int index_type,
                                 const void* values, int value_type,
                                 uint64_t num_cells, int method,
                                 const uint8_t* qc_mask, float* isf, float* post,
                                 uint64_t* row_sums, void* stream) {
  BGPU_REQUIRE(indptr && values && isf, BGPU_ERR_INVALID,
               "indptr, values and isf must not be NULL");
  BGPU_REQUIRE(method >= 0 && method <= 2, BGPU_ERR_INVALID,
               "method must be 0 (logCP10k), 1 (log1pPF) or 2 (PFlog1pPF)");
  BGPU_REQUIRE(method != 2 || post, BGPU_ERR_INVALID, "method 2 needs `post`");
  BGPU_REQUIRE(num_cells >= 1, BGPU_ERR_INVALID, "num_cells must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  BGPU_TRY(check_indptr_any(indptr, index_type, num_cells, s));
  if (index_type == BGPU_INDEX_I64)
    return size_factors_by_value<int64_t>(indptr, value_type, values, num_cells,
                                          method, qc_mask, isf, post, row_sums, s);
  return size_factors_by_value<int32_t>(indptr, value_type, values, num_cells,
                                        method, qc_mask, isf, post, row_sums, s);
}

extern "C" int bgpu_normalize_csr(const void* indptr, int index_type,
                                  const void* values, int value_type,
                                  uint64_t num_cells, const float* isf,
                                  const float* post, float* normalized,
                                  void* stream) {
  BGPU_REQUIRE(indptr && values && isf && normalized, BGPU_ERR_INVALID,
               "indptr, values, isf and normalized must not be NULL");
  cudaStream_t s = (cudaStream_t)stream;
  BGPU_TRY(check_indptr_any(indptr, index_type, num_cells, s));
  if (index_type == BGPU_INDEX_I64)
    return normalize_by_value<int64_t>(indptr, value_type, values, num_cells,
                                       isf, post, normalized, s);
  return normalize_by_value<int32_t>(indptr, value_type, values, num_cells, isf,
                                     post, normalized, s);
}

extern "C" int bgpu_csr_tocsc(uint64_t n_row, uint32_t n_col, const void* Ap,
                              const void* Aj, const void* Ax, int index_type,
                              void* Bp, void* Bi, void* Bx, void* stream) {
  BGPU_REQUIRE(Ap && Bp && n_row >= 1 && n_col >= 1, BGPU_ERR_INVALID,
               "bad csr_tocsc arguments");
  cudaStream_t s = (cudaStream_t)stream;
  BGPU_TRY(check_indptr_any(Ap, index_type, n_row, s));
  if (index_type == BGPU_INDEX_I64)
    return csr_tocsc_typed<int64_t>(n_row, n_col, Ap, Aj, Ax, Bp, Bi, Bx, s);
  return csr_tocsc_typed<int32_t>(n_row, n_col, Ap, Aj, Ax, Bp, Bi, Bx, s);
}
