// Dense kernels of the IRLBA solve (internal).
#pragma once

#include "common.cuh"
#include "multi.cuh"

namespace bgpu {

constexpr int kRowBlock = 1024;  // rows per fixed reduction block (256 threads x 4)

// The last block of a norm-producing U update finishes the norm: B[j, j] =
// alpha = max(sqrt(sum of the norm partials), 1e-8) in FP64 and scal =
// {alpha, 1 / alpha} (pca.pyx:1081-1086), and, when gate
// is non-null, gate = {|y_out|^2, |y_in - mean|^2}. counter: a zeroed device
// word per solve (the last block resets it). B == nullptr: no finish.
struct NormFinish {
  double* B = nullptr;
  uint32_t m = 0, j = 0;
  float* scal = nullptr;
  float* gate = nullptr;
  unsigned* counter = nullptr;
};

// part[b * pstride + c] = U[rows of b, c] . y[rows of b]   for c < ncols
// and, when with_sum, part[b * pstride + ncols] = sum(y[rows of b]).
//
// Adaptive second pass: the dots, reduce and update kernels take an optional
// device `gate` = {|y1|^2, |y0 - mean|^2} of the first pass and return at
// once, writing nothing, when gate[0] >= gate[1] / 2 (the first pass kept at
// least half of the squared norm: "twice is enough", Kahan-Parlett).
int launch_udots(const float* U, uint64_t ldu, uint32_t ncols, const float* y,
                 uint64_t nblocks, float* part, uint32_t pstride, bool with_sum,
                 cudaStream_t s, const float* gate = nullptr);

// y_out = y_in - (mean + U[:, :ncols] . coef)   for rows < n, 0 beyond.
// mean = (*mean_sum) / n when mean_sum is non-null (the reference's
// `dot_product = mean; dot_product += U[row, col] * work[col]`, pca.pyx:1045).
// When norm_part is non-null, norm_part[b * pstride] = sum(y_out^2) per block,
// and with with_centred also norm_part[b * pstride + 1] = sum((y_in - mean)^2).
// y_in may equal y_out (each thread reads its rows before writing them).
// When taken is non-null and the update ran, taken[0] += 1, taken[1] += ncols.
int launch_uupdate(const float* U, uint64_t ldu, uint32_t ncols,
                   const float* coef, const float* mean_sum, uint64_t n,
                   const float* y_in, float* y_out, uint64_t nblocks,
                   float* norm_part, uint32_t pstride, cudaStream_t s,
                   bool with_centred = false, const float* gate = nullptr,
                   unsigned long long* taken = nullptr, NormFinish fin = {});

// CGS2 middle pass in one read of U: y_out = y_in - (mean + U[:, :ncols] coef)
// as launch_uupdate, and part[b * pstride + c] = U[rows of b, c] . y_out[rows
// of b] over 256-row blocks b (uupdate_dots_blocks(n) of them).
size_t uupdate_dots_smem(uint32_t ncols);
uint64_t uupdate_dots_blocks(uint64_t n);
int launch_uupdate_dots(const float* U, uint64_t ldu, uint32_t ncols,
                        const float* coef, const float* mean_sum, uint64_t n,
                        const float* y_in, float* y_out, float* part,
                        uint32_t pstride, cudaStream_t s);

// out[c] = sum_b part[b * pstride + c] (coalesced: lanes take columns, warps
// stride the blocks; the warp sums are added in warp order).
int launch_reduce_cols(const float* part, uint64_t nblocks, uint32_t pstride,
                       uint32_t ncols, float* out, cudaStream_t s,
                       const float* gate = nullptr);

// V-side half step (pca.pyx:1103-1171): given z = (X^T u) / sd, forms
// z - alpha V[:, j], runs `passes` rounds of classical Gram-Schmidt against
// V[:, :j+1] (passes = 0: one round, and a second only when the first kept
// less than half of the squared norm); then either V[:, j+1] = z / beta,
// B[j, j+1] = beta (j < m-1) or rem = z (j == m-1).
int launch_vstep(const float* z, float* V, uint64_t ldv, uint32_t g,
                 uint32_t j, uint32_t m, const float* scal, double* B,
                 float* rem, int passes, cudaStream_t s);

// C = A . Bop (tall-skinny): A is rows x K column-major (lda), Bop(i, c) =
// Bp[i * bsr + c * bsc] (K x ncols), optional per-column scale cs[c] applied
// to Bop. Output column-major (ldc) or, when c_rowmajor, row-major with row
// stride ldc. Each output is one fixed-order dot product (deterministic).
int launch_gemm_ts(const float* A, uint64_t lda, uint64_t rows, uint32_t K,
                   const float* Bp, uint64_t bsr, uint64_t bsc,
                   const float* cs, uint32_t ncols, float* C, uint64_t ldc,
                   bool c_rowmajor, cudaStream_t s);

// C = A . Bm[:, :ncols] on the tensor cores (tc_gemm.cu): A rows x K and Bm
// (K x ncols, ldb) column-major, C column-major (ldc); 3 x BF16 split with
// FP32 accumulation, dominated columns of Bm in the pivoted delta form.
// Scratch: dwork K x ncols floats, piv ncols ints. err receives a device
// error word on a timed-out wait.
bool gemm_tc_supported(uint32_t K, uint32_t ncols);
int launch_gemm_tc(const float* A, uint64_t lda, uint64_t rows, uint32_t K,
                   const float* Bm, uint64_t ldb, uint32_t ncols, float* C,
                   uint64_t ldc, float* dwork, int* piv, int* err, cudaStream_t s);

// Fused multi-solve forms of the step kernels (multi.cuh): one launch over
// every task, each task's CTAs computing what the single launch above
// computes for its arguments. CTAs per task (the caller adds them with
// TaskList::add): udots and uupdate `nblocks` (the single launch's grid),
// reduce_cols ceil(ncols / 32) (tasks with ncols == 0 are left out), vstep
// kVStepCtas (one thread-block cluster).
struct UdotsTask {
  const float* U;
  uint64_t ldu;
  const float* y;
  float* part;
  const float* gate;
  uint32_t ncols, pstride;
  int with_sum;
};
struct ReduceColsTask {
  const float* part;
  uint64_t nblocks;
  float* out;
  const float* gate;
  uint32_t pstride, ncols;
};
struct UupdateTask {
  const float* U;
  uint64_t ldu;
  const float* coef;
  const float* mean_sum;
  uint64_t n;
  const float* y_in;
  float* y_out;
  float* norm_part;
  const float* gate;
  unsigned long long* taken;
  NormFinish fin;
  uint32_t ncols, pstride;
  int with_centred;
};
struct VstepTask {
  const float* z;
  float* V;
  uint64_t ldv;
  const float* scal;
  double* B;
  float* rem;
  uint32_t g, j, m;
  int passes;
};
constexpr uint32_t kVStepCtas = 8;
// whether launch_vstep runs (g, m) on one cluster (the multi form's only path)
bool vstep_cluster_fits(uint32_t g, uint32_t m);
int launch_udots_multi(const TaskList<UdotsTask>& L, cudaStream_t s);
int launch_reduce_cols_multi(const TaskList<ReduceColsTask>& L, cudaStream_t s);
int launch_uupdate_multi(const TaskList<UupdateTask>& L, cudaStream_t s);
int launch_vstep_multi(const TaskList<VstepTask>& L, cudaStream_t s);

// B (m x (m+1), column-major FP64) -> float copy for the small SVD.
int launch_b_to_float(const double* B, uint32_t m, float* Bf, cudaStream_t s);

}  // namespace bgpu
