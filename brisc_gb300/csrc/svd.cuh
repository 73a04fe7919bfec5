// Small SVD and restart bookkeeping (internal).
#pragma once

#include "common.cuh"

namespace bgpu {

struct RestartStatus {
  int converged;
  int num_converged;
  int k_current;
  float remainder_norm;
  float smax;
  int pad[3];
};

size_t jacobi_smem_bytes(uint32_t m, bool fp64);
size_t jacobi_global_bytes(uint32_t m, bool fp64);
float jacobi_threshold(uint32_t m);

// FP64 Newton (Ogita-Aishima) refinement of an FP32 SVD of B (FP64, m x
// (m+1), column-major): `steps` steps on Ub, then Sb, Vbt and the FP64 last
// row of Ub (ub_last) and singular values (sb64) from the refined factors.
// Ub, Sb, Vbt are rewritten in place. work: svd_refine_doubles(m) doubles.
size_t svd_refine_doubles(uint32_t m);
int launch_svd_refine(const double* B, uint32_t m, float* Ub, float* Sb, float* Vbt,
                      double* ub_last, double* sb64, double* work, int steps,
                      cudaStream_t s, double* u64_out = nullptr);
int launch_float_to_double(const float* a, uint64_t n, double* b, cudaStream_t s);

// One-sided Jacobi SVD of B (m x (m+1), column-major), in FP64 when Bd is
// given (Bf ignored) or FP32 from Bf. Outputs float Ub (m x m), Sb (m), Vbt
// (m x (m+1)), column-major; optionally the FP64 last row of Ub (ub_last, m)
// and FP64 singular values (sb64, m). gwork: jacobi_global_bytes(m, fp64)
// bytes when the matrices do not fit in shared memory; info (2 ints: sweeps,
// converged) may be null; ub64 (may be null) receives Ub in FP64.
int launch_jacobi_svd(const float* Bf, const double* Bd, uint32_t m, float* Ub,
                      float* Sb, float* Vbt, double* ub_last, double* sb64,
                      void* gwork, int* info, cudaStream_t s, double* ub64 = nullptr);

// Normalises rem, updates Smax, counts converged Ritz values, picks the next
// k_current and (when not converged) rebuilds B as diag(Sb) plus the residual
// column, exactly as brisc/pca.pyx:1180-1231 orders those steps. With ub_last
// and sb64 the residual test and the new B use the FP64 SVD outputs. ratios
// (k floats, may be null) receives |residual| / (tol * Smax) per value.
int launch_restart_check(const float* Ub, const float* Sb, const double* ub_last,
                         const double* sb64, uint32_t m, uint32_t k, float* rem,
                         uint32_t g, float tol, float* smax, uint32_t kc,
                         double* B, RestartStatus* st, float* ratios,
                         cudaStream_t s);

// Restart SVD by a secular-equation merge (svd_merge.cu), for B as rebuilt
// by the restart (diag(s) in columns < kc, residual column kc) plus the t =
// m - kc Lanczos rows of the cycle: the tail's SVD (size t), then the
// eigenpairs of diag(s^2, mu) + z z^T in FP64. Same outputs as
// launch_jacobi_svd + launch_svd_refine. Workspaces: tailw tail_work_bytes(m),
// mergew merge_work_bytes(m), refine_work svd_refine_doubles(m) doubles,
// jacobi_gwork as for launch_jacobi_svd at size m (may be null where that
// needs none).
constexpr uint32_t kMergeClosedTailMax = 2;  // tails up to this size: closed form
struct MergeWork {
  double *ds, *zs, *dn, *zn, *tau, *zhat, *lam, *rot_c, *rot_s, *znorm2;
  int *src, *defl, *ndpos, *defpos, *rot_p, *rot_q, *korig, *order, *state;
};
size_t tail_work_bytes(uint32_t m);
size_t merge_work_bytes(uint32_t m);
int launch_svd_merge(const double* B, uint32_t m, uint32_t kc, float* Ub, float* Sb,
                     float* Vbt, double* ub_last, double* sb64, void* tailw,
                     void* mergew, double* refine_work, void* jacobi_gwork,
                     int refine_steps, cudaStream_t s);

}  // namespace bgpu
