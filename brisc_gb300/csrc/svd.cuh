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

size_t jacobi_smem_bytes(uint32_t m);
size_t jacobi_global_floats(uint32_t m);
float jacobi_threshold(uint32_t m);

// Bf: m x (m+1) column-major. Ub m x m, Sb m, Vbt m x (m+1), column-major.
// gwork: jacobi_global_floats(m) floats when the matrices do not fit in shared
// memory (m > ~170); info (2 ints: sweeps, converged) may be null.
int launch_jacobi_svd(const float* Bf, uint32_t m, float* Ub, float* Sb,
                      float* Vbt, float* gwork, int* info, cudaStream_t s);

// Normalises rem, updates Smax, counts converged Ritz values, picks the next
// k_current and (when not converged) rebuilds B as diag(Sb) plus the residual
// column, exactly as brisc/pca.pyx:1180-1231 orders those steps.
int launch_restart_check(const float* Ub, const float* Sb, uint32_t m,
                         uint32_t k, float* rem, uint32_t g, float tol,
                         float* smax, uint32_t kc, double* B,
                         RestartStatus* st, cudaStream_t s);

}  // namespace bgpu
