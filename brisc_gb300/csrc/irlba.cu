// IRLBA driver (host C++) and the C-ABI entry points.
//
// The restart loop follows brisc/pca.pyx:982-1231 (the deterministic parallel
// path): for every restart, Lanczos steps j = k_current .. m-1 (X.v, fused U
// pass, X^T.u, V-side step), then the small SVD of B, the convergence test and
// the restart rotation. All vector work stays on the GPU; the host only reads
// a 32-byte restart status per restart (to learn k_current and convergence).
//
// Deviation kept on purpose: when max_iterations is reached
// without convergence, the reference rotates U once more and then multiplies
// by Ub again (pca.pyx:1210-1215 then 1253), mixing in stale buffer columns;
// here the last restart is not rotated, so the returned PCs are the Ritz
// vectors of the final SVD, scaled by their singular values.
#include <array>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "dense.cuh"
#include "matrix.cuh"
#include "pcg.h"
#include "svd.cuh"

namespace bgpu {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }
const char* get_error() { return g_last_error.c_str(); }

int num_sms() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return kNumSMs;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (!cache[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = kNumSMs;
    cache[dev] = v;
  }
  return cache[dev];
}

int device_smem_optin() {
  static std::mutex mu;
  static std::vector<int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 227 * 1024;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (!cache[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
            cudaSuccess || v <= 0)
      v = 227 * 1024;
    cache[dev] = v;
  }
  return cache[dev];
}

// ---------------------------------------------------------------------------
// PCG32 + Box-Muller start vector, restating brisc/cyutils.pyx:1153-1232 and
// brisc/pca.pyx:801-806 operation for operation (float arithmetic as there).
namespace {

inline float pcg_normal(uint64_t* state) {  // cyutils.pyx:1180-1191
  float u1;
  while (true) {
    u1 = pcg_uniform(state);
    if (u1 != 0) break;
  }
  const float u2 = pcg_uniform(state);
  const float r = std::sqrt(-2 * std::log(u1));
  const float theta = (float)(2 * 3.14159265358979323846 * (double)u2);
  return r * std::cos(theta);
}

}  // namespace

int start_vector(uint64_t seed, uint32_t g, float* out) {
  uint64_t state = pcg_srand(seed);
  for (uint32_t i = 0; i < g; ++i) out[i] = pcg_normal(&state);
  float nrm = 0;  // cyutils.pyx:1089-1094
  for (uint32_t i = 0; i < g; ++i) nrm += out[i] * out[i];
  nrm = std::sqrt(nrm);
  const float inv = 1 / nrm;
  for (uint32_t i = 0; i < g; ++i) out[i] *= inv;
  return BGPU_OK;
}

// ---------------------------------------------------------------------------
namespace {

// Solver buffers come from the stream-ordered allocator and go back on the
// same stream: unlike cudaMalloc/cudaFree, neither waits for the whole
// device, so solves on different streams (batched subsets, served requests)
// never stall one another at their start or end.
struct Buf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  Buf() = default;
  Buf(const Buf&) = delete;
  ~Buf() { reset(); }
  void reset() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
  }
  template <typename T>
  T* as() const { return (T*)p; }
};

int balloc(Buf& b, size_t bytes, bool zero, cudaStream_t s) {
  if (bytes == 0) bytes = 16;
  b.s = s;
  cudaError_t e = cudaMallocAsync(&b.p, bytes, s);
  if (e != cudaSuccess) {
    b.p = nullptr;
    set_error(std::string("cudaMalloc(") + std::to_string(bytes) +
              ") failed: " + cudaGetErrorString(e));
    return BGPU_ERR_ALLOC;
  }
  if (zero) BGPU_CUDA(cudaMemsetAsync(b.p, 0, bytes, s));
  return BGPU_OK;
}

constexpr int kRefineSteps = 3;  // Newton steps after the FP32 Jacobi

struct HostStatus {
  RestartStatus v{};
  RestartStatus* h = &v;
};

struct Solver {
  const Matrix& X;
  uint64_t n;
  uint32_t g, k, m;
  uint64_t ldu, ldv, nb;
  uint32_t ps;
  int passes;
  bool adaptive;  // second U-side pass only where the first cancelled
  cudaStream_t s;
  float tol;

  Buf U, Unew, V, Vnew, y0, y1, part, coef, zpart, zvec, rem, sd, Bf, Ub, Sb,
      Vbt, oaw, svdwork, scal, smax, B, st, sdpart, svdinfo, ub_last,
      sb64, ratios, rotd, rotpiv, tailw, mergew,
      derr, taken, ticket;
  uint32_t svd_mode = 0;     // opts.svd_mode
  bool svd64 = false;        // full FP64 Jacobi (svd_mode 1)
  uint32_t merged_svds = 0;  // restarts solved by the secular merge
  int rot_mode = 0;    // 1 = SIMT FP32 rotation, 2 = tensor-core 3 x BF16
  bool trace = false;  // BGPU_TRACE=1: one stderr line per restart
  HostStatus hst;

  // accounting
  uint64_t launches = 0;
  uint64_t second_host = 0;  // second passes of a fixed-CGS2 solve
  double reorth_bytes = 0, rotation_bytes = 0;
  // profiling: event pairs around each kernel class, in two pools that
  // alternate by restart: a restart's events are read on the host while the
  // GPU runs the next rotation, not while it waits at the restart's sync
  bool profile = false;
  std::vector<cudaEvent_t> ev[2];
  // kinds: 0 X.v, 1 X^T.u, 2 SVD, 3 U pass, 4 V step, 5 rotation
  std::vector<int> ev_kind[2];
  size_t ev_used[2] = {0, 0};
  int cur = 0;
  double t_kind[6] = {0, 0, 0, 0, 0, 0};

  ~Solver() {
    for (auto& pool : ev)
      for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }

  int ev_begin(int kind) {
    if (!profile) return BGPU_OK;
    auto& pool = ev[cur];
    size_t& used = ev_used[cur];
    if (used + 2 > pool.size()) {
      for (int i = 0; i < 2; ++i) {
        cudaEvent_t e;
        BGPU_CUDA(cudaEventCreate(&e));
        pool.push_back(e);
      }
      ev_kind[cur].push_back(0);
    }
    ev_kind[cur][used / 2] = kind;
    BGPU_CUDA(cudaEventRecord(pool[used], s));
    return BGPU_OK;
  }
  int ev_end() {
    if (!profile) return BGPU_OK;
    BGPU_CUDA(cudaEventRecord(ev[cur][ev_used[cur] + 1], s));
    ev_used[cur] += 2;
    return BGPU_OK;
  }
  // Reads a pool whose events have all completed (the stream was
  // synchronised after the last of them).
  int ev_collect(int pool) {
    for (size_t i = 0; i < ev_used[pool]; i += 2) {
      float ms = 0.f;
      BGPU_CUDA(cudaEventElapsedTime(&ms, ev[pool][i], ev[pool][i + 1]));
      t_kind[ev_kind[pool][i / 2]] += ms * 1e-3;
    }
    ev_used[pool] = 0;
    return BGPU_OK;
  }

  Solver(const Matrix& X_, const bgpu_solve_opts& o, cudaStream_t s_)
      : X(X_), n(X_.n), g(X_.g), k(o.k), m(o.subspace_size), s(s_),
        tol(o.tolerance) {
    ldu = basis_ld(n);
    ldv = basis_ld(g);
    nb = ceil_div(n, kRowBlock);
    ps = m + 2;
    passes = o.reorth_passes == 1 ? 1 : 2;
    adaptive = o.reorth_passes == 0;
  }

  int alloc() {
    BGPU_TRY(balloc(U, ldu * m * 4, true, s));
    BGPU_TRY(balloc(Unew, ldu * m * 4, true, s));
    BGPU_TRY(balloc(V, ldv * m * 4, true, s));
    BGPU_TRY(balloc(Vnew, ldv * m * 4, true, s));
    BGPU_TRY(balloc(y0, ldu * 4, true, s));
    BGPU_TRY(balloc(y1, ldu * 4, true, s));
    BGPU_TRY(balloc(part, std::max<uint64_t>(nb, uupdate_dots_blocks(n)) * ps * 4, true, s));
    BGPU_TRY(balloc(coef, 2 * (size_t)ps * 4, true, s));
    BGPU_TRY(balloc(zpart, (size_t)X.num_panels * g * 4, true, s));
    BGPU_TRY(balloc(zvec, ldv * 4, true, s));
    BGPU_TRY(balloc(derr, 16, true, s));
    BGPU_TRY(balloc(rem, ldv * 4, true, s));
    BGPU_TRY(balloc(sd, ldv * 4, true, s));
    BGPU_TRY(balloc(Bf, (size_t)m * (m + 1) * 4, true, s));
    BGPU_TRY(balloc(Ub, (size_t)m * m * 4, true, s));
    BGPU_TRY(balloc(Sb, (size_t)m * 4, true, s));
    BGPU_TRY(balloc(Vbt, (size_t)m * (m + 1) * 4, true, s));
    BGPU_TRY(balloc(rotd, (size_t)m * m * 4, false, s));  // tensor-core rotation scratch
    BGPU_TRY(balloc(rotpiv, (size_t)m * 4, false, s));
    if (svd_mode == 0) {  // secular-merge workspaces
      BGPU_TRY(balloc(tailw, tail_work_bytes(m), false, s));
      BGPU_TRY(balloc(mergew, merge_work_bytes(m), false, s));
    }
    BGPU_TRY(balloc(oaw, svd_refine_doubles(m) * 8, true, s));
    if (jacobi_smem_bytes(m, svd64) > 220 * 1024)
      BGPU_TRY(balloc(svdwork, jacobi_global_bytes(m, svd64), true, s));
    BGPU_TRY(balloc(ub_last, (size_t)m * 8, true, s));
    BGPU_TRY(balloc(sb64, (size_t)m * 8, true, s));
    BGPU_TRY(balloc(ratios, (size_t)m * 4, true, s));
    BGPU_TRY(balloc(scal, 64, true, s));
    BGPU_TRY(balloc(smax, 64, false, s));
    BGPU_TRY(balloc(B, (size_t)m * (m + 1) * 8, true, s));
    BGPU_TRY(balloc(st, sizeof(RestartStatus), true, s));
    BGPU_TRY(balloc(sdpart, (size_t)X.num_panels * g * 16, false, s));
    BGPU_TRY(balloc(svdinfo, 16, true, s));
    BGPU_TRY(balloc(taken, 16, true, s));
    BGPU_TRY(balloc(ticket, 16, true, s));
    return BGPU_OK;
  }

  float* Ucol(uint32_t j) const { return U.as<float>() + (uint64_t)j * ldu; }
  float* Vcol(uint32_t j) const { return V.as<float>() + (uint64_t)j * ldv; }

  // One Lanczos step on stream `s` (the solve's own stream, or the stream
  // of a batch that launches this solve's kernels on it).
  int step(uint32_t j, cudaStream_t s) {
    float* y0p = y0.as<float>();
    float* y1p = y1.as<float>();
    float* partp = part.as<float>();
    float* coefp = coef.as<float>();
    float* coef2 = coefp + ps;
    float* Up = U.as<float>();
    BGPU_TRY(ev_begin(0));
    if (X.sell)
      BGPU_TRY(launch_xv_sell(X, Vcol(j), sd.as<float>(), y0p, s));
    else if (X.stream_ok && X.impl == 0)
      BGPU_TRY(launch_matvec_stream(X, Vcol(j), sd.as<float>(), y0p,
                                    derr.as<int>(), s));
    else
      BGPU_TRY(launch_matvec(X, Vcol(j), sd.as<float>(), y0p, s));
    BGPU_TRY(ev_end());
    launches += 1;
    const double col = (double)n * 4.0;
    BGPU_TRY(ev_begin(3));
    float* yfin;
    float* scalp = scal.as<float>();
    // the last update of the step finishes the norm in its last block:
    // B[j, j] = alpha, scal = {alpha, 1 / alpha}
    NormFinish fin;
    fin.B = B.as<double>();
    fin.m = m;
    fin.j = j;
    fin.scal = scalp;
    fin.counter = ticket.as<unsigned>();
    if (j == 0) {
      BGPU_TRY(launch_udots(Up, ldu, 0, y0p, nb, partp, ps, true, s));
      BGPU_TRY(launch_reduce_cols(partp, nb, ps, 1, coefp, s));
      BGPU_TRY(launch_uupdate(Up, ldu, 0, coefp, coefp, n, y0p, y1p, nb, partp,
                              ps, s, false, nullptr, nullptr, fin));
      launches += 3;
      yfin = y1p;
    } else {
      BGPU_TRY(launch_udots(Up, ldu, j, y0p, nb, partp, ps, true, s));
      BGPU_TRY(launch_reduce_cols(partp, nb, ps, j + 1, coefp, s));
      launches += 2;
      // algorithmic U-pass bytes (dots + update per pass): 2 n j 4 passes;
      // an adaptive solve adds its second passes from the device count at
      // the end
      reorth_bytes += 2.0 * j * (adaptive ? 1 : passes) * col;
      if (passes == 1) {
        BGPU_TRY(launch_uupdate(Up, ldu, j, coefp, coefp + j, n, y0p, y1p, nb,
                                partp, ps, s, false, nullptr, nullptr, fin));
        launches += 1;
        yfin = y1p;
      } else if (adaptive) {
        // One pass in place, as the reference (y0 <- y0 - (mean + U c1)),
        // with the block sums of |y1|^2 and |y0 - mean|^2; its last block
        // finishes alpha and writes their totals as the gate. The second
        // pass (dots, reduce, update, in place) runs only where the first
        // kept less than half of the squared norm, and then finishes alpha
        // again; its kernels return at once otherwise.
        float* gate = coef2 + m;  // past the second pass's j <= m - 1 dots
        NormFinish fin1 = fin;
        fin1.gate = gate;
        BGPU_TRY(launch_uupdate(Up, ldu, j, coefp, coefp + j, n, y0p, y0p, nb,
                                partp, ps, s, true, nullptr, nullptr, fin1));
        BGPU_TRY(launch_udots(Up, ldu, j, y0p, nb, partp, ps, false, s, gate));
        BGPU_TRY(launch_reduce_cols(partp, nb, ps, j, coef2, s, gate));
        BGPU_TRY(launch_uupdate(Up, ldu, j, coef2, nullptr, n, y0p, y0p, nb,
                                partp, ps, s, false, gate,
                                taken.as<unsigned long long>(), fin));
        launches += 4;
        yfin = y0p;
      } else {
        if (uupdate_dots_smem(j) <= 227 * 1024) {
          BGPU_TRY(launch_uupdate_dots(Up, ldu, j, coefp, coefp + j, n, y0p, y1p,
                                       partp, ps, s));
          BGPU_TRY(launch_reduce_cols(partp, uupdate_dots_blocks(n), ps, j, coef2, s));
          launches += 2;
        } else {
          BGPU_TRY(launch_uupdate(Up, ldu, j, coefp, coefp + j, n, y0p, y1p, nb,
                                  nullptr, ps, s));
          BGPU_TRY(launch_udots(Up, ldu, j, y1p, nb, partp, ps, false, s));
          BGPU_TRY(launch_reduce_cols(partp, nb, ps, j, coef2, s));
          launches += 3;
        }
        BGPU_TRY(launch_uupdate(Up, ldu, j, coef2, nullptr, n, y1p, y0p, nb,
                                partp, ps, s, false, nullptr, nullptr, fin));
        ++second_host;
        launches += 1;
        yfin = y0p;
      }
    }
    BGPU_TRY(ev_end());
    BGPU_TRY(ev_begin(1));
    if (X.sell)
      BGPU_TRY(launch_xt_sell(X, yfin, scalp + 1, Ucol(j), zpart.as<float>(), s));
    else if (X.stream_ok && X.impl == 0)
      BGPU_TRY(launch_rmatvec_stream(X, yfin, scalp + 1, Ucol(j),
                                     zpart.as<float>(), derr.as<int>(), s));
    else
      BGPU_TRY(launch_rmatvec_partials(X, yfin, scalp + 1, Ucol(j),
                                       zpart.as<float>(), s));
    BGPU_TRY(launch_reduce_panels_t(X, zpart.as<float>(), sd.as<float>(),
                                    zvec.as<float>(), s));
    launches += 1;
    BGPU_TRY(ev_end());
    BGPU_TRY(ev_begin(4));
    BGPU_TRY(launch_vstep(zvec.as<float>(), V.as<float>(), ldv, g, j, m, scalp,
                          B.as<double>(), rem.as<float>(), adaptive ? 0 : passes,
                          s));
    BGPU_TRY(ev_end());
    launches += 2;  // reduce_panels_t, vstep
    return BGPU_OK;
  }

  // Gene scaling (pca.pyx:790-799), start vector (pca.pyx:801-806) and the
  // first smax (pca.pyx:688). Synchronises: v0 and smax0 are host values.
  int begin(uint64_t seed) {
    BGPU_TRY(launch_gene_stddev(X, sdpart.as<double>(), sd.as<float>(), s));
    launches += 2;
    std::vector<float> v0(g);
    start_vector(seed, g, v0.data());
    BGPU_CUDA(cudaMemcpyAsync(Vcol(0), v0.data(), g * 4, cudaMemcpyHostToDevice, s));
    const float smax0 = 2.4221817809573368e-05f;  // pca.pyx:688
    BGPU_CUDA(cudaMemcpyAsync(smax.p, &smax0, 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaStreamSynchronize(s));
    return BGPU_OK;
  }

  // The restart's small SVD of B (pca.pyx:1178) after a cycle that started
  // at column kc.
  int restart_svd(uint32_t kc) {
    BGPU_TRY(ev_begin(2));
    if (svd_mode == 0 && kc >= 1) {
      // B = restart arrow + the cycle's Lanczos rows: the tail's SVD (t = m -
      // kc rows) and an FP64 secular-equation merge instead of a full SVD
      BGPU_TRY(launch_svd_merge(B.as<double>(), m, kc, Ub.as<float>(), Sb.as<float>(),
                                Vbt.as<float>(), ub_last.as<double>(), sb64.as<double>(),
                                tailw.p, mergew.p, oaw.as<double>(), svdwork.p,
                                kRefineSteps, s));
      launches += 7 + (m - kc > kMergeClosedTailMax ? 1 + 4 * kRefineSteps + 4 : 0);
      ++merged_svds;
    } else if (svd_mode == 1) {
      BGPU_TRY(launch_jacobi_svd(nullptr, B.as<double>(), m, Ub.as<float>(), Sb.as<float>(),
                                 Vbt.as<float>(), ub_last.as<double>(), sb64.as<double>(),
                                 svdwork.p, svdinfo.as<int>(), s));
      launches += 2;
    } else {
      BGPU_TRY(launch_b_to_float(B.as<double>(), m, Bf.as<float>(), s));
      BGPU_TRY(launch_jacobi_svd(Bf.as<float>(), nullptr, m, Ub.as<float>(), Sb.as<float>(),
                                 Vbt.as<float>(), nullptr, nullptr, svdwork.p,
                                 svdinfo.as<int>(), s));
      // FP64 Newton refinement of the FP32 factors: three quadratically
      // convergent steps separate the vectors of close singular values (the
      // Jacobi leaves pairs 6e-5 apart mixed by ~2 %), so the convergence test
      // reads FP64-accurate last entries of Ub, as with an FP64 SVD
      BGPU_TRY(launch_svd_refine(B.as<double>(), m, Ub.as<float>(), Sb.as<float>(),
                                 Vbt.as<float>(), ub_last.as<double>(), sb64.as<double>(),
                                 oaw.as<double>(), kRefineSteps, s));
      launches += 2 + 1 + 4 * kRefineSteps + 4;
    }
    BGPU_TRY(ev_end());
    return BGPU_OK;
  }

  // Convergence test and next k_current (pca.pyx:1180-1209) into st, then
  // st and the device error word copied to host_st / host_err (pinned
  // memory for a copy that does not block the host).
  int restart_check(uint32_t kc, RestartStatus* host_st, int* host_err) {
    BGPU_TRY(launch_restart_check(Ub.as<float>(), Sb.as<float>(), ub_last.as<double>(),
                                  sb64.as<double>(), m, k, rem.as<float>(), g, tol,
                                  smax.as<float>(), kc, B.as<double>(),
                                  st.as<RestartStatus>(),
                                  trace ? ratios.as<float>() : nullptr, s));
    // restart status and the device error word in one stream round trip (no
    // legacy-stream copies: those could wait on other streams' work)
    BGPU_CUDA(cudaMemcpyAsync(host_st, st.p, sizeof(RestartStatus), cudaMemcpyDeviceToHost,
                              s));
    BGPU_CUDA(cudaMemcpyAsync(host_err, derr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    return BGPU_OK;
  }

  // Restart rotation (pca.pyx:1210-1226): U <- U Ub[:, :kc], V <- V Vbt^T,
  // V[:, kc] = the remainder.
  int rotate(uint32_t kc) {
    BGPU_TRY(ev_begin(5));
    if (rot_mode == 2)
      BGPU_TRY(launch_gemm_tc(U.as<float>(), ldu, n, m, Ub.as<float>(), m, kc,
                              Unew.as<float>(), ldu, rotd.as<float>(), rotpiv.as<int>(),
                              derr.as<int>(), s));
    else
      BGPU_TRY(launch_gemm_ts(U.as<float>(), ldu, n, m, Ub.as<float>(), 1, m, nullptr, kc,
                              Unew.as<float>(), ldu, false, s));
    BGPU_TRY(launch_gemm_ts(V.as<float>(), ldv, g, m, Vbt.as<float>(), m, 1, nullptr, kc,
                            Vnew.as<float>(), ldv, false, s));
    BGPU_CUDA(cudaMemcpyAsync(Vnew.as<float>() + (uint64_t)kc * ldv, rem.p, g * 4,
                              cudaMemcpyDeviceToDevice, s));
    BGPU_TRY(ev_end());
    std::swap(U.p, Unew.p);
    std::swap(V.p, Vnew.p);
    launches += 2;
    rotation_bytes += ((double)n + g) * ((double)m + kc) * 4.0;
    return BGPU_OK;
  }

  // Final PCs (pca.pyx:1239-1255): pout = U . (Ub[:, :k] * Sb[:k]), C order.
  int final_pcs(float* pout) {
    BGPU_TRY(launch_gemm_ts(U.as<float>(), ldu, n, m, Ub.as<float>(), 1, m, Sb.as<float>(),
                            k, pout, k, true, s));
    launches += 1;
    return BGPU_OK;
  }
};

// Settings shared by the single and the batched drivers.
int check_opts(const Matrix& X, const bgpu_solve_opts& o) {
  BGPU_REQUIRE(o.k >= 1, BGPU_ERR_INVALID, "num_PCs (k) must be >= 1");
  BGPU_REQUIRE(o.subspace_size >= o.k, BGPU_ERR_INVALID,
               "subspace_size must be >= num_PCs");
  BGPU_REQUIRE(X.n >= 2 && X.g >= 2, BGPU_ERR_INVALID,
               "PCA needs at least two cells and two genes");
  BGPU_REQUIRE((uint64_t)o.subspace_size <= std::min<uint64_t>(X.n, X.g),
               BGPU_ERR_INVALID,
               "subspace_size must be <= min(num_cells, num_genes)");
  BGPU_REQUIRE(o.subspace_size <= 1024, BGPU_ERR_UNSUPPORTED,
               "subspace_size must be <= 1024");
  BGPU_REQUIRE(o.max_iterations >= 1, BGPU_ERR_INVALID,
               "max_iterations must be >= 1");
  BGPU_REQUIRE(o.tolerance > 0.f, BGPU_ERR_INVALID, "tolerance must be > 0");
  BGPU_REQUIRE(o.svd_mode <= 2, BGPU_ERR_INVALID, "svd_mode must be 0, 1 or 2");
  BGPU_REQUIRE(o.rotation_mode <= 2, BGPU_ERR_INVALID, "rotation_mode must be 0, 1 or 2");
  return BGPU_OK;
}

void configure(Solver& S, const bgpu_solve_opts& o) {
  S.profile = o.profile != 0;
  S.svd_mode = o.svd_mode;
  S.svd64 = o.svd_mode == 1;
  // subspaces beyond one shared-memory staging run as K / column chunks
  const bool tc_ok = o.subspace_size <= 1024;
  S.rot_mode = o.rotation_mode == 0 ? (tc_ok ? 2 : 1) : (int)o.rotation_mode;
  const char* et = std::getenv("BGPU_TRACE");
  S.trace = et && et[0] == '1';
}

}  // namespace

int irlba_solve(const Matrix& X, const bgpu_solve_opts& o, float* pcs,
                int pcs_on_device, float* svals, float* loadings,
                bgpu_solve_info* info, cudaStream_t s) {
  const auto t0 = std::chrono::steady_clock::now();
  BGPU_TRY(check_opts(X, o));
  BGPU_REQUIRE(pcs != nullptr, BGPU_ERR_INVALID, "PCs must not be NULL");

  Solver S(X, o, s);
  configure(S, o);
  BGPU_TRY(S.alloc());
  const uint32_t m = S.m, k = S.k, g = S.g;
  BGPU_TRY(S.begin(o.seed));

  uint32_t kc = 0, restarts = 0, steps = 0;
  RestartStatus last{};
  bool converged = false;
  for (uint32_t it = 0; it < o.max_iterations; ++it) {
    for (uint32_t j = kc; j < m; ++j) {
      if (o.cancel && *o.cancel) {
        cudaStreamSynchronize(s);
        set_error("solve cancelled");
        return BGPU_ERR_CANCELLED;
      }
      BGPU_TRY(S.step(j, s));
      ++steps;
    }
    ++restarts;
    BGPU_TRY(S.restart_svd(kc));
    int derr = 0;
    BGPU_TRY(S.restart_check(kc, S.hst.h, &derr));
    BGPU_CUDA(cudaStreamSynchronize(s));
    const int done_pool = S.cur;  // this restart's events, read after the rotation
    S.cur ^= 1;
    {
      BGPU_REQUIRE(derr == 0, BGPU_ERR_DEVICE,
                   "a bulk copy into shared memory did not complete within its "
                   "time limit (device error word " + std::to_string(derr) + ")");
    }
    last = *S.hst.h;
    if (S.trace) {
      std::vector<float> rat(k);
      int sw[2] = {0, 0};
      BGPU_CUDA(cudaMemcpyAsync(rat.data(), S.ratios.p, k * 4, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaMemcpyAsync(sw, S.svdinfo.p, 8, cudaMemcpyDeviceToHost, s));
      BGPU_CUDA(cudaStreamSynchronize(s));
      float worst_conv = 0.f, best_open = 1e30f;
      for (float r : rat) {
        if (r < 1.f) worst_conv = std::max(worst_conv, r);
        else best_open = std::min(best_open, r);
      }
      std::fprintf(stderr,
                   "[bgpu] restart %u steps %u kc %u -> %d nconv %d rn %.6g "
                   "smax %.6g sweeps %d conv-ratio max %.3g open-ratio min %.3g\n",
                   it, steps, kc, last.k_current, last.num_converged,
                   last.remainder_norm, last.smax, sw[0], worst_conv, best_open);
    }
    if (last.converged) { converged = true; break; }
    if (it + 1 == o.max_iterations) break;
    kc = (uint32_t)last.k_current;
    BGPU_TRY(S.rotate(kc));
    BGPU_TRY(S.ev_collect(done_pool));  // the rotation runs meanwhile
  }

  // Final PCs (pca.pyx:1239-1255): PCs = U . (Ub[:, :k] * Sb[:k]), C order.
  Buf pdev;
  float* pout = pcs;
  if (!pcs_on_device) {
    BGPU_TRY(balloc(pdev, S.n * k * 4, false, s));
    pout = pdev.as<float>();
  }
  BGPU_TRY(S.final_pcs(pout));
  if (!pcs_on_device)
    BGPU_CUDA(cudaMemcpyAsync(pcs, pout, S.n * k * 4, cudaMemcpyDeviceToHost, s));
  if (svals)
    BGPU_CUDA(cudaMemcpyAsync(svals, S.Sb.p, k * 4, cudaMemcpyDeviceToHost, s));
  Buf ldev;
  if (loadings) {
    BGPU_TRY(balloc(ldev, (size_t)g * k * 4, false, s));
    BGPU_TRY(launch_gemm_ts(S.V.as<float>(), S.ldv, g, m, S.Vbt.as<float>(), m, 1,
                            nullptr, k, ldev.as<float>(), k, true, s));
    BGPU_CUDA(cudaMemcpyAsync(loadings, ldev.p, (size_t)g * k * 4,
                              cudaMemcpyDeviceToHost, s));
  }
  unsigned long long taken[2] = {0, 0};
  if (S.adaptive)
    BGPU_CUDA(cudaMemcpyAsync(taken, S.taken.p, sizeof(taken), cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  S.reorth_bytes += 2.0 * (double)taken[1] * (double)S.n * 4.0;
  BGPU_TRY(S.ev_collect(0));  // whatever the last restarts left in the pools
  BGPU_TRY(S.ev_collect(1));
  if (info) {
    info->converged = converged ? 1 : 0;
    info->restarts = restarts;
    info->lanczos_steps = steps;
    info->rmatvecs = steps;
    info->num_converged = (uint32_t)last.num_converged;
    info->k_current = (uint32_t)last.k_current;
    info->seconds = std::chrono::duration<double>(
                        std::chrono::steady_clock::now() - t0).count();
    info->matvec_seconds = S.t_kind[0];
    info->rmatvec_seconds = S.t_kind[1];
    info->svd_seconds = S.t_kind[2];
    info->reorth_seconds = S.t_kind[3];
    info->vstep_seconds = S.t_kind[4];
    info->rotation_seconds = S.t_kind[5];
    info->matvec_bytes = matvec_bytes(X);
    info->rmatvec_bytes = rmatvec_bytes(X);
    info->reorth_bytes = S.reorth_bytes;
    info->rotation_bytes = S.rotation_bytes;
    info->kernel_launches = S.launches + (loadings ? 1 : 0);
    info->second_passes = S.adaptive ? taken[0] : S.second_host;
  }
  return BGPU_OK;
}

// ---------------------------------------------------------------------------
// Batched solves in lock step (per-subset PCAs of one shared matrix: brisc's
// SingleCell.pca() run on each subset, single_cell.py:11800-11808).
//
// Every solve keeps its own Solver (buffers, Lanczos state, restart
// decisions), but the ten kernels of a Lanczos step run as ONE launch each
// over every solve that is stepping (multi.cuh), on the batch's stream. A
// solve that finishes its cycle's last step runs its restart (small SVD,
// convergence test, rotation) on a stream of its own, concurrently with the
// other solves' steps; the host reads its restart status from pinned memory
// when the status event has completed and only then lets it step again. So
// the launches of a step are shared by all solves, and a solve's kernels
// compute exactly what its single solve computes: the results are
// bit-identical to irlba_solve's.
namespace {

struct BatchMember {
  std::unique_ptr<Solver> S;
  const bgpu_solve_opts* o = nullptr;
  cudaStream_t st = nullptr;  // restarts, rotations, final PCs
  cudaEvent_t ev_status = nullptr, ev_ready = nullptr;
  RestartStatus* hst = nullptr;  // pinned
  int* herr = nullptr;           // pinned
  Buf pdev;                      // final PCs when the caller's are host arrays
  uint32_t kc = 0, j = 0, it = 0, restarts = 0, steps = 0;
  RestartStatus last{};
  bool converged = false;
  bool wait_ready = false;  // the batch stream waits for ev_ready before the next step
  // kWaiting: restart issued, status not read; kRotating: rotation issued,
  // not yet complete (the solve steps again once the host has seen ev_ready,
  // so the batch stream never waits on a restarting solve's stream)
  enum { kReady, kWaiting, kRotating, kDone } state = kReady;
  double done_at = 0;  // seconds from the batch's start to its final PCs' launch
  std::chrono::steady_clock::time_point restart_at;  // when its restart was issued
};

struct StepLists {
  TaskList<XvTask> xv;
  TaskList<UdotsTask> d1, d2;
  TaskList<ReduceColsTask> r1, r2;
  TaskList<UupdateTask> u1, u2;
  TaskList<XtTask> xt;
  TaskList<ReducePanelsTask> rp;
  TaskList<VstepTask> vs;
  void clear() {
    task_list_init(xv);
    task_list_init(d1);
    task_list_init(d2);
    task_list_init(r1);
    task_list_init(r2);
    task_list_init(u1);
    task_list_init(u2);
    task_list_init(xt);
    task_list_init(rp);
    task_list_init(vs);
  }
};
constexpr uint32_t kStepLaunches = 10;

// Step j >= 1 of up to kMaxTasks adaptive solves as ten launches on s: the
// launches of Solver::step for an adaptive solve (X.v, U pass with its gated
// second pass, X^T.u, panel reduction, V step), each over all the solves.
int fused_step(StepLists& L, BatchMember* const* ms, uint32_t cnt, cudaStream_t s,
               cudaEvent_t* ev = nullptr) {
  L.clear();
  for (uint32_t i = 0; i < cnt; ++i) {
    Solver& S = *ms[i]->S;
    const Matrix& X = S.X;
    const uint32_t j = ms[i]->j;
    BGPU_REQUIRE(j >= 1 && j < S.m, BGPU_ERR_INVALID, "batch: a fused step needs 1 <= j < m");
    float* U = S.U.as<float>();
    float* y0 = S.y0.as<float>();
    float* part = S.part.as<float>();
    float* coef = S.coef.as<float>();
    float* coef2 = coef + S.ps;
    float* gate = coef2 + S.m;  // past the second pass's j <= m - 1 dots
    float* scal = S.scal.as<float>();
    NormFinish fin;
    fin.B = S.B.as<double>();
    fin.m = S.m;
    fin.j = j;
    fin.scal = scal;
    fin.counter = S.ticket.as<unsigned>();
    NormFinish fin1 = fin;
    fin1.gate = gate;
    const uint32_t nb = (uint32_t)S.nb;
    L.xv.add(XvTask{xv_view(X), S.Vcol(j), S.sd.as<float>(), y0}, xv_sell_ctas(X));
    L.d1.add(UdotsTask{U, S.ldu, y0, part, nullptr, j, S.ps, 1}, nb);
    L.r1.add(ReduceColsTask{part, S.nb, coef, nullptr, S.ps, j + 1},
             (uint32_t)ceil_div(j + 1, 32));
    L.u1.add(UupdateTask{U, S.ldu, coef, coef + j, S.n, y0, y0, part, nullptr, nullptr, fin1,
                         j, S.ps, 1},
             nb);
    L.d2.add(UdotsTask{U, S.ldu, y0, part, gate, j, S.ps, 0}, nb);
    L.r2.add(ReduceColsTask{part, S.nb, coef2, gate, S.ps, j}, (uint32_t)ceil_div(j, 32));
    L.u2.add(UupdateTask{U, S.ldu, coef2, nullptr, S.n, y0, y0, part, gate,
                         S.taken.as<unsigned long long>(), fin, j, S.ps, 0},
             nb);
    L.xt.add(XtTask{xt_view(X), y0, scal + 1, S.Ucol(j), S.zpart.as<float>()},
             xt_sell_ctas(X));
    L.rp.add(ReducePanelsTask{S.zpart.as<float>(), S.sd.as<float>(), S.zvec.as<float>(),
                              X.num_panels, S.g},
             reduce_panels_ctas(X));
    L.vs.add(VstepTask{S.zvec.as<float>(), S.V.as<float>(), S.ldv, scal, S.B.as<double>(),
                       S.rem.as<float>(), S.g, j, S.m, 0},
             kVStepCtas);
    S.reorth_bytes += 2.0 * j * (double)S.n * 4.0;  // first pass; second passes counted at the end
    S.launches += kStepLaunches;
  }
  // ev (tracing): kStepLaunches + 1 timing events around the launches
  int e = 0;
  auto mark = [&]() -> int {
    if (ev) BGPU_CUDA(cudaEventRecord(ev[e++], s));
    return BGPU_OK;
  };
  BGPU_TRY(mark());
  BGPU_TRY(launch_xv_sell_multi(L.xv, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_udots_multi(L.d1, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_reduce_cols_multi(L.r1, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_uupdate_multi(L.u1, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_udots_multi(L.d2, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_reduce_cols_multi(L.r2, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_uupdate_multi(L.u2, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_xt_sell_multi(L.xt, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_reduce_panels_multi(L.rp, s));
  BGPU_TRY(mark());
  BGPU_TRY(launch_vstep_multi(L.vs, s));
  BGPU_TRY(mark());
  return BGPU_OK;
}

bool batch_supported(const Matrix& X, const bgpu_solve_opts& o, std::string* why) {
  // m >= 2 keeps every cycle's steps at j >= 1 (k_current >= min(k, m - 1))
  if (o.subspace_size < 2) *why = "subspace_size is below 2";
  else if (!X.sell) *why = "the matrix is not in the sliced-ELL layout";
  else if (o.reorth_passes != 0) *why = "reorth_passes is not adaptive (0)";
  else if (!vstep_cluster_fits(X.g, o.subspace_size))
    *why = "the V step does not fit one thread-block cluster";
  else return true;
  return false;
}

}  // namespace

int irlba_solve_batch(const Matrix* const* Xs, const bgpu_solve_opts* opts, uint32_t count,
                      float* const* pcs, int pcs_on_device, float* const* svals,
                      bgpu_solve_info* infos, uint64_t* launches_out, cudaStream_t main) {
  const auto t0 = std::chrono::steady_clock::now();
  BGPU_REQUIRE(count >= 1, BGPU_ERR_INVALID, "batch: no solves");
  for (uint32_t i = 0; i < count; ++i) {
    BGPU_REQUIRE(Xs[i] && pcs[i], BGPU_ERR_INVALID, "batch: NULL matrix or PCs");
    BGPU_TRY(check_opts(*Xs[i], opts[i]));
    std::string why;
    BGPU_REQUIRE(batch_supported(*Xs[i], opts[i], &why), BGPU_ERR_UNSUPPORTED,
                 "batch: solve " + std::to_string(i) + ": " + why);
  }
  std::vector<BatchMember> M(count);
  void* pinned = nullptr;
  cudaEvent_t tick_ev[2] = {nullptr, nullptr};
  // on every return: no kernel of the batch is in flight when the solvers'
  // buffers go back to the pool, and the streams outlive their frees
  struct Guard {
    std::vector<BatchMember>& M;
    cudaStream_t main;
    void*& pinned;
    cudaEvent_t* tick_ev;
    ~Guard() {
      cudaStreamSynchronize(main);
      for (auto& b : M)
        if (b.st) cudaStreamSynchronize(b.st);
      for (auto& b : M) {
        b.S.reset();
        b.pdev.reset();
        if (b.st) {
          cudaStreamSynchronize(b.st);
          cudaStreamDestroy(b.st);
        }
        if (b.ev_status) cudaEventDestroy(b.ev_status);
        if (b.ev_ready) cudaEventDestroy(b.ev_ready);
      }
      for (int i = 0; i < 2; ++i)
        if (tick_ev[i]) cudaEventDestroy(tick_ev[i]);
      if (pinned) cudaFreeHost(pinned);
    }
  } guard{M, main, pinned, tick_ev};

  BGPU_CUDA(cudaMallocHost(&pinned, (size_t)count * (sizeof(RestartStatus) + 16)));
  for (int i = 0; i < 2; ++i)
    BGPU_CUDA(cudaEventCreateWithFlags(&tick_ev[i], cudaEventDisableTiming));
  // Restarts run at the device's highest stream priority: each is a chain of
  // small one-CTA kernels that a solve waits for, and the block scheduler
  // then places their CTAs ahead of the fused steps' queued CTAs instead of
  // behind them.
  int prio_low = 0, prio_high = 0;
  BGPU_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  const char* et = std::getenv("BGPU_TRACE");
  const bool trace = et && et[0] == '1';
  double t_sync = 0.0, lat_sum = 0.0, lat_max = 0.0;
  auto since = [&](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
  };
  for (uint32_t i = 0; i < count; ++i) {
    BatchMember& b = M[i];
    b.o = &opts[i];
    b.hst = reinterpret_cast<RestartStatus*>(pinned) + i;
    b.herr = reinterpret_cast<int*>(reinterpret_cast<char*>(pinned) +
                                    (size_t)count * sizeof(RestartStatus) + 16 * i);
    BGPU_CUDA(cudaStreamCreateWithPriority(&b.st, cudaStreamNonBlocking, prio_high));
    BGPU_CUDA(cudaEventCreateWithFlags(&b.ev_status, cudaEventDisableTiming));
    BGPU_CUDA(cudaEventCreateWithFlags(&b.ev_ready, cudaEventDisableTiming));
    b.S.reset(new Solver(*Xs[i], opts[i], b.st));
    configure(*b.S, opts[i]);
    b.S->profile = false;
    b.S->trace = false;
    BGPU_TRY(b.S->alloc());
    BGPU_TRY(b.S->begin(opts[i].seed));
    if (!pcs_on_device) BGPU_TRY(balloc(b.pdev, b.S->n * b.S->k * 4, false, b.st));
    BGPU_CUDA(cudaEventRecord(b.ev_ready, b.st));
    b.wait_ready = true;
  }

  std::unique_ptr<StepLists> lists(new StepLists());
  uint64_t fused_launches = 0, fused_member_steps = 0;
  uint32_t active = count;
  uint64_t tick = 0;

  auto start_restart = [&](BatchMember& b, cudaEvent_t after) -> int {
    BGPU_CUDA(cudaStreamWaitEvent(b.st, after, 0));
    ++b.restarts;
    BGPU_TRY(b.S->restart_svd(b.kc));
    BGPU_TRY(b.S->restart_check(b.kc, b.hst, b.herr));
    BGPU_CUDA(cudaEventRecord(b.ev_status, b.st));
    b.state = BatchMember::kWaiting;
    b.restart_at = std::chrono::steady_clock::now();
    return BGPU_OK;
  };
  auto finish = [&](BatchMember& b, uint32_t i) -> int {
    BGPU_TRY(b.S->final_pcs(pcs_on_device ? pcs[i] : b.pdev.as<float>()));
    b.done_at = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    b.state = BatchMember::kDone;
    --active;
    return BGPU_OK;
  };
  // a restart status has arrived: stop, or rotate and step again
  auto restarted = [&](BatchMember& b, uint32_t i) -> int {
    const double lat = since(b.restart_at);
    lat_sum += lat;
    lat_max = std::max(lat_max, lat);
    BGPU_REQUIRE(*b.herr == 0, BGPU_ERR_DEVICE,
                 "a bulk copy into shared memory did not complete within its "
                 "time limit (device error word " + std::to_string(*b.herr) + ")");
    b.last = *b.hst;
    if (b.last.converged) {
      b.converged = true;
      return finish(b, i);
    }
    if (b.it + 1 == b.o->max_iterations) return finish(b, i);
    b.kc = (uint32_t)b.last.k_current;
    BGPU_TRY(b.S->rotate(b.kc));
    BGPU_CUDA(cudaEventRecord(b.ev_ready, b.st));
    b.j = b.kc;
    ++b.it;
    b.state = BatchMember::kRotating;
    return BGPU_OK;
  };
  auto cancelled = [&]() {
    for (uint32_t i = 0; i < count; ++i)
      if (opts[i].cancel && *opts[i].cancel) return true;
    return false;
  };

  // step 0 of every solve (its own launch sequence: the first U pass has no
  // basis to orthogonalise against)
  for (uint32_t i = 0; i < count; ++i) {
    BatchMember& b = M[i];
    BGPU_CUDA(cudaStreamWaitEvent(main, b.ev_ready, 0));
    b.wait_ready = false;
    BGPU_TRY(b.S->step(0, main));
    b.j = 1;
    ++b.steps;
  }
  BGPU_CUDA(cudaEventRecord(tick_ev[0], main));
  ++tick;
  for (uint32_t i = 0; i < count; ++i)
    if (M[i].j == M[i].S->m) BGPU_TRY(start_restart(M[i], tick_ev[0]));

  // Restart statuses that have arrived (those solves rotate) and rotations
  // that have completed (those solves step again). *waiting: the solves
  // still restarting or rotating.
  auto poll = [&](uint32_t* waiting) -> int {
    *waiting = 0;
    for (uint32_t i = 0; i < count; ++i) {
      BatchMember& b = M[i];
      if (b.state != BatchMember::kWaiting && b.state != BatchMember::kRotating) continue;
      const cudaError_t e =
          cudaEventQuery(b.state == BatchMember::kWaiting ? b.ev_status : b.ev_ready);
      if (e == cudaErrorNotReady) {
        (void)cudaGetLastError();  // not an error: still in flight
        ++*waiting;
        continue;
      }
      BGPU_CUDA(e);
      if (b.state == BatchMember::kWaiting) {
        BGPU_TRY(restarted(b, i));
        if (b.state == BatchMember::kRotating) ++*waiting;
      } else {
        b.state = BatchMember::kReady;  // its rotation is complete
      }
    }
    return BGPU_OK;
  };

  std::vector<cudaEvent_t> kev;  // tracing: per-launch timing events
  struct KevGuard {
    std::vector<cudaEvent_t>& v;
    ~KevGuard() {
      for (cudaEvent_t e : v) cudaEventDestroy(e);
    }
  } kev_guard{kev};
  std::vector<BatchMember*> ready;
  while (active) {
    if (cancelled()) {
      set_error("solve cancelled");
      return BGPU_ERR_CANCELLED;
    }
    uint32_t waiting = 0;
    BGPU_TRY(poll(&waiting));
    // The host stays at most two steps ahead of the device: it waits for
    // the step before last, reading restart statuses meanwhile, so that a
    // solve whose restart finishes rejoins at the next step it issues.
    cudaEvent_t ev = tick_ev[tick & 1];
    if (tick >= 2) {
      const auto w0 = std::chrono::steady_clock::now();
      while (true) {
        const cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) BGPU_CUDA(e);
        (void)cudaGetLastError();
        BGPU_TRY(poll(&waiting));
      }
      t_sync += since(w0);
    }
    ready.clear();
    for (auto& b : M)
      if (b.state == BatchMember::kReady) ready.push_back(&b);
    if (ready.empty()) {
      if (!active) break;
      // every open solve is restarting: wait for the first status to arrive
      const auto w0 = std::chrono::steady_clock::now();
      while (waiting && ready.empty()) {
        BGPU_TRY(poll(&waiting));
        for (auto& b : M)
          if (b.state == BatchMember::kReady) ready.push_back(&b);
      }
      t_sync += since(w0);
      if (ready.empty()) continue;  // the last solves finished
    }
    for (BatchMember* b : ready)
      if (b->wait_ready) {
        BGPU_CUDA(cudaStreamWaitEvent(main, b->ev_ready, 0));
        b->wait_ready = false;
      }
    for (size_t c0 = 0; c0 < ready.size(); c0 += kMaxTasks) {
      const uint32_t cnt = (uint32_t)std::min<size_t>(kMaxTasks, ready.size() - c0);
      cudaEvent_t* tev = nullptr;
      if (trace) {  // timing events around this step's launches
        const size_t base = kev.size();
        kev.resize(base + kStepLaunches + 1);
        for (size_t q = base; q < kev.size(); ++q)
          BGPU_CUDA(cudaEventCreate(&kev[q]));
        tev = kev.data() + base;
      }
      BGPU_TRY(fused_step(*lists, ready.data() + c0, cnt, main, tev));
      fused_launches += kStepLaunches;
      fused_member_steps += cnt;
    }
    BGPU_CUDA(cudaEventRecord(ev, main));
    ++tick;
    for (BatchMember* b : ready) {
      ++b->j;
      ++b->steps;
      if (b->j == b->S->m) BGPU_TRY(start_restart(*b, ev));
    }
  }

  // results: host copies after every solve has finished
  std::vector<std::array<unsigned long long, 2>> taken(count);
  for (uint32_t i = 0; i < count; ++i) {
    BatchMember& b = M[i];
    Solver& S = *b.S;
    if (!pcs_on_device)
      BGPU_CUDA(cudaMemcpyAsync(pcs[i], b.pdev.p, S.n * S.k * 4, cudaMemcpyDeviceToHost, b.st));
    if (svals && svals[i])
      BGPU_CUDA(cudaMemcpyAsync(svals[i], S.Sb.p, S.k * 4, cudaMemcpyDeviceToHost, b.st));
    BGPU_CUDA(cudaMemcpyAsync(taken[i].data(), S.taken.p, 16, cudaMemcpyDeviceToHost, b.st));
  }
  uint64_t solo_launches = 0;
  for (uint32_t i = 0; i < count; ++i) {
    BatchMember& b = M[i];
    BGPU_CUDA(cudaStreamSynchronize(b.st));
    Solver& S = *b.S;
    S.reorth_bytes += 2.0 * (double)taken[i][1] * (double)S.n * 4.0;
    solo_launches += S.launches;
  }
  solo_launches -= fused_member_steps * kStepLaunches;
  if (launches_out) *launches_out = solo_launches + fused_launches;
  if (trace) {
    static const char* names[kStepLaunches] = {"xv", "udots", "reduce", "uupdate", "udots2",
                                               "reduce2", "uupdate2", "xt", "panels",
                                               "vstep"};
    double kt[kStepLaunches] = {};
    BGPU_CUDA(cudaStreamSynchronize(main));
    for (size_t q = 0; q + kStepLaunches < kev.size() + 1; q += kStepLaunches + 1)
      for (uint32_t i = 0; i < kStepLaunches; ++i) {
        float ms = 0.f;
        BGPU_CUDA(cudaEventElapsedTime(&ms, kev[q + i], kev[q + i + 1]));
        kt[i] += ms;
      }
    std::string line = "[bgpu] batch step kernels (ms):";
    for (uint32_t i = 0; i < kStepLaunches; ++i)
      line += std::string(" ") + names[i] + " " + std::to_string(kt[i]);
    std::fprintf(stderr, "%s\n", line.c_str());
    uint64_t restarts = 0;
    for (auto& b : M) restarts += b.restarts;
    std::fprintf(stderr,
                 "[bgpu] batch: %u solves, %llu ticks, %llu fused launches, %llu solo launches, "
                 "%.4f s, host waiting %.4f s, restart latency mean %.3g s max %.3g s over %llu\n",
                 count, (unsigned long long)tick, (unsigned long long)fused_launches,
                 (unsigned long long)solo_launches, since(t0), t_sync,
                 restarts ? lat_sum / (double)restarts : 0.0, lat_max,
                 (unsigned long long)restarts);
  }
  if (infos) {
    for (uint32_t i = 0; i < count; ++i) {
      BatchMember& b = M[i];
      Solver& S = *b.S;
      bgpu_solve_info& info = infos[i];
      info = bgpu_solve_info{};
      info.converged = b.converged ? 1 : 0;
      info.restarts = b.restarts;
      info.lanczos_steps = b.steps;
      info.rmatvecs = b.steps;
      info.num_converged = (uint32_t)b.last.num_converged;
      info.k_current = (uint32_t)b.last.k_current;
      info.seconds = b.done_at;  // the solve's latency within the batch
      info.matvec_bytes = matvec_bytes(S.X);
      info.rmatvec_bytes = rmatvec_bytes(S.X);
      info.reorth_bytes = S.reorth_bytes;
      info.rotation_bytes = S.rotation_bytes;
      info.kernel_launches = S.launches;  // each fused launch counted once per solve it served
      info.second_passes = taken[i][0];
    }
  }
  return BGPU_OK;
}

}  // namespace bgpu

// ===========================================================================
// C ABI
using namespace bgpu;

struct bgpu_matrix {
  Matrix m;
};

extern "C" const char* bgpu_last_error(void) { return get_error(); }

extern "C" const char* bgpu_version(void) { return "brisc_gb300 0.1.0 (sm_103a)"; }

extern "C" void bgpu_solve_opts_default(bgpu_solve_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->k = 50;
  o->subspace_size = 100;
  o->tolerance = 1e-6f;
  o->max_iterations = 100;
  o->seed = 0;
  o->chunk_size = 1024;
  o->reorth_passes = 0;
  o->rotation_mode = 0;
  o->cancel = nullptr;
  o->use_graphs = 0;
}

static void choose_shapes(Matrix& m) {
  const double avg = m.n ? (double)m.nnz / (double)m.n : 0.0;
  int G = 4;
  while (G < 32 && G * 8 < avg) G *= 2;  // about two 4-entry loads per lane
  m.spmv_group = G;
  m.spmv_blocks = num_sms() * 8;
  m.rmat_colgroup = m.g <= 512 ? 64 : 256;
  // X.v kernel: the segmented stream keeps every lane busy on short rows;
  // 8 lanes per row amortise their per-row work better on long ones.
  m.spmv_seg = m.csr_heads && avg < 64.0;
  // forced choices (bgpu_matrix_desc.kernels)
  if (m.kernels & BGPU_KERNELS_VECTOR) m.impl = 1;
  if (m.kernels & BGPU_KERNELS_XV_ROWS) m.spmv_seg = false;
  if (m.kernels & BGPU_KERNELS_XV_SEG) m.spmv_seg = m.csr_heads;
}

extern "C" int bgpu_matrix_create(bgpu_matrix** out, const bgpu_matrix_desc* d,
                                  void* stream) {
  BGPU_REQUIRE(out != nullptr, BGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  bgpu_matrix* h = new (std::nothrow) bgpu_matrix();
  BGPU_REQUIRE(h != nullptr, BGPU_ERR_ALLOC, "host allocation failed");
  int rc = matrix_build(&h->m, d, (cudaStream_t)stream);
  if (rc != BGPU_OK) {
    matrix_free(&h->m);
    delete h;
    return rc;
  }
  choose_shapes(h->m);
  *out = h;
  return BGPU_OK;
}

extern "C" int bgpu_matrix_create_rows(bgpu_matrix** out, const bgpu_matrix_desc* d,
                                       const int64_t* rows, uint64_t num_rows,
                                       void* stream) {
  BGPU_REQUIRE(out != nullptr, BGPU_ERR_INVALID, "out is NULL");
  *out = nullptr;
  bgpu_matrix* h = new (std::nothrow) bgpu_matrix();
  BGPU_REQUIRE(h != nullptr, BGPU_ERR_ALLOC, "host allocation failed");
  int rc = matrix_build_rows(&h->m, d, rows, num_rows, (cudaStream_t)stream);
  if (rc != BGPU_OK) {
    matrix_free(&h->m);
    delete h;
    return rc;
  }
  choose_shapes(h->m);
  *out = h;
  return BGPU_OK;
}

extern "C" int bgpu_matrix_destroy(bgpu_matrix* mat) {
  if (!mat) return BGPU_OK;
  matrix_free(&mat->m);
  delete mat;
  return BGPU_OK;
}

extern "C" int bgpu_matrix_bytes(const bgpu_matrix* mat, uint64_t* bytes) {
  BGPU_REQUIRE(mat && bytes, BGPU_ERR_INVALID, "NULL argument");
  *bytes = mat->m.bytes;
  return BGPU_OK;
}

extern "C" int bgpu_matrix_layout(const bgpu_matrix* mat, int* layout) {
  BGPU_REQUIRE(mat && layout, BGPU_ERR_INVALID, "NULL argument");
  *layout = mat->m.sell ? BGPU_LAYOUT_SELL
                        : (mat->m.mode == kFloat ? BGPU_LAYOUT_FLOAT : BGPU_LAYOUT_PANELS);
  return BGPU_OK;
}

extern "C" int bgpu_matrix_matvec(const bgpu_matrix* mat, const float* v,
                                  const float* sd, float* y, void* stream) {
  BGPU_REQUIRE(mat && v && y, BGPU_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (mat->m.sell) {
    BGPU_TRY(launch_xv_sell(mat->m, v, sd, y, s));
    BGPU_CUDA(cudaStreamSynchronize(s));
    return BGPU_OK;
  }
  if (!(mat->m.stream_ok && mat->m.impl == 0))
    return launch_matvec(mat->m, v, sd, y, s);
  Buf err;
  BGPU_TRY(balloc(err, 16, true, s));
  BGPU_TRY(launch_matvec_stream(mat->m, v, sd, y, err.as<int>(), s));
  int h = 0;
  BGPU_CUDA(cudaMemcpyAsync(&h, err.p, 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  BGPU_REQUIRE(h == 0, BGPU_ERR_DEVICE, "bulk copy wait timed out");
  return BGPU_OK;
}

extern "C" int bgpu_matrix_rmatvec(const bgpu_matrix* mat, const float* u,
                                   const float* sd, float* z, void* stream) {
  BGPU_REQUIRE(mat && u && z, BGPU_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  Buf part;
  BGPU_TRY(balloc(part, (size_t)mat->m.num_panels * mat->m.g * 4, false, s));
  Buf err;
  BGPU_TRY(balloc(err, 16, true, s));
  if (mat->m.sell)
    BGPU_TRY(launch_xt_sell(mat->m, u, nullptr, nullptr, part.as<float>(), s));
  else if (mat->m.stream_ok && mat->m.impl == 0)
    BGPU_TRY(launch_rmatvec_stream(mat->m, u, nullptr, nullptr, part.as<float>(),
                                   err.as<int>(), s));
  else
    BGPU_TRY(launch_rmatvec_partials(mat->m, u, nullptr, nullptr,
                                     part.as<float>(), s));
  BGPU_TRY(launch_reduce_panels_t(mat->m, part.as<float>(), sd, z, s));
  int h = 0;
  BGPU_CUDA(cudaMemcpyAsync(&h, err.p, 4, cudaMemcpyDeviceToHost, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  BGPU_REQUIRE(h == 0, BGPU_ERR_DEVICE, "bulk copy wait timed out");
  return BGPU_OK;
}

extern "C" int bgpu_matrix_gene_stddev(const bgpu_matrix* mat, float* sd,
                                       void* stream) {
  BGPU_REQUIRE(mat && sd, BGPU_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  Buf part;
  BGPU_TRY(balloc(part, (size_t)mat->m.num_panels * mat->m.g * 16, false, s));
  BGPU_TRY(launch_gene_stddev(mat->m, part.as<double>(), sd, s));
  BGPU_CUDA(cudaStreamSynchronize(s));
  return BGPU_OK;
}

extern "C" int bgpu_irlba(const bgpu_matrix* mat, const bgpu_solve_opts* opts,
                          float* pcs, int pcs_on_device, float* singular_values,
                          float* loadings, bgpu_solve_info* info, void* stream) {
  BGPU_REQUIRE(mat && opts, BGPU_ERR_INVALID, "NULL argument");
  return irlba_solve(mat->m, *opts, pcs, pcs_on_device, singular_values,
                     loadings, info, (cudaStream_t)stream);
}

extern "C" int bgpu_irlba_batch(const bgpu_matrix* const* mats,
                                const bgpu_solve_opts* opts, uint32_t count, float* const* pcs,
                                int pcs_on_device, float* const* singular_values,
                                bgpu_solve_info* infos, uint64_t* kernel_launches,
                                void* stream) {
  BGPU_REQUIRE(mats && opts && pcs, BGPU_ERR_INVALID, "NULL argument");
  std::vector<const Matrix*> xs(count);
  for (uint32_t i = 0; i < count; ++i) {
    BGPU_REQUIRE(mats[i], BGPU_ERR_INVALID, "batch: NULL matrix");
    xs[i] = &mats[i]->m;
  }
  return irlba_solve_batch(xs.data(), opts, count, pcs, pcs_on_device, singular_values, infos,
                           kernel_launches, (cudaStream_t)stream);
}

extern "C" int bgpu_rotate_basis(const float* A, uint64_t lda, uint64_t rows,
                                 uint32_t K, const float* Bm, uint64_t ldb,
                                 uint32_t ncols, float* C, uint64_t ldc, int mode,
                                 void* stream) {
  BGPU_REQUIRE(A && Bm && C && K >= 1 && ncols >= 1 && ncols <= K && lda >= rows &&
                   ldb >= K && ldc >= rows,
               BGPU_ERR_INVALID, "bad rotation arguments");
  BGPU_REQUIRE(mode == 1 || mode == 2, BGPU_ERR_INVALID, "mode must be 1 or 2");
  cudaStream_t s = (cudaStream_t)stream;
  if (mode == 1)
    BGPU_TRY(launch_gemm_ts(A, lda, rows, K, Bm, 1, ldb, nullptr, ncols, C, ldc,
                            false, s));
  else {
    Buf err, dwork, piv;
    BGPU_TRY(balloc(err, 16, true, s));
    BGPU_TRY(balloc(dwork, (size_t)K * ncols * 4, false, s));
    BGPU_TRY(balloc(piv, (size_t)ncols * 4, false, s));
    BGPU_TRY(launch_gemm_tc(A, lda, rows, K, Bm, ldb, ncols, C, ldc, dwork.as<float>(),
                            piv.as<int>(), err.as<int>(), s));
    int h = 0;
    BGPU_CUDA(cudaMemcpyAsync(&h, err.p, 4, cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaStreamSynchronize(s));
    BGPU_REQUIRE(h == 0, BGPU_ERR_DEVICE, "tensor-core rotation wait timed out");
  }
  BGPU_CUDA(cudaStreamSynchronize(s));
  return BGPU_OK;
}

extern "C" int bgpu_start_vector(uint64_t seed, uint32_t num_genes,
                                 float* out_host) {
  BGPU_REQUIRE(out_host && num_genes >= 1, BGPU_ERR_INVALID, "bad arguments");
  return start_vector(seed, num_genes, out_host);
}

extern "C" int bgpu_irlba_f32(const float* data_matvec, const void* indices_matvec,
                              const void* indptr_matvec, const float* data_rmatvec,
                              const void* indices_rmatvec, const void* indptr_rmatvec,
                              int index_type, uint64_t num_cells, uint32_t num_genes,
                              uint32_t k, uint32_t subspace_size, float tolerance,
                              uint32_t max_iterations, uint64_t seed,
                              int match_parallel, int is_csr, uint32_t num_threads,
                              uint64_t chunk_size, float* PCs, int* converged) {
  (void)data_rmatvec;
  (void)indices_rmatvec;
  (void)indptr_rmatvec;
  BGPU_REQUIRE(!match_parallel || num_threads == 1, BGPU_ERR_INVALID,
               "match_parallel must be False unless num_threads is 1");
  BGPU_REQUIRE(num_threads >= 1, BGPU_ERR_INVALID, "num_threads must be >= 1");
  BGPU_REQUIRE(chunk_size >= 1, BGPU_ERR_INVALID, "chunk_size must be >= 1");
  BGPU_REQUIRE(index_type == BGPU_INDEX_I32 || index_type == BGPU_INDEX_I64,
               BGPU_ERR_INVALID, "index_type must be BGPU_INDEX_I32 or _I64");
  cudaStream_t s = nullptr;
  const bool have_csr = is_csr || num_threads != 1 || match_parallel;
  const size_t isz = index_type == BGPU_INDEX_I64 ? 8 : 4;
  bgpu_matrix_desc d{};
  d.index_type = index_type;
  d.value_type = BGPU_VALUE_F32;
  d.num_cells = num_cells;
  d.num_genes = num_genes;
  d.norm_method = BGPU_NORM_NONE;
  Buf tp, ti, tx, cp, ci, cx;
  if (have_csr) {
    int64_t nnz = index_type == BGPU_INDEX_I64
                      ? ((const int64_t*)indptr_matvec)[num_cells]
                      : ((const int32_t*)indptr_matvec)[num_cells];
    d.indptr = indptr_matvec;
    d.indices = indices_matvec;
    d.values = data_matvec;
    d.on_device = 0;
    d.nnz = (uint64_t)nnz;
  } else {
    // The matvec arrays hold the CSC copy (num_genes columns): transpose it on
    // the GPU (a CSC of X is the CSR of X^T).
    int64_t nnz = index_type == BGPU_INDEX_I64
                      ? ((const int64_t*)indptr_matvec)[num_genes]
                      : ((const int32_t*)indptr_matvec)[num_genes];
    BGPU_TRY(balloc(cp, (num_genes + 1) * isz, false, s));
    BGPU_TRY(balloc(ci, nnz * isz, false, s));
    BGPU_TRY(balloc(cx, nnz * 4, false, s));
    BGPU_CUDA(cudaMemcpyAsync(cp.p, indptr_matvec, (num_genes + 1) * isz,
                              cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(ci.p, indices_matvec, nnz * isz, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaMemcpyAsync(cx.p, data_matvec, nnz * 4, cudaMemcpyHostToDevice, s));
    BGPU_TRY(balloc(tp, (num_cells + 1) * isz, false, s));
    BGPU_TRY(balloc(ti, nnz * isz, false, s));
    BGPU_TRY(balloc(tx, nnz * 4, false, s));
    BGPU_TRY(bgpu_csr_tocsc(num_genes, (uint32_t)std::min<uint64_t>(num_cells, 0xffffffffu),
                            cp.p, ci.p, cx.p, index_type, tp.p, ti.p, tx.p, s));
    d.indptr = tp.p;
    d.indices = ti.p;
    d.values = tx.p;
    d.on_device = 1;
    d.nnz = (uint64_t)nnz;
  }
  bgpu_matrix* mat = nullptr;
  BGPU_TRY(bgpu_matrix_create(&mat, &d, s));
  bgpu_solve_opts o;
  bgpu_solve_opts_default(&o);
  o.k = k;
  o.subspace_size = subspace_size;
  o.tolerance = tolerance;
  o.max_iterations = max_iterations;
  o.seed = seed;
  o.chunk_size = chunk_size;
  bgpu_solve_info info{};
  int rc = bgpu_irlba(mat, &o, PCs, 0, nullptr, nullptr, &info, s);
  bgpu_matrix_destroy(mat);
  if (rc == BGPU_OK && converged) *converged = info.converged;
  return rc;
}
