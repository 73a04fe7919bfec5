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
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
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
  ~Buf() { if (p) cudaFreeAsync(p, s); }
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

  int step(uint32_t j) {
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
};

}  // namespace

constexpr int kRefineSteps = 3;  // Newton steps after the FP32 Jacobi

int irlba_solve(const Matrix& X, const bgpu_solve_opts& o, float* pcs,
                int pcs_on_device, float* svals, float* loadings,
                bgpu_solve_info* info, cudaStream_t s) {
  const auto t0 = std::chrono::steady_clock::now();
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
  BGPU_REQUIRE(pcs != nullptr, BGPU_ERR_INVALID, "PCs must not be NULL");

  Solver S(X, o, s);
  S.profile = o.profile != 0;
  {
    BGPU_REQUIRE(o.svd_mode <= 2, BGPU_ERR_INVALID, "svd_mode must be 0, 1 or 2");
    S.svd_mode = o.svd_mode;
    S.svd64 = o.svd_mode == 1;
    BGPU_REQUIRE(o.rotation_mode <= 2, BGPU_ERR_INVALID, "rotation_mode must be 0, 1 or 2");
    // subspaces beyond one shared-memory staging run as K / column chunks
    const bool tc_ok = o.subspace_size <= 1024;
    S.rot_mode = o.rotation_mode == 0 ? (tc_ok ? 2 : 1) : (int)o.rotation_mode;
    const char* et = std::getenv("BGPU_TRACE");
    S.trace = et && et[0] == '1';
  }
  BGPU_TRY(S.alloc());
  const uint32_t m = S.m, k = S.k, g = S.g;

  // Gene scaling (pca.pyx:790-799) and start vector (pca.pyx:801-806).
  BGPU_TRY(launch_gene_stddev(X, S.sdpart.as<double>(), S.sd.as<float>(), s));
  S.launches += 2;
  {
    std::vector<float> v0(g);
    start_vector(o.seed, g, v0.data());
    BGPU_CUDA(cudaMemcpyAsync(S.Vcol(0), v0.data(), g * 4, cudaMemcpyHostToDevice, s));
    const float smax0 = 2.4221817809573368e-05f;  // pca.pyx:688
    BGPU_CUDA(cudaMemcpyAsync(S.smax.p, &smax0, 4, cudaMemcpyHostToDevice, s));
    BGPU_CUDA(cudaStreamSynchronize(s));  // v0, smax0 are host stack values
  }

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
      BGPU_TRY(S.step(j));
      ++steps;
    }
    ++restarts;
    BGPU_TRY(S.ev_begin(2));
    if (S.svd_mode == 0 && kc >= 1) {
      // B = restart arrow + the cycle's Lanczos rows: the tail's SVD (t = m -
      // kc rows) and an FP64 secular-equation merge instead of a full SVD
      BGPU_TRY(launch_svd_merge(S.B.as<double>(), m, kc, S.Ub.as<float>(),
                                S.Sb.as<float>(), S.Vbt.as<float>(),
                                S.ub_last.as<double>(), S.sb64.as<double>(), S.tailw.p,
                                S.mergew.p, S.oaw.as<double>(), S.svdwork.p,
                                kRefineSteps, s));
      S.launches += 7 + (m - kc > kMergeClosedTailMax ? 1 + 4 * kRefineSteps + 4 : 0);
      ++S.merged_svds;
    } else if (S.svd_mode == 1) {
      BGPU_TRY(launch_jacobi_svd(nullptr, S.B.as<double>(), m, S.Ub.as<float>(),
                                 S.Sb.as<float>(), S.Vbt.as<float>(),
                                 S.ub_last.as<double>(), S.sb64.as<double>(),
                                 S.svdwork.p, S.svdinfo.as<int>(), s));
      S.launches += 2;
    } else {
      BGPU_TRY(launch_b_to_float(S.B.as<double>(), m, S.Bf.as<float>(), s));
      BGPU_TRY(launch_jacobi_svd(S.Bf.as<float>(), nullptr, m, S.Ub.as<float>(),
                                 S.Sb.as<float>(), S.Vbt.as<float>(), nullptr,
                                 nullptr, S.svdwork.p, S.svdinfo.as<int>(), s));
      // FP64 Newton refinement of the FP32 factors: three quadratically
      // convergent steps separate the vectors of close singular values (the
      // Jacobi leaves pairs 6e-5 apart mixed by ~2 %), so the convergence test
      // reads FP64-accurate last entries of Ub, as with an FP64 SVD
      BGPU_TRY(launch_svd_refine(S.B.as<double>(), m, S.Ub.as<float>(), S.Sb.as<float>(),
                                 S.Vbt.as<float>(), S.ub_last.as<double>(),
                                 S.sb64.as<double>(), S.oaw.as<double>(), kRefineSteps, s));
      S.launches += 2 + 1 + 4 * kRefineSteps + 4;
    }
    BGPU_TRY(S.ev_end());
    BGPU_TRY(launch_restart_check(
        S.Ub.as<float>(), S.Sb.as<float>(), S.ub_last.as<double>(),
        S.sb64.as<double>(), m, k, S.rem.as<float>(), g,
        o.tolerance, S.smax.as<float>(), kc, S.B.as<double>(),
        S.st.as<RestartStatus>(), S.trace ? S.ratios.as<float>() : nullptr, s));
    // restart status and the device error word in one stream round trip (no
    // legacy-stream copies: those could wait on other streams' work)
    int derr = 0;
    BGPU_CUDA(cudaMemcpyAsync(S.hst.h, S.st.p, sizeof(RestartStatus),
                              cudaMemcpyDeviceToHost, s));
    BGPU_CUDA(cudaMemcpyAsync(&derr, S.derr.p, sizeof(int), cudaMemcpyDeviceToHost, s));
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
    // Restart rotation (pca.pyx:1210-1226): U <- U Ub[:, :kc], V <- V Vbt^T.
    BGPU_TRY(S.ev_begin(5));
    if (S.rot_mode == 2)
      BGPU_TRY(launch_gemm_tc(S.U.as<float>(), S.ldu, S.n, m, S.Ub.as<float>(), m, kc,
                              S.Unew.as<float>(), S.ldu, S.rotd.as<float>(),
                              S.rotpiv.as<int>(), S.derr.as<int>(), s));
    else
      BGPU_TRY(launch_gemm_ts(S.U.as<float>(), S.ldu, S.n, m, S.Ub.as<float>(), 1,
                              m, nullptr, kc, S.Unew.as<float>(), S.ldu, false, s));
    BGPU_TRY(launch_gemm_ts(S.V.as<float>(), S.ldv, g, m, S.Vbt.as<float>(), m,
                            1, nullptr, kc, S.Vnew.as<float>(), S.ldv, false, s));
    BGPU_CUDA(cudaMemcpyAsync(S.Vnew.as<float>() + (uint64_t)kc * S.ldv,
                              S.rem.p, g * 4, cudaMemcpyDeviceToDevice, s));
    BGPU_TRY(S.ev_end());
    BGPU_TRY(S.ev_collect(done_pool));  // the rotation runs meanwhile
    std::swap(S.U.p, S.Unew.p);
    std::swap(S.V.p, S.Vnew.p);
    S.launches += 2;
    S.rotation_bytes += ((double)S.n + g) * ((double)m + kc) * 4.0;
  }

  // Final PCs (pca.pyx:1239-1255): PCs = U . (Ub[:, :k] * Sb[:k]), C order.
  Buf pdev;
  float* pout = pcs;
  if (!pcs_on_device) {
    BGPU_TRY(balloc(pdev, S.n * k * 4, false, s));
    pout = pdev.as<float>();
  }
  BGPU_TRY(launch_gemm_ts(S.U.as<float>(), S.ldu, S.n, m, S.Ub.as<float>(), 1, m,
                          S.Sb.as<float>(), k, pout, k, true, s));
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
    info->kernel_launches = S.launches + 1 + (loadings ? 1 : 0);
    info->second_passes = S.adaptive ? taken[0] : S.second_host;
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
