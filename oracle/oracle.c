/*
 * ORACLE -- test infrastructure only. CPU restatement of the reference's
 * algorithms on brisc's sparse-PCA path, used by tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline leg as the checker. Never linked into, or called
 * by, the product library.
 *
 * Pinned against the reference itself: tests/golden/ holds vectors produced by
 * the reference's own compiled modules (see tests/golden/make_golden.py), and
 * tests/test_oracle.py checks every function here against them.
 *
 * Serial restatements (single-thread code paths of the reference):
 *   oracle_rand / oracle_srand      brisc/cyutils.pyx:1153-1158, 1228-1232 (PCG32)
 *   oracle_random_normal            brisc/cyutils.pyx:1175-1191 (Box-Muller, float)
 *   oracle_start_vector             brisc/pca.pyx:683, 801-806 (+ norm, cyutils.pyx:1089-1094)
 *   oracle_csr_tocsc                brisc/cysparse.pyx:1199-1230 (serial branch)
 *   oracle_normalize_csr_*          brisc/normalize.pyx:9-127 (serial branch)
 *   oracle_clipped_stddev_csc       brisc/pca.pyx:51-86 (serial branch)
 *   oracle_thread_offsets           brisc/cyutils.pyx:900-920
 *
 * Build: cc -O2 -fPIC -shared oracle.c -o liboracle.so -lm (no -ffast-math:
 * the float arithmetic must round as written).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

uint32_t oracle_rand(uint64_t* state) {
  uint64_t x = *state;
  *state = x * 6364136223846793005ULL + 1442695040888963407ULL;
  uint32_t s = (uint32_t)((x ^ (x >> 18)) >> 27);
  uint32_t rot = (uint32_t)(x >> 59);
  return (s >> rot) | (s << ((0u - rot) & 31u));
}

uint64_t oracle_srand(uint64_t seed) {
  uint64_t state = seed + 1442695040888963407ULL;
  oracle_rand(&state);
  return state;
}

static float oracle_random_uniform(uint64_t* state) {
  /* `<float> rand(state) / UINT_MAX`: float / (float)UINT_MAX */
  return (float)oracle_rand(state) / (float)4294967295u;
}

float oracle_random_normal(uint64_t* state) {
  float u1, u2, r, theta;
  for (;;) {
    u1 = oracle_random_uniform(state);
    if (u1 != 0) break;
  }
  u2 = oracle_random_uniform(state);
  r = sqrtf(-2 * logf(u1));
  theta = (float)(2 * 3.14159265358979323846 * (double)u2);
  return r * cosf(theta);
}

void oracle_raw_rand(uint64_t seed, uint32_t count, uint32_t* out) {
  uint64_t st = oracle_srand(seed);
  for (uint32_t i = 0; i < count; ++i) out[i] = oracle_rand(&st);
}

void oracle_raw_normals(uint64_t seed, uint32_t count, float* out) {
  uint64_t st = oracle_srand(seed);
  for (uint32_t i = 0; i < count; ++i) out[i] = oracle_random_normal(&st);
}

void oracle_start_vector(uint64_t seed, uint32_t g, float* out) {
  uint64_t st = oracle_srand(seed);
  float nrm = 0, inv;
  for (uint32_t i = 0; i < g; ++i) out[i] = oracle_random_normal(&st);
  for (uint32_t i = 0; i < g; ++i) nrm += out[i] * out[i];
  nrm = sqrtf(nrm);
  inv = 1 / nrm;
  for (uint32_t i = 0; i < g; ++i) out[i] *= inv;
}

/* Stable CSR -> CSC, 4-byte values copied bit for bit (cysparse.pyx:1199-1230). */
void oracle_csr_tocsc(uint64_t n_row, uint32_t n_col, const int64_t* Ap,
                      const int64_t* Aj, const uint32_t* Ax, int64_t* Bp,
                      int64_t* Bi, uint32_t* Bx) {
  int64_t nnz = Ap[n_row], cumsum = 0;
  memset(Bp, 0, sizeof(int64_t) * (n_col + 1));
  for (int64_t e = 0; e < nnz; ++e) Bp[Aj[e]] += 1;
  for (uint32_t c = 0; c < n_col; ++c) {
    int64_t t = Bp[c];
    Bp[c] = cumsum;
    cumsum += t;
  }
  Bp[n_col] = nnz;
  for (uint64_t r = 0; r < n_row; ++r)
    for (int64_t e = Ap[r]; e < Ap[r + 1]; ++e) {
      int64_t c = Aj[e], d = Bp[c];
      Bi[d] = (int64_t)r;
      Bx[d] = Ax[e];
      Bp[c] += 1;
    }
  for (uint32_t c = n_col; c > 0; --c) Bp[c] = Bp[c - 1];
  Bp[0] = 0;
}

/* normalize_csr, serial branch (normalize.pyx:31-127). Counts are given as
 * double (exact for integer counts and float32 data); `qc` may be NULL.
 * Outputs the normalised values, the uint64 row sums, the inverse size factor
 * of every cell and (method 2) the per-cell post factor. */
void oracle_normalize_csr(const double* data, const int64_t* indptr,
                          uint64_t n, const uint8_t* qc, int method,
                          float* normalized, uint64_t* row_sums, float* isf,
                          float* post) {
  uint64_t total = 0, nqc = 0;
  float nf;
  for (uint64_t i = 0; i < n; ++i) {
    uint64_t s = 0;
    for (int64_t j = indptr[i]; j < indptr[i + 1]; ++j)
      s += (uint64_t)data[j];
    row_sums[i] = s;
    if (!qc || qc[i]) {
      total += s;
      nqc += 1;
    }
  }
  if (method == 0)
    nf = 10000;
  else
    nf = (float)total / (float)nqc;
  for (uint64_t i = 0; i < n; ++i) {
    volatile float f = nf / (float)row_sums[i];
    isf[i] = f;
    for (int64_t j = indptr[i]; j < indptr[i + 1]; ++j)
      normalized[j] = log1pf((float)data[j] * f);
  }
  if (method == 2) {
    float* nrs = (float*)malloc(sizeof(float) * (n ? n : 1));
    float new_total = 0;
    for (uint64_t i = 0; i < n; ++i) {
      float s = 0;
      for (int64_t j = indptr[i]; j < indptr[i + 1]; ++j) s += normalized[j];
      nrs[i] = s;
    }
    for (uint64_t i = 0; i < n; ++i)
      if (!qc || qc[i]) new_total += nrs[i];
    volatile float nf2v = new_total / (float)nqc;
    float nf2 = nf2v;
    for (uint64_t i = 0; i < n; ++i) {
      float q = nf2 / nrs[i];
      post[i] = q;
      for (int64_t j = indptr[i]; j < indptr[i + 1]; ++j) normalized[j] *= q;
    }
    free(nrs);
  }
}

/* clipped_stddev_csc, serial branch (pca.pyx:69-86): float32 sums. */
void oracle_clipped_stddev_csc(const float* data, const int64_t* indptr,
                               uint64_t n, uint32_t g, float clip_val,
                               float* sd) {
  float inv = (float)(1.0 / ((double)n * (double)(n - 1)));
  for (uint32_t c = 0; c < g; ++c) {
    float s = 0, ss = 0;
    for (int64_t i = indptr[c]; i < indptr[c + 1]; ++i) {
      float v = data[i];
      s += v;
      ss += v * v;
    }
    sd[c] = sqrtf(inv * ((float)n * ss - s * s));
    if (sd[c] < clip_val) sd[c] = clip_val;
  }
}

/* get_thread_offsets (cyutils.pyx:900-920): nnz-balanced row partition. */
void oracle_thread_offsets(const int64_t* indptr, uint64_t num_major,
                           uint32_t num_threads, uint32_t* offsets) {
  uint64_t per = (uint64_t)indptr[num_major] / num_threads;
  offsets[0] = 0;
  for (uint32_t t = 1; t < num_threads; ++t) {
    uint64_t target = t * per, lo = 0, hi = num_major + 1;
    while (lo < hi) { /* lower_bound over indptr[0 .. num_major] */
      uint64_t mid = (lo + hi) / 2;
      if ((uint64_t)indptr[mid] < target) lo = mid + 1; else hi = mid;
    }
    offsets[t] = (uint32_t)(lo < num_major ? lo : num_major);
  }
  offsets[num_threads] = (uint32_t)num_major;
}

/* Lemire's bounded integer (brisc/cyutils.pyx:1161-1172). */
static uint32_t oracle_randint(uint32_t bound, uint64_t* state) {
  uint64_t m = (uint64_t)oracle_rand(state) * (uint64_t)bound;
  uint32_t l = (uint32_t)m;
  if (l < bound) {
    uint32_t threshold = (0u - bound) % bound;
    while (l < threshold) {
      m = (uint64_t)oracle_rand(state) * (uint64_t)bound;
      l = (uint32_t)m;
    }
  }
  return (uint32_t)(m >> 32);
}

/* The "inside-out" Fisher-Yates cell order of brisc/harmonize.pyx:503-509,
 * from srand(seed). */
void oracle_fisher_yates(uint64_t seed, uint32_t n, uint32_t* order) {
  uint64_t state = oracle_srand(seed);
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t j = oracle_randint(i + 1, &state);
    order[i] = order[j];
    order[j] = i;
  }
}

/* The random k-means initialisation of brisc/kmeans.pyx:13-38: num_clusters
 * distinct cells drawn from srand(seed). */
void oracle_kmeans_init(uint64_t seed, uint32_t n, uint32_t nc, uint32_t* cells) {
  uint64_t state = oracle_srand(seed);
  uint64_t words = ((uint64_t)n + 63) / 64;
  uint64_t* bits = (uint64_t*)calloc(words, 8);
  for (uint32_t i = 0; i < nc; ++i) {
    for (;;) {
      uint32_t j = oracle_randint(n, &state);
      if (!(bits[j >> 6] & (1ull << (j & 63)))) {
        bits[j >> 6] |= 1ull << (j & 63);
        cells[i] = j;
        break;
      }
    }
  }
  free(bits);
}
