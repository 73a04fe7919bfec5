/*
 * briscgpu.h -- C ABI of brisc_gb300, a GB300-native (sm_103a) implementation
 * of brisc's sparse-PCA hot path: SingleCell.pca() -> irlba().
 *
 * Plain C: pointers, sizes and an opaque CUDA stream (`void*`, a cudaStream_t;
 * NULL = the legacy default stream). No torch or numpy types cross this
 * boundary. Every function returns an int status (BGPU_OK == 0); on failure
 * bgpu_last_error() returns a message for the calling thread.
 *
 * Reference interfaces replaced (paths inside the brisc project):
 *   brisc/pca.pyx:661-678          irlba(...)                -> bgpu_irlba_f32, bgpu_irlba
 *   brisc/single_cell.py:11800-11808
 *                                  pca() on each cell subset -> bgpu_irlba_batch
 *   brisc/pca.pyx:440-475          matvec_csr_parallel_raw   -> bgpu_matrix_matvec
 *   brisc/pca.pyx:478-511          rmatvec_csc_parallel_raw  -> bgpu_matrix_rmatvec
 *   brisc/pca.pyx:51-103           clipped_stddev_csc        -> bgpu_matrix_gene_stddev
 *   brisc/pca.pyx:514-545          svd (LAPACK sgesdd)       -> bgpu_small_svd
 *   brisc/cyutils.pyx:1153-1232,
 *   brisc/pca.pyx:801-806          PCG32 + Box-Muller start  -> bgpu_start_vector
 *   brisc/normalize.pyx:9-268      normalize_csr             -> bgpu_normalize_csr,
 *                                                               bgpu_size_factors
 *   brisc/cysparse.pyx:1179-1295   csr_tocsc                 -> bgpu_csr_tocsc
 * and, either side of the path (the gene statistics feeding it, the first
 * consumers of the PCs):
 *   brisc/hvg.pyx:9-530            gene_mean_and_variance_*,
 *                                  clipped_sum_*             -> bgpu_gene_mean_var,
 *                                                               bgpu_clipped_sum
 *   brisc/kmeans.pyx:889-1433      kmeans                    -> bgpu_kmeans
 *   brisc/knn.pyx:13-515           knn_self                  -> bgpu_knn_self
 *   brisc/harmonize.pyx:244-266    normalize_rows            -> bgpu_normalize_rows
 *   brisc/harmonize.pyx:269-871    harmony                   -> bgpu_harmony
 *   brisc/hdf5.pyx:163,
 *   brisc/single_cell.py:1848-1883 h5py offsets + read_all_datasets
 *                                                            -> bgpu_h5ad_inspect,
 *                                                               bgpu_h5ad_read
 */
#ifndef BRISCGPU_H
#define BRISCGPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define BGPU_API __attribute__((visibility("default")))
#else
#define BGPU_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  BGPU_OK = 0,
  BGPU_ERR_INVALID = 1,      /* bad argument (mirrors the reference's ValueError) */
  BGPU_ERR_CUDA = 2,         /* a CUDA runtime call failed                        */
  BGPU_ERR_ALLOC = 3,        /* device allocation failed                          */
  BGPU_ERR_UNSUPPORTED = 4,  /* input outside the supported layout limits         */
  BGPU_ERR_CANCELLED = 5,    /* the cancel flag was raised between restarts       */
  BGPU_ERR_DEVICE = 6,       /* a kernel reported an error status word            */
  BGPU_ERR_IO = 7            /* reading a file failed                             */
};

/* ---- element types of caller arrays ------------------------------------ */
enum {
  BGPU_INDEX_I32 = 0,  /* int32 indptr / indices (signed_integer = int)        */
  BGPU_INDEX_I64 = 1   /* int64 indptr / indices (signed_integer = long long)  */
};
enum {
  BGPU_VALUE_U16 = 0,  /* raw counts, uint16                                   */
  BGPU_VALUE_U32 = 1,  /* raw counts, uint32 (must be <= 65535)                */
  BGPU_VALUE_I32 = 2,  /* raw counts, int32  (must be in [0, 65535])           */
  BGPU_VALUE_F32 = 3,  /* float32: already-normalised values, or float counts  */
  /* the HVG statistics below also take the reference's other `numeric` types */
  BGPU_VALUE_I64 = 4,  /* int64 counts                                          */
  BGPU_VALUE_U64 = 5,  /* uint64 counts                                         */
  BGPU_VALUE_F64 = 6   /* float64 counts                                        */
};

/* Normalisation applied to the stored values (brisc/normalize.pyx method_number).
 * BGPU_NORM_NONE: values are already normalised float32 (what pca() receives
 * after SingleCell.normalize()). The other three fuse the normalisation into
 * every product: value = log1pf(count * isf[cell]) (* post[cell] for method 2). */
enum {
  BGPU_NORM_NONE = -1,
  BGPU_NORM_LOGCP10K = 0,
  BGPU_NORM_LOG1PPF = 1,
  BGPU_NORM_PFLOG1PPF = 2
};

BGPU_API const char* bgpu_last_error(void);
BGPU_API const char* bgpu_version(void);

/* ---- device-resident matrix -------------------------------------------- */
/* A cells x genes CSR matrix laid out for the solver: a packed CSR copy for
 * X.v and a row-panel transposed (CSC) copy for X^T.u, both built on the GPU,
 * plus per-cell size factors for the fused normalisation. */
typedef struct bgpu_matrix bgpu_matrix;

typedef struct bgpu_matrix_desc {
  const void* indptr;        /* num_cells + 1 entries, index_type              */
  const void* indices;       /* nnz gene indices, index_type                   */
  const void* values;        /* nnz values, value_type                         */
  int index_type;            /* BGPU_INDEX_*                                   */
  int value_type;            /* BGPU_VALUE_*                                   */
  int on_device;             /* 1: pointers are device memory; 0: host memory  */
  uint64_t num_cells;
  uint32_t num_genes;
  uint64_t nnz;
  int norm_method;           /* BGPU_NORM_*                                    */
  /* Per-cell inverse size factors (float32, num_cells, same memory space as the
   * arrays above). Required for methods 0-2: the reference computes them from
   * row sums over ALL genes before HVG subsetting (brisc/normalize.pyx:36-81),
   * so the caller supplies them (bgpu_size_factors computes them on the GPU). */
  const float* inv_size_factors;
  /* Per-cell post-log factors for BGPU_NORM_PFLOG1PPF (normalize.pyx:231-268);
   * NULL otherwise. */
  const float* post_factors;
  /* Rows per transposed panel (power of two in [1024, 65536]); 0 = automatic. */
  uint32_t panel_rows;
  /* Product kernels: 0 = automatic (the sliced-ELL layout for counts with at
   * most 4096 genes, else the panel layout with rules on the mean entries per
   * row). Nonzero: an OR of BGPU_KERNELS_* forcing a choice, for comparing
   * layouts; every choice computes the same products to FP32 rounding, in
   * its own fixed order. No counterpart in the reference. */
  uint32_t kernels;
  /* Rows per X^T.u panel of the sliced-ELL layout: 0 = automatic (one wave
   * of CTAs over the panels), else a multiple of 32 in [128, 512]. Longer
   * panels make fewer, longer (panel, gene) sums: what batched subsets want,
   * whose CTAs come from every subset at once. The panel rows set the order
   * of the per-gene sums, so two layouts of one matrix give the same bits
   * when they have the same panel rows. No counterpart in the reference. */
  uint32_t sell_panel_rows;
} bgpu_matrix_desc;

enum {
  BGPU_KERNELS_PANELS = 1,   /* panel layout even where sliced-ELL applies    */
  BGPU_KERNELS_NATURAL = 2,  /* panel X.v rows in natural, not length, order  */
  BGPU_KERNELS_WORDS32 = 4,  /* panel X^T.u over the 32-bit words             */
  BGPU_KERNELS_XV_ROWS = 8,  /* panel X.v: 8 lanes per row                    */
  BGPU_KERNELS_XV_SEG = 16,  /* panel X.v: segmented stream (needs row heads) */
  BGPU_KERNELS_VECTOR = 32   /* register-vector kernels instead of tables     */
};

BGPU_API int bgpu_matrix_create(bgpu_matrix** out, const bgpu_matrix_desc* desc,
                       void* stream);
/* The layout of the row subset X[rows, :] of the matrix `desc` describes
 * (rows: int64 cell indices, in the memory space of desc's arrays, any order,
 * num_rows >= 1). The subset is its own matrix: a solve on it centres and
 * scales genes over the subset's cells only, as a PCA of one cell type
 * (SingleCell.pca() on a subset, brisc/single_cell.py:11800-11808). Used for
 * batched per-subset PCAs over one shared matrix. */
BGPU_API int bgpu_matrix_create_rows(bgpu_matrix** out, const bgpu_matrix_desc* desc,
                                     const int64_t* rows, uint64_t num_rows,
                                     void* stream);
/* Releases the matrix's device memory, stream-ordered on the stream it was
 * created on (that stream must still exist). Call it once no queued work uses
 * the matrix any more (bgpu_irlba returns only after its work has completed). */
BGPU_API int bgpu_matrix_destroy(bgpu_matrix* mat);
/* Device bytes held by the matrix layout. */
BGPU_API int bgpu_matrix_bytes(const bgpu_matrix* mat, uint64_t* bytes);

/* Which layout (and so which product kernels) the matrix was built with. No
 * counterpart in the reference (its products read the caller's CSR/CSC). */
enum {
  BGPU_LAYOUT_PANELS = 0,  /* counts: packed CSR words + row-panel transpose   */
  BGPU_LAYOUT_SELL = 1,    /* counts, <= 4096 genes: sliced-ELL rows for X.v
                              and sliced-ELL (panel, gene) segments for X^T.u  */
  BGPU_LAYOUT_FLOAT = 2    /* pre-normalised float32 values                    */
};
BGPU_API int bgpu_matrix_layout(const bgpu_matrix* mat, int* layout);

/* y = X . (v / sd)   (brisc/pca.pyx:440-475; no centring). Device pointers.
 * sd may be NULL (treated as all ones). y has num_cells entries. */
BGPU_API int bgpu_matrix_matvec(const bgpu_matrix* mat, const float* v, const float* sd,
                       float* y, void* stream);
/* z = (X^T . u) / sd  (brisc/pca.pyx:478-511; u assumed zero-mean by the
 * caller, as there). Device pointers; sd may be NULL. */
BGPU_API int bgpu_matrix_rmatvec(const bgpu_matrix* mat, const float* u, const float* sd,
                        float* z, void* stream);
/* Clipped per-gene sample standard deviation of the normalised values
 * (brisc/pca.pyx:51-103, clip 1e-8 as pca.pyx:687). Accumulated in FP64. */
BGPU_API int bgpu_matrix_gene_stddev(const bgpu_matrix* mat, float* sd, void* stream);

/* ---- IRLBA solve ------------------------------------------------------- */
typedef struct bgpu_solve_opts {
  uint32_t k;                /* num_PCs                                         */
  uint32_t subspace_size;    /* m (>= k, <= min(num_cells, num_genes))          */
  float tolerance;           /* relative residual tolerance                      */
  uint32_t max_iterations;   /* restarts                                         */
  uint64_t seed;             /* PCG32 seed of the start vector                   */
  uint64_t chunk_size;       /* accepted for signature parity: the GPU reduces
                                over fixed 1024-row blocks whatever its value   */
  uint32_t reorth_passes;    /* U-side Gram-Schmidt per Lanczos step:
                                0 = adaptive (default): one classical pass as
                                the reference, and a second one only at steps
                                where the first removed more than half of the
                                vector's squared norm ("twice is enough",
                                Kahan-Parlett); 1 = one pass always;
                                2 = two passes always (CGS2). The V side
                                follows the same rule.                          */
  uint32_t rotation_mode;    /* restart rotation of U: 0 = default (tensor
                                cores), 1 = FP32 SIMT GEMM, 2 = tcgen05 3 x
                                BF16 split GEMM with FP32 accumulation and the
                                dominant column of each rotation column added
                                in FP32 (K / column chunks beyond 112 / 128)   */
  volatile int32_t* cancel;  /* host flag polled between Lanczos steps; may be
                                NULL (replaces PyErr_CheckSignals, pca.pyx:1173) */
  int use_graphs;            /* reserved for CUDA-graph replay of the Lanczos
                                steps; accepted and currently ignored            */
  int profile;               /* time the sparse products and the small SVD with
                                CUDA events (fills the *_seconds fields)         */
  uint32_t svd_mode;         /* restart SVD of B (replaces sgesdd, pca.pyx:1178):
                                0 = default: at the first restart FP32 Jacobi
                                + FP64 Newton refinement of the whole B; at
                                every later restart an FP64 secular-equation
                                merge of the restart arrow with the cycle's
                                Lanczos rows (only those t = m - kc rows get a
                                small SVD of their own); 1 = FP64 Jacobi of
                                the whole B every restart; 2 = FP32 Jacobi +
                                FP64 Newton of the whole B every restart. B
                                and the convergence test are FP64 always.    */
} bgpu_solve_opts;

typedef struct bgpu_solve_info {
  int32_t converged;
  uint32_t restarts;         /* IRLBA iterations run                             */
  uint32_t lanczos_steps;    /* X.v products                                      */
  uint32_t rmatvecs;         /* X^T.u products                                    */
  uint32_t num_converged;    /* at the last restart                               */
  uint32_t k_current;        /* at the last restart                               */
  double seconds;            /* wall time of the solve (device work included)    */
  /* Filled when opts.profile is set (CUDA events around each launch group): */
  double matvec_seconds;     /* summed X.v kernel time                            */
  double rmatvec_seconds;    /* summed X^T.u kernel time (panel partials)         */
  double svd_seconds;        /* summed small-SVD time                             */
  double reorth_seconds;     /* summed U-pass time (dots, updates, norms)         */
  double vstep_seconds;      /* summed V-side step time                           */
  double rotation_seconds;   /* summed restart-rotation GEMM time                 */
  /* Bytes the device layout streams in one X.v / X^T.u launch (4 per
   * stored entry in the counts layout, plus offsets, factors and vectors): */
  double matvec_bytes;
  double rmatvec_bytes;
  double reorth_bytes;       /* summed algorithmic U-pass bytes, 2 n j 4 per
                                Gram-Schmidt pass and step                     */
  double rotation_bytes;     /* summed (n + g)(m + kc) 4 of the restart rotations */
  uint64_t kernel_launches;  /* kernels launched by this solve                    */
  uint64_t second_passes;    /* Lanczos steps that ran a second U-side pass       */
} bgpu_solve_info;

BGPU_API void bgpu_solve_opts_default(bgpu_solve_opts* opts);

/* Solve on a device-resident matrix. `pcs` is num_cells x k, C order, float32
 * (brisc/pca.pyx:678 `PCs`); pcs_on_device selects its memory space.
 * singular_values (k floats, host) and loadings (num_genes x k, C order,
 * host; the right singular vectors, V . Vbt^T[:, :k]) may be NULL. */
BGPU_API int bgpu_irlba(const bgpu_matrix* mat, const bgpu_solve_opts* opts,
               float* pcs, int pcs_on_device, float* singular_values,
               float* loadings, bgpu_solve_info* info, void* stream);

/* `count` independent solves (per-subset PCAs of one shared matrix, as
 * SingleCell.pca() run on each subset, brisc/single_cell.py:11800-11808) in
 * lock step: each kernel of a Lanczos step is one launch over every solve
 * that is stepping; each solve restarts (small SVD, convergence test,
 * rotation) on a stream of its own while the others step. mats[i], opts[i],
 * pcs[i] and singular_values[i] (may be NULL, or hold NULLs) are solve i's,
 * as for bgpu_irlba (no loadings); infos (may be NULL) receives count
 * records. Every solve's PCs and singular values are bit-identical to its
 * bgpu_irlba solve. *kernel_launches (may be NULL) receives the launches
 * the batch made. BGPU_ERR_UNSUPPORTED (nothing run) unless every matrix is
 * in the sliced-ELL layout (BGPU_LAYOUT_SELL), every opts.subspace_size is
 * >= 2 and every opts.reorth_passes is 0 (adaptive). infos[i].seconds is the
 * time from the call to solve i's last kernel launch. Synchronises `stream`
 * before returning. */
BGPU_API int bgpu_irlba_batch(const bgpu_matrix* const* mats, const bgpu_solve_opts* opts,
               uint32_t count, float* const* pcs, int pcs_on_device,
               float* const* singular_values, bgpu_solve_info* infos,
               uint64_t* kernel_launches, void* stream);

/* Drop-in for brisc/pca.pyx:661-678 with the same arguments and meaning: host
 * arrays, float32 normalised values, CSR for the matvec and (optionally) CSC
 * for the rmatvec. The CSC arrays may be NULL: the transpose is built on the
 * GPU either way. `match_parallel` and `num_threads` are validated as the
 * reference's caller does (single_cell.py:11833-11840) and otherwise unused;
 * `is_csr` = 0 means the matvec arrays hold a CSC copy (the reference's
 * num_threads=1 CSC path), which is transposed on the GPU. Writes *converged. */
BGPU_API int bgpu_irlba_f32(const float* data_matvec, const void* indices_matvec,
                   const void* indptr_matvec, const float* data_rmatvec,
                   const void* indices_rmatvec, const void* indptr_rmatvec,
                   int index_type, uint64_t num_cells, uint32_t num_genes,
                   uint32_t k, uint32_t subspace_size, float tolerance,
                   uint32_t max_iterations, uint64_t seed, int match_parallel,
                   int is_csr, uint32_t num_threads, uint64_t chunk_size,
                   float* PCs, int* converged);

/* ---- path building blocks (parity-testable individually) ---------------- */

/* V[:, 0] of brisc/pca.pyx:801-806: `num_genes` Box-Muller normals from the
 * reference's PCG32 (cyutils.pyx:1153-1232), normalised. Host function. */
BGPU_API int bgpu_start_vector(uint64_t seed, uint32_t num_genes, float* out_host);

/* Restart rotation C = A . Bm[:, :ncols] (brisc/pca.pyx:1210-1215, the
 * reference's matmul_nn_f_out at pca.pyx:578-616, U <- U . Ub[:, :kc]).
 * Device pointers, all column-major: A rows x K (lda), Bm K x >= ncols (ldb),
 * C rows x ncols (ldc). mode 1: FP32 SIMT; mode 2: tensor cores (tcgen05,
 * 3 x BF16 split operands, six cross products accumulated in FP32; a column
 * of Bm dominated by one entry (|entry| >= 1/2) is applied as that column of
 * A, added in FP32, plus the tensor-core product with the rest; ncols > 128
 * runs as column chunks, K beyond ~230 as K chunks added in a fixed order;
 * A's columns must start 16-byte aligned: A aligned, lda a multiple of 4).
 * Synchronous. */
BGPU_API int bgpu_rotate_basis(const float* A, uint64_t lda, uint64_t rows,
                               uint32_t K, const float* Bm, uint64_t ldb,
                               uint32_t ncols, float* C, uint64_t ldc, int mode,
                               void* stream);

/* SVD of one m x (m+1) column-major float32 matrix B (the reference's
 * `svd(B, Ub, Sb, Vbt, ...)`, pca.pyx:531-545, JOBZ='S'). Device pointers:
 * Ub m x m, Sb m (descending), Vbt m x (m+1), all column-major. */
BGPU_API int bgpu_small_svd(const float* B, uint32_t m, float* Ub, float* Sb,
                   float* Vbt, void* stream);

/* The same SVD as bgpu_small_svd, for callers that cannot allocate device
 * memory: their process gives all of it to its own pool allocator, or they run
 * in a loop where cudaMalloc/cudaFree would stall the device. No counterpart in
 * the reference (its sgesdd call allocates host workspace, pca.pyx:514-528).
 * Allocates nothing: its scratch is a fixed device array inside the library
 * (about 1.6 MB per GPU that loads it, held until exit). m <= 256, else
 * BGPU_ERR_INVALID. The first call on each device looks the array up. Calls
 * share the array: two whose work overlaps on the GPU race. The call
 * synchronises `stream` before it returns (the SVD has completed), so it
 * cannot be captured into a CUDA graph. */
BGPU_API int bgpu_small_svd_noalloc(const float* B, uint32_t m, float* Ub,
                                    float* Sb, float* Vbt, void* stream);

/* Per-cell normalisation factors (brisc/normalize.pyx:9-268), on the GPU,
 * over a full-gene counts CSR (device pointers). Writes inverse size factors
 * `isf` (num_cells floats) and, for method 2, `post` (num_cells floats).
 * qc_mask (num_cells bytes, nonzero = passed) may be NULL. row_sums (uint64,
 * num_cells) may be NULL. */
BGPU_API int bgpu_size_factors(const void* indptr, int index_type, const void* values,
                      int value_type, uint64_t num_cells, int method,
                      const uint8_t* qc_mask, float* isf, float* post,
                      uint64_t* row_sums, void* stream);

/* Materialised normalisation (brisc/normalize.pyx:9 normalize_csr): writes
 * normalized[nnz] = log1pf(count * isf[row]) (* post[row]). Device pointers. */
BGPU_API int bgpu_normalize_csr(const void* indptr, int index_type, const void* values,
                       int value_type, uint64_t num_cells, const float* isf,
                       const float* post, float* normalized, void* stream);

/* Stable CSR -> CSC transpose (brisc/cysparse.pyx:1179-1295): rows ascending
 * within each column. Device pointers; Ap/Aj/Bp/Bi share index_type; Ax/Bx
 * are 4-byte values (float32/int32/uint32) copied bit for bit. */
BGPU_API int bgpu_csr_tocsc(uint64_t n_row, uint32_t n_col, const void* Ap,
                   const void* Aj, const void* Ax, int index_type, void* Bp,
                   void* Bi, void* Bx, void* stream);

/* ---- highly-variable-gene statistics (brisc/hvg.pyx) -------------------- */
/* A raw count matrix in CSR (cells x genes) or CSC (genes x cells), with the
 * subset of cells the reference's functions take. The counts are cast to
 * uint64 as the reference casts them (values must be non-negative) and summed
 * exactly; the results are bit-identical to the reference's. */
typedef struct bgpu_hvg_input {
  const void* data;          /* nnz values, value_type (any BGPU_VALUE_*)       */
  int value_type;
  const void* indices;       /* nnz gene (CSR) or cell (CSC) indices            */
  const void* indptr;        /* num_major + 1 offsets                           */
  int index_type;            /* BGPU_INDEX_*                                    */
  uint64_t nnz;
  uint64_t num_major;        /* rows (CSR) or genes (CSC) of indptr             */
  int is_csr;
  uint32_t num_genes;        /* num_dataset_genes (CSR; for CSC mean/variance
                                the leading genes of indptr)                   */
  const int64_t* cell_indices; /* CSR subset (may be NULL)                      */
  uint64_t num_cell_indices;
  const int8_t* cell_mask;   /* CSC subset, one byte per cell (may be NULL)     */
  uint64_t cell_mask_len;
  int on_device;             /* 1: every array here and every output is a
                                device pointer; 0: host arrays                 */
} bgpu_hvg_input;

/* Per-gene mean, sample variance and nonzero count (float, float, uint32;
 * num_genes each). Replaces gene_mean_and_variance_csr (brisc/hvg.pyx:9-139:
 * without cell_indices every stored entry counts, with it the first
 * num_cells listed cells) and gene_mean_and_variance_csc (hvg.pyx:142-252,
 * cells where cell_mask is nonzero). num_cells divides as in the reference. */
BGPU_API int bgpu_gene_mean_var(const bgpu_hvg_input* in, uint64_t num_cells,
                                float* mean, float* var, uint32_t* nonzero_count,
                                void* stream);
/* Per-gene sums and squared sums of counts, each count above clip_val[gene]
 * replaced by clip_val[gene]. Replaces clipped_sum_csr (hvg.pyx:255-403:
 * rows [0, num_cells), or every listed cell) and clipped_sum_csc
 * (hvg.pyx:406-530: every gene of indptr, num_cells unused). Outputs have
 * num_genes (CSR) or num_major (CSC) entries. */
BGPU_API int bgpu_clipped_sum(const bgpu_hvg_input* in, uint64_t num_cells,
                              const float* clip_val, float* batch_counts_sum,
                              float* squared_batch_counts_sum, void* stream);

/* ---- k-nearest neighbours on the principal components ----------------- */
/* knn_self (brisc/knn.pyx:13-515, called by SingleCell.neighbors at
 * brisc/single_cell.py:12613-12626): for every cell of X (num_cells x
 * num_dimensions, row-major float32, rows grouped by k-means cluster), the
 * num_neighbors nearest other cells among the cells of its
 * num_clusters_searched nearest clusters. Same arguments as the reference,
 * minus its chunk sizes, is_mac and num_threads (CPU scheduling knobs with no
 * effect on the result): sorted_order maps a row of X to the original cell
 * id; centroids (num_clusters x num_dimensions) and num_cells_per_cluster
 * (uint32, summing to num_cells) describe the clusters in row order;
 * cell_norms holds each row's squared norm. Outputs, row-major per row of X:
 * neighbors (num_cells x num_neighbors, original ids) and distances (squared
 * Euclidean |x|^2 + |c|^2 - 2 x.c) in ascending distance, and
 * nearest_clusters / centroid_distances (num_cells x num_clusters_searched)
 * in ascending partial distance |c|^2 - 2 x.c. All pointers are device
 * pointers. Limits: num_dimensions <= 128, num_neighbors <= 128,
 * num_clusters_searched <= 256, num_clusters <= 32768. Synchronous. */
BGPU_API int bgpu_knn_self(const float* X, const uint32_t* sorted_order,
                           const float* centroids,
                           const uint32_t* num_cells_per_cluster, uint32_t* neighbors,
                           float* distances, const float* cell_norms,
                           float* centroid_distances, uint32_t* nearest_clusters,
                           uint64_t num_cells, uint32_t num_dimensions,
                           uint32_t num_clusters, uint32_t num_neighbors,
                           uint32_t num_clusters_searched, void* stream);

/* kmeans (brisc/kmeans.pyx:889-1433, called by SingleCell.neighbors at
 * brisc/single_cell.py:12532-12545), random initialisation only (the
 * reference's default; kmeans_barbar must be 0, else BGPU_ERR_UNSUPPORTED).
 * X: num_cells x num_dimensions row-major float32. Outputs: cluster_labels
 * (uint32 per cell), centroids and centroids_new (num_clusters x
 * num_dimensions; they swap every iteration, so the final centroids are in
 * centroids_new when *iterations is odd, as in the reference),
 * num_cells_per_cluster, min_distances (the partial distance |c|^2 - 2 x.c
 * to the assigned centroid) and, when not NULL, cell_norms (|x|^2). The
 * M step sums chunk_size cells at a time, in the reference's order.
 * num_init_iterations and oversampling_factor belong to k-means|| and are
 * not taken. Device pointers; synchronous. Limits: 128 dimensions, 32768
 * clusters. */
BGPU_API int bgpu_kmeans(const float* X, uint32_t* cluster_labels, float* centroids,
                         float* centroids_new, uint32_t* num_cells_per_cluster,
                         float* min_distances, float* cell_norms, int kmeans_barbar,
                         uint32_t num_kmeans_iterations, float tolerance,
                         uint32_t chunk_size, uint64_t seed, uint64_t num_cells,
                         uint32_t num_dimensions, uint32_t num_clusters,
                         uint32_t* iterations, void* stream);

/* normalize_rows (brisc/harmonize.pyx:244-266, called by
 * SingleCell.harmonize at brisc/single_cell.py:13819): out = arr with each
 * row scaled to unit Euclidean norm. num_rows x num_columns row-major
 * float32, device pointers; arr == out is allowed. Asynchronous on stream. */
BGPU_API int bgpu_normalize_rows(const float* arr, float* out, uint64_t num_rows,
                                 uint32_t num_columns, void* stream);

/* harmony (brisc/harmonize.pyx:269-871, called by SingleCell.harmonize at
 * brisc/single_cell.py:13864-13875). Same arguments as the reference, minus
 * verbose and num_threads: PCs (num_cells x num_PCs), Z (the row-normalised
 * PCs on entry, the Harmony embedding on return), Y (num_clusters x num_PCs:
 * the k-means centroids of Z on entry, the last normalised centroids on
 * return), R (num_cells x num_clusters soft assignments, output),
 * batch_labels (uint32 per cell, < num_batches). The cells are visited in the
 * reference's PCG32 Fisher-Yates order from seed, in blocks of
 * ceil(num_cells * block_proportion) cells and chunks of chunk_size cells
 * within a block. *iterations receives the number of correction rounds run.
 * tau > 0 repeats the reference's arithmetic (its theta discount negates an
 * unsigned count, harmonize.pyx:416), whose output is then NaN.
 * Device pointers; synchronous. Limits: num_PCs <= 128, num_clusters <= 256,
 * num_batches <= 64, chunk_size <= 1024, num_cells < 2^32, and num_PCs x
 * num_clusters plus three num_batches x num_clusters floats within one CTA's
 * shared memory (BGPU_ERR_UNSUPPORTED otherwise). */
BGPU_API int bgpu_harmony(const float* PCs, float* Z, float* Y, float* R,
                          const uint32_t* batch_labels, uint32_t num_batches,
                          uint32_t max_iterations, uint32_t max_clustering_iterations,
                          float block_proportion, float tolerance, int early_stopping,
                          float clustering_tolerance, float theta, float tau, float alpha,
                          float sigma, uint32_t chunk_size, uint64_t seed,
                          uint64_t num_cells, uint32_t num_PCs, uint32_t num_clusters,
                          uint32_t* iterations, void* stream);

/* ---- .h5ad count matrix straight to the device -------------------------- */
/* The reference reads an AnnData file's sparse X by asking h5py for each
 * dataset's byte offset (brisc/single_cell.py:1848-1883) and preading the
 * contiguous bytes into host arrays with OpenMP threads (brisc/hdf5.pyx:163
 * read_all_datasets). Here the HDF5 metadata is parsed by the library itself
 * (no HDF5 library is needed) and the bytes go from the file through pinned
 * staging buffers into device memory. */
enum {  /* element types of index arrays in a file */
  BGPU_H5_I32 = 0, BGPU_H5_I64 = 1, BGPU_H5_U32 = 2, BGPU_H5_U64 = 3
};
typedef struct bgpu_h5_dataset {
  uint64_t file_offset;   /* byte offset of the contiguous storage in the file  */
  uint64_t num_bytes;
  uint64_t num_elements;
  uint32_t element_size;
  int type;               /* data: BGPU_VALUE_*; indices and indptr: BGPU_H5_* */
} bgpu_h5_dataset;
typedef struct bgpu_h5ad_matrix {
  char X_key[64];         /* the group read: X_key, or the reference's choice   */
  int is_csr;             /* encoding-type csr_matrix (1) or csc_matrix (0)     */
  uint64_t num_rows, num_columns, nnz;  /* the shape attribute; stored entries */
  bgpu_h5_dataset data, indices, indptr;
} bgpu_h5ad_matrix;

/* Parses the file's metadata and describes its sparse X: the group X_key, or
 * (X_key NULL or "") 'layers/UMIs' when present, else 'raw/X', else 'X', as
 * SingleCell's reader chooses (brisc/single_cell.py:497-522, 610-657), with
 * its checks and messages (unsupported encoding-type, both layers['UMIs'] and
 * raw.X, a corrupted indptr). Only contiguous, unfiltered datasets can be
 * streamed (BGPU_ERR_UNSUPPORTED otherwise; the reference falls back to a
 * slower reader there). Host only. */
BGPU_API int bgpu_h5ad_inspect(const char* path, const char* X_key, bgpu_h5ad_matrix* out);
enum {
  BGPU_H5_READ_AUTO = 0,    /* mapped where the driver allows it, else staged   */
  BGPU_H5_READ_STAGED = 1,  /* host threads pread into pinned buffers and copy  */
  BGPU_H5_READ_MAPPED = 2   /* the file range mapped read-only and registered
                               (cudaHostRegisterReadOnly): the copy engines read
                               the page cache directly; UNSUPPORTED if refused  */
};
/* Reads the three datasets `m` describes into device arrays (data:
 * m->data.num_bytes bytes, and so on). Staged: num_threads host threads (0 =
 * all hardware threads) each pread 4 MB pieces into two pinned buffers of its
 * own and copy them to the device while reading the next. Waits for `stream`
 * first; synchronous. */
BGPU_API int bgpu_h5ad_read(const char* path, const bgpu_h5ad_matrix* m, void* data,
                            void* indices, void* indptr, uint32_t method,
                            uint32_t num_threads, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BRISCGPU_H */
