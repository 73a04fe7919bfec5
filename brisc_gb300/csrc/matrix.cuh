// Device layout of one cells x genes matrix (internal).
//
// HBM layout (n cells, g genes, nnz stored entries):
//   rowptr      int64[n + 1]              CSR row offsets (shared by both copies:
//                                          the elements of row panel p occupy
//                                          [rowptr[p*P], rowptr[(p+1)*P]) in the
//                                          CSR copy AND in the transposed copy)
//   kCounts mode (fused normalisation, 4 bytes per stored entry):
//     csr_packed  uint32[nnz4]            (gene << 16) | count; bit 31 flags the
//                                          first entry of a row when g <= 32768
//     csc_packed  uint32[nnz4]            (local_row << 16) | count, grouped by
//                                          row panel, then gene, rows ascending;
//                                          bit 31 flags the first entry of each
//                                          (panel, gene) segment
//     rtab_c      float32[panels*16*P]    per panel, [count][row] table of
//                                          log1pf(count * isf) (count 0 -> 0)
//     csc16       uint16[nnz16]           compact panel copy (g <= 2048, P =
//                                          1024): head << 15 | row << 5 | code,
//                                          code = count (0-15) or 16 (>= 16)
//     isf, post   float32[n]              per-cell factors (post may be null)
//   kFloat mode (pre-normalised values, 6 bytes per stored entry):
//     csr_val float32[nnz4], csr_col uint16[nnz4]
//     csc_val float32[nnz4], csc_row uint16[nnz4] (local row within the panel)
//   colptr      int32[num_panels * (g + 1)] per-panel gene offsets relative to
//                                          the panel's first element
// nnz4 = nnz rounded up to a multiple of 4 (+4): every 128-bit load of four
// entries starting at a multiple of 4 stays inside the allocation.
#pragma once

#include <vector>

#include "common.cuh"
#include "multi.cuh"

namespace bgpu {

enum MatrixMode { kCounts = 0, kFloat = 1 };

// Sliced-ELL views (sell.cu): scalar shape fields live in the Matrix, the
// pointers are filled in per launch.
struct XvView {  // X.v: 32-row groups, rows ordered by length
  const uint2* data;         // units of four 16-bit entries, lane-interleaved
  const uint32_t* grp;       // per group: first unit
  const uint16_t* units;     // per group: units per lane
  const int32_t* perm;       // position -> cell row (-1: padding)
  const float* isf;          // per position
  const float* post;         // per position (PFlog1pPF) or null
  const uint16_t* esc_n;     // per position: counts >= 16 of the row
  const uint32_t* esc_base;  // per position: first escape record
  const uint32_t* esc;       // escape records gene << 16 | count
  uint32_t groups;
  uint32_t g;
  uint64_t n;
  uint64_t total_units;
};
struct XtView {  // X^T.u: (panel, gene) segments in 32-segment groups
  const uint2* data;         // units of four 16-bit shared-memory offsets
  const uint32_t* grp;       // per group: first unit
  const uint16_t* units;     // per group: units per lane
  const uint16_t* gene;      // per group and lane: gene (0xffff: none)
  const uint32_t* pgrp;      // per panel: first group (panels + 1)
  const uint32_t* esc_base;  // per panel: first escape record (panels + 1)
  const uint32_t* esc;       // escape records local_row << 16 | count
  const float* isf;
  const float* post;
  uint64_t n;
  uint64_t total_units;
  uint32_t g;
  uint32_t P;                // rows per panel (<= 512)
  uint32_t ppc;              // consecutive panels per CTA
  uint32_t panels;
  uint32_t ctas;             // CTAs of a launch = rows of the partials
  uint32_t esc_max;          // most escapes in one panel
  uint32_t groups;
};

// Per-cell table of normalised values for small counts:
// tab[c] = log1pf(c * isf) for 1 <= c < 16 and tab[0] = 0.
constexpr int kCountTab = 16;

struct Matrix {
  uint64_t n = 0;
  uint32_t g = 0;
  uint64_t nnz = 0;
  uint64_t nnz_alloc = 0;
  int mode = kCounts;
  int norm_method = BGPU_NORM_NONE;

  int64_t* rowptr = nullptr;
  uint32_t* csr_packed = nullptr;
  float* csr_val = nullptr;
  uint16_t* csr_col = nullptr;

  uint32_t pshift = 13;  // log2 of panel rows
  uint32_t P = 8192;
  uint32_t num_panels = 0;
  int32_t* colptr = nullptr;
  uint32_t* csc_packed = nullptr;
  float* csc_val = nullptr;
  uint16_t* csc_row = nullptr;

  float* isf = nullptr;
  float* post = nullptr;
  float* rtab_r = nullptr;  // [cell][kCountTab] (X.v)
  float* rtab_c = nullptr;  // [panel][kCountTab][P] (X^T.u)
  uint16_t* csc16 = nullptr;  // compact panel entries (stream16.cu)
  int32_t* row_order = nullptr;  // X.v row schedule, longest rows first

  float* sd = nullptr;  // cached clipped gene std (computed on first use)
  int device = 0;
  cudaStream_t stream = nullptr;  // creation stream: the arrays are released on it
  uint64_t bytes = 0;

  // Autotuned SpMV shapes (chosen at creation from the nnz-per-row histogram).
  int spmv_group = 16;     // lanes per row (register-vector kernel)
  int spmv_blocks = 0;     // CTAs (register-vector kernel)
  int rmat_colgroup = 256; // genes per CTA (register-vector transposed product)

  // Table-driven products (stream.cu) for the counts layout.
  bool stream_ok = false;  // count tables built; the table-driven kernels apply
  bool csr_heads = false;  // CSR words carry row-head flags (segmented X.v)
  bool compact = false;    // 16-bit panel copy built: X^T.u uses it
  bool spmv_seg = false;   // X.v by the segmented stream (short rows) rather
                           // than 8 lanes per row
  int impl = 0;            // 0 = table-driven kernels, 1 = register-vector kernels
  uint32_t kernels = 0;    // bgpu_matrix_desc.kernels (BGPU_KERNELS_*)

  // Sliced-ELL layout (sell.cu), counts mode with g <= 4096: when `sell` is
  // set both products run on it and the panel layout above is not built.
  bool sell = false;
  uint32_t sell_P = 0;  // requested X^T.u panel rows (bgpu_matrix_desc.sell_panel_rows)
  XvView xv{};
  XtView xt{};
  uint2* xv_data = nullptr;
  uint32_t* xv_grp = nullptr;
  uint16_t* xv_units = nullptr;
  int32_t* xv_perm = nullptr;
  float* xv_isf = nullptr;
  float* xv_post = nullptr;
  uint16_t* xv_esc_n = nullptr;
  uint32_t* xv_esc_base = nullptr;
  uint32_t* xv_esc = nullptr;
  uint2* xt_data = nullptr;
  uint32_t* xt_grp = nullptr;
  uint16_t* xt_units = nullptr;
  uint16_t* xt_gene = nullptr;
  uint32_t* xt_pgrp = nullptr;
  uint32_t* xt_esc_base = nullptr;
  uint32_t* xt_esc = nullptr;
};

// Per-launch views passed by value to kernels.
struct CsrView {
  const int64_t* rowptr;
  const uint32_t* packed;
  const float* val;
  const uint16_t* col;
  const float* isf;
  const float* post;
  uint64_t n;
  uint32_t g;
  const float* rtab;  // [cell][kCountTab], counts mode
};
struct CscView {
  const int64_t* rowptr;
  const int32_t* colptr;
  const uint32_t* packed;
  const float* val;
  const uint16_t* row;
  const float* isf;
  const float* post;
  uint64_t n;
  uint32_t g;
  uint32_t pshift;
  uint32_t num_panels;
  const float* rtab;  // [panel][kCountTab][P], counts mode
};

inline CsrView csr_view(const Matrix& m) {
  return CsrView{m.rowptr, m.csr_packed, m.csr_val, m.csr_col, m.isf,
                 m.post,   m.n,          m.g,       m.rtab_r};
}
inline CscView csc_view(const Matrix& m) {
  return CscView{m.rowptr, m.colptr, m.csc_packed, m.csc_val, m.csc_row,
                 m.isf,    m.post,   m.n,          m.g,       m.pshift,
                 m.num_panels, m.rtab_c};
}

// layout.cu
int matrix_build(Matrix* m, const bgpu_matrix_desc* d, cudaStream_t s);
// The layout of X[rows, :] (rows in the memory space of d's arrays).
int matrix_build_rows(Matrix* m, const bgpu_matrix_desc* d, const int64_t* rows,
                      uint64_t nr, cudaStream_t s);
void matrix_free(Matrix* m);

// spmv.cu: raw products on the layout (device pointers)
int launch_matvec(const Matrix& m, const float* v, const float* sd, float* y,
                  cudaStream_t s);
// X^T u: per-panel partials (gene-major: partT[gene * num_panels + panel]),
// reduced in panel order by launch_reduce_panels_t. `u_scale_dev` (device
// scalar, may be null) multiplies u on load; when `u_out` is non-null the
// scaled u is also written there.
int launch_rmatvec_partials(const Matrix& m, const float* u,
                            const float* u_scale_dev, float* u_out,
                            float* partials, cudaStream_t s);
int launch_gene_stddev(const Matrix& m, double* partials, float* sd,
                       cudaStream_t s);

// stream.cu: table-driven products for the counts layout (partials of X^T u
// are gene-major: partT[gene * num_panels + panel]). build_stream_tiles builds
// the per-cell count tables when the layout allows the table-driven kernels.
bool stream_supported(const Matrix& m);
int build_stream_tiles(Matrix* m, const std::vector<int64_t>& panel_rowptr,
                       cudaStream_t s, uint64_t* bytes_acc);
int launch_matvec_stream(const Matrix& m, const float* v, const float* sd,
                         float* y, int* err, cudaStream_t s);
int launch_rmatvec_stream(const Matrix& m, const float* u, const float* u_scale,
                          float* u_out, float* partT, int* err, cudaStream_t s);
int launch_reduce_panels_t(const Matrix& m, const float* partT, const float* sd,
                           float* z, cudaStream_t s);

// stream16.cu: X^T.u on the compact 16-bit panel entries.
bool compact16_supported(const Matrix& m);
int build_compact16(Matrix* m, cudaStream_t s, uint64_t* bytes_acc);
int launch_rmatvec16(const Matrix& m, const float* u, const float* u_scale,
                     float* u_out, float* partT, int* err, cudaStream_t s);

// sell.cu: sliced-ELL layout and products. build_sell sets *built when the
// layout applies (counts mode, g <= 4096, within its per-panel limits).
bool sell_supported(const Matrix& m);
int build_sell(Matrix* m, cudaStream_t s, bool* built);
int launch_xv_sell(const Matrix& m, const float* v, const float* sd, float* y,
                   cudaStream_t s);
// X^T.u partials, gene-major: partT[gene * xt.ctas + cta] (reduced in CTA
// order by launch_reduce_panels_t, with m.num_panels == xt.ctas).
int launch_xt_sell(const Matrix& m, const float* u, const float* u_scale, float* u_out,
                   float* partT, cudaStream_t s);
// Per-gene FP64 moments: partials[cta * g + gene] = {sum, sum of squares}.
int launch_xt_moments(const Matrix& m, double* partials, cudaStream_t s);
XvView xv_view(const Matrix& m);
XtView xt_view(const Matrix& m);

// Fused multi-solve forms (multi.cuh) of the two products and of the
// partials' reduction: a task runs on the CTAs its single launch would use,
// xv_sell_ctas(m), xt_sell_ctas(m) and reduce_panels_ctas(m).
struct XvTask {
  XvView X;
  const float* v;
  const float* sd;
  float* y;
};
struct XtTask {
  XtView X;
  const float* u;
  const float* u_scale;
  float* u_out;
  float* partT;
};
struct ReducePanelsTask {
  const float* partT;
  const float* sd;
  float* z;
  uint32_t num_panels, g;
};
uint32_t xv_sell_ctas(const Matrix& m);
uint32_t xt_sell_ctas(const Matrix& m);
uint32_t reduce_panels_ctas(const Matrix& m);
int launch_xv_sell_multi(const TaskList<XvTask>& L, cudaStream_t s);
int launch_xt_sell_multi(const TaskList<XtTask>& L, cudaStream_t s);
int launch_reduce_panels_multi(const TaskList<ReducePanelsTask>& L, cudaStream_t s);

// Bytes of the algorithmic traffic of one X.v / X^T.u launch (used for the
// roofline figure). Counts what the chosen layout must stream.
double matvec_bytes(const Matrix& m);
double rmatvec_bytes(const Matrix& m);

}  // namespace bgpu
