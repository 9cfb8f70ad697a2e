/*
 * lapy_gb300 — C ABI of the GB300 (sm_103a) linear-FEM Laplace–Beltrami path.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t
 * (passed as void*), returns an int status (LAPY_OK == 0, negative on error)
 * and never throws.  No function allocates device memory: buffers, including
 * scratch ("workspace"), are allocated by the caller, whose size the matching
 * *_workspace_bytes() query returns.  Indices are int32, matrix values f64
 * unless the name says f32.
 *
 * The reference (Deep-MI/LaPy) is pure Python over SciPy; it has no FFI.
 * Each entry point below names the reference function whose work it performs;
 * the Python package lapy_gb300 binds them with ctypes and mirrors the
 * reference's Python API (Solver, heat.diffusion, diffgeo, shapedna).
 */
#ifndef LAPY_GB300_H
#define LAPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define LAPY_OK 0
#define LAPY_ERR_INVALID (-1)   /* bad argument (size, pointer, alignment)   */
#define LAPY_ERR_CUDA (-2)      /* CUDA runtime error                        */
#define LAPY_ERR_NOCONV (-3)    /* iteration cap reached before tolerance    */
#define LAPY_ERR_BREAKDOWN (-4) /* Krylov breakdown (p'Ap <= 0, rank loss)   */
#define LAPY_ERR_NAN (-5)       /* NaN/Inf met in the iteration              */
#define LAPY_ERR_TIMEOUT (-6)   /* a bounded device-side wait gave up        */
#define LAPY_ERR_WORKSPACE (-7) /* workspace smaller than the query result   */
#define LAPY_ERR_PATTERN (-8)   /* matrix pattern not contained in A's       */

/* Library version (major*10000 + minor*100 + patch). */
int lapy_version(void);
/* Human-readable text for a status code. */
const char* lapy_status_string(int status);
/* Detail text of the last error recorded by this thread ("" if none). */
const char* lapy_last_error(void);
/* Kernel launches issued by this library since it was loaded. */
long long lapy_launch_count(void);
/* Diagnostics (host only): consistency of the persistent PCG's warp plan for
 * the segments seg_row[0..nseg] (virtual warps / CTAs, reduction slots, row
 * coverage).  LAPY_OK, or LAPY_ERR_INVALID with lapy_last_error() saying what
 * failed. */
int lapy_plan_check(const int32_t* seg_row, int nseg);
/* Host only: the aggregation and row order the batched two-level eigensolver
 * uses (no counterpart in the reference, which factorises exactly): for a
 * symmetric CSR pattern on the host (indptr, indices; n rows in segments
 * seg_row[0..nseg]), connected aggregates of about agg_target rows (>= 64)
 * per segment, numbered breadth-first over the aggregate graph; perm[i] is
 * the original row placed at position i (rows of an aggregate contiguous,
 * segments keep their ranges) and labels[i] its aggregate's number within
 * its segment (-1: the segment gets no coarse space).  Deterministic. */
int lapy_aggregate_order(int64_t n, const int32_t* indptr, const int32_t* indices, const int32_t* seg_row,
                         int nseg, int agg_target, int32_t* perm, int32_t* labels);
/* PCG profile: when enabled, every persistent PCG launch is timed with CUDA
 * events and its work counted.  lapy_profile_read fills up to n of
 * {pcg_ms, pcg_launches, pcg_iterations, rows_processed, nnz_processed,
 *  algorithmic_bytes, lanczos_segment_steps, second_cgs_passes,
 *  then 7 per-phase milliseconds of the PCG launches (device clock between
 *  grid barriers): initialisation, SpMM, update, coarse restriction, coarse
 *  solve, direction update, final publication}. */
#define LAPY_PCG_PHASES 7
void lapy_profile_enable(int on);
void lapy_profile_reset(void);
int lapy_profile_read(double* out, int n);

/* ---- FEM assembly: symbolic CSR build ----------------------------------
 * Replaces the COO -> CSC duplicate summation of
 *   lapy/solver.py:171-178 (_fem_tria), :286-293 (_fem_tria_aniso),
 *   :472-501 (_fem_tetra)
 * i.e. scipy.sparse.csc_matrix((data, (i, j))).  The element connectivity
 * `elems` (m x npe, npe = 3 or 4, row-major int32) yields the local (i, j)
 * pairs in the reference's order; the CSR pattern of the n x n result is the
 * set of distinct pairs, rows ascending, columns ascending inside a row
 * (A is symmetric, so these arrays equal the reference's CSC arrays).
 *
 * Two calls, because nnz is only known after the first:
 *   lapy_csr_symbolic_count  -> indptr (n+1, device) and *nnz_out (host)
 *   lapy_csr_symbolic_fill   -> indices (nnz), seg_ptr (nnz+1), seg_src (m*L)
 * seg_src lists the local-entry positions (e*L + l, L = npe*npe) sorted by
 * (row, col, position); seg_ptr[k]..seg_ptr[k+1] is the run summed into
 * nonzero k.  The numeric kernels below use (seg_ptr, seg_src).
 */
size_t lapy_csr_symbolic_workspace_bytes(int64_t n, int64_t m, int npe);
int lapy_csr_symbolic_count(const int32_t* elems, int64_t m, int npe, int64_t n,
                            int32_t* indptr, int64_t* nnz_out, void* workspace,
                            size_t ws_bytes, void* stream);
int lapy_csr_symbolic_fill(const int32_t* elems, int64_t m, int npe, int64_t n,
                           const int32_t* indptr, int64_t nnz, int32_t* indices,
                           int32_t* seg_ptr, int32_t* seg_src, void* workspace,
                           size_t ws_bytes, void* stream);

/* ---- FEM assembly: numeric ---------------------------------------------
 * Element math in the coordinate type (coords_f32 != 0: float32 coordinates,
 * as the reference's mesh readers produce; else float64), then summed per
 * nonzero in (element, local) order into out_f32 ? float32 : float64 values.
 *
 * lapy_fem_tria_numeric    <- lapy/solver.py:105-194  (_fem_tria)
 * lapy_fem_tria_aniso_numeric <- lapy/solver.py:196-308 (_fem_tria_aniso);
 *      u1, u2: m x 3 float64 curvature frame, aniso_mat: m x 2 float64
 *      (tria_mesh.py:1221-1279 and solver.py:88-90 produce them on the host)
 * lapy_fem_tet_numeric     <- lapy/solver.py:379-533  (_fem_tetra)
 *
 * a_vals, m_vals: nnz values of A and M on the pattern from the symbolic
 * step.  lump != 0: m_vals instead receives n diagonal values (the lumped
 * mass, solver.py:188-193 / :527-532).  `work` must hold
 * lapy_fem_numeric_workspace_bytes(m, npe) bytes.
 */
size_t lapy_fem_numeric_workspace_bytes(int64_t m, int npe);
int lapy_fem_tria_numeric(const void* v, int coords_f32, const int32_t* t, int64_t m,
                          int64_t n, const int32_t* indptr, const int32_t* indices,
                          const int32_t* seg_ptr, const int32_t* seg_src, int64_t nnz,
                          int lump, int out_f32, void* a_vals, void* m_vals, void* work,
                          size_t ws_bytes, void* stream);
int lapy_fem_tria_aniso_numeric(const void* v, int coords_f32, const int32_t* t,
                                int64_t m, const double* u1, const double* u2,
                                const double* aniso_mat, int64_t n, const int32_t* indptr,
                                const int32_t* indices, const int32_t* seg_ptr,
                                const int32_t* seg_src, int64_t nnz, int lump, int out_f32,
                                void* a_vals, void* m_vals, void* work, size_t ws_bytes,
                                void* stream);
int lapy_fem_tet_numeric(const void* v, int coords_f32, const int32_t* t, int64_t m,
                         int64_t n, const int32_t* indptr, const int32_t* indices,
                         const int32_t* seg_ptr, const int32_t* seg_src, int64_t nnz,
                         int lump, int out_f32, void* a_vals, void* m_vals, void* work,
                         size_t ws_bytes, void* stream);
/* Batched form of lapy_fem_tria_numeric (npe 3) / lapy_fem_tet_numeric
 * (npe 4) for meshes concatenated into one block-diagonal system: seg_elem
 * (device, nseg+1 int32, nondecreasing from 0 to m) gives each mesh's element
 * range, and each mesh's degenerate elements are clamped with that mesh's own
 * mean measure, as one lapy/solver.py:158-159 (:436-437) call per mesh does.
 * `work` must hold lapy_fem_batch_numeric_workspace_bytes(m, npe, nseg). */
size_t lapy_fem_batch_numeric_workspace_bytes(int64_t m, int npe, int nseg);
int lapy_fem_batch_numeric(int npe, const void* v, int coords_f32, const int32_t* t, int64_t m,
                           int nseg, const int32_t* seg_elem, int64_t n, const int32_t* indptr,
                           const int32_t* indices, const int32_t* seg_ptr, const int32_t* seg_src,
                           int64_t nnz, int lump, int out_f32, void* a_vals, void* m_vals, void* work,
                           size_t ws_bytes, void* stream);

/* Position of the diagonal entry of every row (-1 if absent). */
int lapy_csr_diag_index(int64_t n, const int32_t* indptr, const int32_t* indices,
                        int32_t* diag_pos, void* stream);

/* Map the pattern (b_indptr, b_indices) into A's pattern: pos[k] = index in A
 * of B's nonzero k.  Returns LAPY_ERR_PATTERN if some entry is not in A.
 * `work`: >= 256 bytes of device scratch.  Used when a caller replaces
 * Solver.mass (lapy/diffgeo.py:149 sets it to the identity). */
int lapy_csr_pattern_map(int64_t n, const int32_t* a_indptr, const int32_t* a_indices,
                         const int32_t* b_indptr, const int32_t* b_indices,
                         int64_t b_nnz, int32_t* pos, void* work, void* stream);

/* Batch construction (the reference handles one mesh per call; a batch of
 * meshes is concatenated into one block-diagonal system).
 * lapy_h2d_concat: `count` host buffers (src[i], bytes[i]) copied back to
 * back into the device buffer dst, in order, on `stream`.  With a pinned
 * host buffer of at least the total size (`pinned`, `pinned_bytes`; may be
 * null), the buffers are first gathered into it on a few host threads and
 * copied with one transfer; it must stay untouched until the copy on
 * `stream` has completed.  Without one, each buffer is its own copy.
 * lapy_seg_offset_elements: t_out (device, m x npe int32) = t_in (device, the
 * meshes' own vertex indices concatenated; int64 if idx64 else int32) +
 * seg_row[s] for the elements [seg_elem[s], seg_elem[s+1]) of mesh s
 * (seg_elem, seg_row: device, nseg+1 each).  seg_max (device, nseg+1 int32)
 * receives each mesh's largest index, and seg_max[nseg] != 0 if an index was
 * outside its mesh's rows.
 * lapy_seg_unit_vector: out (device, n) = the indicator of vertex vid[s] of
 * every mesh s (the right-hand sides of heat.diffusion, lapy/heat.py:215-221,
 * for one seed vertex per mesh). */
int lapy_h2d_concat(int count, const void* const* src, const size_t* bytes, void* dst, void* pinned,
                    size_t pinned_bytes, void* stream);
int lapy_seg_offset_elements(int64_t m, int npe, int nseg, const int32_t* seg_elem,
                             const int32_t* seg_row, const void* t_in, int idx64, int32_t* t_out,
                             int32_t* seg_max, void* stream);
int lapy_seg_unit_vector(int64_t n, int nseg, const int32_t* seg_row, const int32_t* vid, double* out,
                         void* stream);

/* Mean edge length over the strict upper triangle of the pattern
 * (lapy/tria_mesh.py:735-748, lapy/tet_mesh.py:182-195: the mean of
 * ||v_i - v_j|| over the distinct edges).  Result written to *out (host). */
int lapy_avg_edge_length(const void* v, int coords_f32, int64_t n, const int32_t* indptr,
                         const int32_t* indices, double* out, void* work,
                         size_t ws_bytes, void* stream);
size_t lapy_avg_edge_length_workspace_bytes(int64_t n);
/* Batched form: out[s] (device, nseg doubles) = mean edge length of segment s
 * of a block-diagonal batch (seg_row: device, nseg+1 row offsets); t_out
 * (device, may be NULL) receives each mesh's heat time step
 * t = m * avg_edge_length**2 (lapy/heat.py:206). */
int lapy_seg_avg_edge_length(const void* v, int coords_f32, int nseg, const int32_t* seg_row,
                             const int32_t* indptr, const int32_t* indices, double m, double* out,
                             double* t_out, void* stream);

/* ---- sparse matrix-vector products -------------------------------------
 * Y = alpha * Mat * X + beta * Y for X, Y row-major n x ncol.  Used wherever
 * the reference multiplies by A or M (solver.py:844-846, heat.py:208 ...).
 * group: lanes per row (4, 8, 16 or 32; 0 = autotuned choice). */
int lapy_csr_spmm_f64(int64_t n, const int32_t* indptr, const int32_t* indices,
                      const double* vals, int ncol, const double* x, double* y,
                      double alpha, double beta, int group, void* stream);
int lapy_csr_spmm_f32(int64_t n, const int32_t* indptr, const int32_t* indices,
                      const float* vals, int ncol, const float* x, float* y,
                      float alpha, float beta, int group, void* stream);
/* Standalone FP32 SELL product Y = Mat X (X, Y row-major n x ncol, ncol in
 * {1, 2, 4, 8}): the sliced-ELL copy (32-row slices) and the pipelined
 * product of the inner PCG, outside the persistent kernel.  It stands for
 * the sparse products inside the reference's ARPACK/SuperLU operator
 * (solver.py:707-713) when measured alone.  _build casts vals to FP32 and
 * builds the slices into `work` (size from _workspace_bytes); the handle
 * points into `work`, which must outlive it. */
typedef struct {
  int32_t nunit;             /* 32-row units */
  const int32_t* unit_row;   /* device, nunit + 1 */
  const int32_t* slice_ptr;  /* device, nunit + 1 */
  const int32_t* col;        /* device */
  const float* val;          /* device */
} lapy_sell_f32;
size_t lapy_sell_f32_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row);
int lapy_sell_f32_build(int64_t n, const int32_t* indptr, const int32_t* indices, const double* vals,
                        int64_t nnz, int nseg, const int32_t* seg_row, lapy_sell_f32* out, void* work,
                        size_t ws_bytes, void* stream);
int lapy_sell_f32_spmm(const lapy_sell_f32* m, int ncol, const float* x, float* y, void* stream);
/* Diagonal-matrix variant Y = alpha * diag(d) X + beta * Y. */
int lapy_diag_mm_f64(int64_t n, const double* d, int ncol, const double* x, double* y,
                     double alpha, double beta, void* stream);

/* ---- heat kernel products (lapy/heat.py:19-111) ------------------------
 * H (nrows x nt, row-major) = W S, W row r = evecs[rows[r], 0:nev] (rows NULL:
 * row r), squared element-wise when `squared` (the diagonal K(t, x, x));
 * evecs row-major with leading dimension ld >= nev; S (nev x nt, row-major)
 * the exp(-lambda t) factors.  Replaces the final np.matmul of heat.diagonal
 * (heat.py:59) and heat.kernel (heat.py:108). */
int lapy_heat_product_f64(int64_t nrows, const int64_t* rows, const double* evecs, int64_t ld, int nev,
                          int squared, const double* S, int nt, double* H, void* stream);

/* ---- element-wise helpers ----------------------------------------------
 * out = a*x + b*y (y may be NULL).  Forms hmat = M + t*A (lapy/heat.py:208)
 * and A - sigma*M (lapy/solver.py:707) on a shared pattern. */
int lapy_vec_axpby(int64_t n, double a, const double* x, double b, const double* y,
                   double* out, void* stream);
/* Batched form of hmat = M + t*A (lapy/heat.py:208) with one coefficient pair
 * per segment: out = alpha[s]*x + beta[s]*y on the rows of segment s
 * (seg_row, alpha, beta: device arrays).  y_is_diag: y is an n-vector added
 * at diag_pos (a lumped mass). */
int lapy_csr_seg_axpby(int nseg, const int32_t* seg_row, const int32_t* indptr,
                       const int32_t* diag_pos, const double* alpha, const double* x,
                       const double* beta, const double* y, int y_is_diag, double* out,
                       void* stream);
/* vals[diag_pos[i]] += b * d[i]: adds a lumped (diagonal) mass to a matrix. */
int lapy_csr_add_diag(int64_t n, const int32_t* diag_pos, double b, const double* d,
                      double* vals, void* stream);
/* Dirichlet masking (lapy/solver.py:847-865): rows and columns of masked
 * vertices become identity rows, so the masked system equals the reduced
 * system A[free][:, free] of the reference.  dmask: n bytes, 1 = Dirichlet. */
int lapy_csr_dirichlet_mask(int64_t n, const int32_t* indptr, const int32_t* indices,
                            const double* vals, const uint8_t* dmask, double* out_vals,
                            void* stream);

/* ---- linear solves -------------------------------------------------------
 * Replaces splu(K).solve(B) of lapy/solver.py:873-877 (Poisson) and
 * lapy/heat.py:223-227 (heat).  K (n x n CSR, f64) is block diagonal over
 * `nseg` segments (seg_row: host array, nseg+1 row offsets); B and X are
 * row-major n x ncol.  mixed != 0: FP32 Jacobi-PCG inside FP64 iterative
 * refinement (each round to inner_rtol); mixed == 0: FP64 Jacobi-PCG.
 * Stops when ||B - K X|| <= rtol ||B|| per (segment, column).
 * status_out / relres_out: host arrays nseg*ncol (row s*ncol + c). */
size_t lapy_pcg_solve_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row,
                                      int ncol, int mixed);
int lapy_pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices,
                   const double* k_vals, int64_t nnz, int nseg, const int32_t* seg_row,
                   int ncol, const double* b, double* x, double rtol, int maxiter, int mixed,
                   double inner_rtol, int32_t* status_out, double* relres_out,
                   int64_t* iters_out, void* ws, size_t ws_bytes, void* stream);

/* Allocation-free lapy_pcg_solve (no counterpart in the reference, whose
 * solves run on the host).  For callers that cannot allocate device memory —
 * a process whose device memory is reserved by another allocator, a code path
 * where allocating is not allowed, a plain C caller without a workspace — the
 * scratch is a static device array of LAPY_STATIC_SCRATCH_BYTES that every
 * GPU loading the library holds until exit.  Problems needing more scratch
 * (lapy_pcg_solve_workspace_bytes) are rejected with LAPY_ERR_WORKSPACE.  The
 * first call on a device looks up the array's address (cudaGetSymbolAddress);
 * the address is kept for the life of the process, so the entry point must not be used on a device after
 * a cudaDeviceReset of it.  Like lapy_pcg_solve it returns once the solve has
 * finished on `stream`.  All calls share the array and each leaves its
 * contents behind: calls that overlap on the GPU (two streams or two host
 * threads) race.  Nothing is allocated or freed. */
#define LAPY_STATIC_SCRATCH_BYTES ((size_t)32 << 20)
int lapy_pcg_solve_static(int64_t n, const int32_t* indptr, const int32_t* indices,
                          const double* k_vals, int64_t nnz, int nseg, const int32_t* seg_row,
                          int ncol, const double* b, double* x, double rtol, int maxiter,
                          int mixed, double inner_rtol, int32_t* status_out,
                          double* relres_out, int64_t* iters_out, void* stream);

/* ---- curvature frame (anisotropic Laplace-Beltrami pre-step) -------------
 * Replaces TriaMesh.curvature / curvature_tria (lapy/tria_mesh.py:1078-1279)
 * and, through them, the host work of Solver(mesh, aniso=...)
 * (lapy/solver.py:72-91).  v: n x 3 f64, t: m x 3 int32 (oriented), the
 * mesh's CSR pattern (indptr, indices: diagonal and edges, as the symbolic
 * assembly builds it), `smoothit` Laplace smoothing steps of the vertex
 * tensors.  Outputs (device, either may be NULL), planar f64 blocks:
 *   vtx_out (13 n): u_min (n x 3), u_max (n x 3), c_min, c_max, c_mean,
 *                   c_gauss (n each), normals (n x 3)
 *   tri_out (8 m):  u1 (m x 3), u2 (m x 3), c_min, c_max (m each)
 * A mesh that is not oriented returns LAPY_ERR_INVALID with the reference's
 * message; an element edge missing from the pattern LAPY_ERR_PATTERN. */
size_t lapy_tria_curvature_workspace_bytes(int64_t n, int64_t m, int64_t nnz);
int lapy_tria_curvature(const double* v, int64_t n, const int32_t* t, int64_t m, const int32_t* indptr,
                        const int32_t* indices, int64_t nnz, int smoothit, double* vtx_out, double* tri_out,
                        void* work, size_t ws_bytes, void* stream);

/* ---- incomplete Cholesky IC(0) -------------------------------------------
 * No counterpart in the reference, which factors exactly (splu of A - sigma
 * M at lapy/solver.py:707-712, of M + t A at lapy/heat.py:226): IC(0) is the
 * incomplete factorization the GPU path offers as a preconditioner for the
 * same SPD systems, beside Jacobi and the learned factor.
 *
 * lapy_ic0_factor: K (n x n CSR, sorted columns, full diagonal, f64) ~ L L'
 * with L on K's own pattern.  l_vals (nnz) receives L on the lower part
 * (columns <= row) and the mirror L[j][i] on each upper entry (i, j).  Rows
 * are factored level by level (level of row i: 1 + the largest level of its
 * lower neighbours); arithmetic in ascending column order without fused
 * multiply-add.  A pivot that is not positive is replaced by K[i][i] and
 * counted in *n_fixed (host).  n_levels (host, 2 ints): forward and backward
 * level counts.  `work` (lapy_ic0_workspace_bytes(n, nnz, ncol)) keeps the
 * level plan for later lapy_ic0_apply calls on the same matrix.
 * lapy_ic0_apply: z = (L L')^-1 r for ncol row-major columns.
 * lapy_ic0_pcg_solve: lapy_pcg_solve with the IC(0) preconditioner (factored
 * inside; FP32 iterations in FP64 refinement); *n_fixed as above. */
size_t lapy_ic0_workspace_bytes(int64_t n, int64_t nnz, int ncol);
int lapy_ic0_factor(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                    int64_t nnz, double* l_vals, int32_t* n_fixed, int32_t* n_levels, void* work,
                    size_t ws_bytes, void* stream);
int lapy_ic0_apply(int64_t n, const int32_t* indptr, const int32_t* indices, const double* l_vals,
                   int64_t nnz, int ncol, const double* r, double* z, void* work, size_t ws_bytes,
                   void* stream);
size_t lapy_ic0_pcg_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row, int ncol);
int lapy_ic0_pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                       int64_t nnz, int nseg, const int32_t* seg_row, int ncol, const double* b, double* x,
                       double rtol, int maxiter, double inner_rtol, int32_t* status_out, double* relres_out,
                       int64_t* iters_out, int32_t* n_fixed, void* ws, size_t ws_bytes, void* stream);

/* ---- generalized eigenproblem -------------------------------------------
 * Replaces Solver.eigs (lapy/solver.py:667-716): the k eigenpairs of
 * A x = lambda M x nearest sigma, by block shift-invert Lanczos (block width
 * `block` in {1,2,4,8,16}) on (A - sigma M)^-1 M in the M inner product, for
 * every segment of a block-diagonal batch at once.  M is given on A's pattern
 * (m_is_diag == 0, nnz values) or as its diagonal (m_is_diag != 0, n values).
 * evals: device nseg*k (ascending per segment); evecs: device row-major n x k,
 * M-orthonormal per segment.  status_out / nbasis_out: host nseg.
 * tol: Ritz residual tolerance; inner_rtol: inner-solve residual target.
 * precond: preconditioner of the inner PCG, LAPY_PRECOND_JACOBI or
 * LAPY_PRECOND_TWO_LEVEL (Jacobi plus a per-mesh aggregation coarse space
 * with a dense coarse inverse; the reference factorises instead, splu). */
#define LAPY_PRECOND_JACOBI 0
#define LAPY_PRECOND_TWO_LEVEL 2
size_t lapy_eigs_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row,
                                 int k, int block, int max_vectors, int precond);
int lapy_eigs_shift_invert(int64_t n, const int32_t* indptr, const int32_t* indices,
                           const double* a_vals, const double* m_vals, int m_is_diag,
                           int64_t nnz, int nseg, const int32_t* seg_row, double sigma, int k,
                           int block, int max_vectors, double tol, double inner_rtol,
                           int inner_maxiter, int precond, uint64_t seed, double* evals, double* evecs,
                           int32_t* status_out, int32_t* nbasis_out, int64_t* inner_iters_out,
                           void* ws, size_t ws_bytes, void* stream);
/* lapy_eigs_shift_invert with the solver's tunable knobs (the reference has no
 * counterpart: ARPACK and SuperLU have none of these).  Zero fields keep the
 * defaults; tuning == NULL is lapy_eigs_shift_invert.  Results agree with
 * the defaults' to the eigenvalue tolerance; only the time changes.
 *   agg_target   rows per aggregate of the two-level coarse space (64..1024)
 *   round_rtol   residual reduction of each FP32 refinement round (0..1)
 *   fold_pieces  fold PCG partial sums per CTA above this many pieces
 *   fold_aggs    ... above this many coarse unknowns per segment
 *   ctas_per_sm  resident PCG CTAs per SM to launch (1..5) */
typedef struct lapy_eigs_tuning {
  int agg_target;
  double round_rtol;
  int fold_pieces;
  int fold_aggs;
  int ctas_per_sm;
} lapy_eigs_tuning;
int lapy_eigs_shift_invert_tuned(int64_t n, const int32_t* indptr, const int32_t* indices,
                                 const double* a_vals, const double* m_vals, int m_is_diag, int64_t nnz,
                                 int nseg, const int32_t* seg_row, double sigma, int k, int block,
                                 int max_vectors, double tol, double inner_rtol, int inner_maxiter,
                                 int precond, uint64_t seed, double* evals, double* evecs,
                                 int32_t* status_out, int32_t* nbasis_out, int64_t* inner_iters_out,
                                 void* ws, size_t ws_bytes, void* stream, const lapy_eigs_tuning* tuning);

/* ---- learned sparse approximate inverse (per-edge MLP) -------------------
 * No counterpart in the reference (it factorises with splu).  For an SPD
 * system K on a symmetric mesh pattern, G is lower triangular on the lower
 * pattern; a per-edge network (6 -> 64 -> 64 -> 1, tanh, BF16 weights, FP32
 * arithmetic, parameter layout W1[64][6] b1[64] W2[64][64] b2[64] W3[64] b3)
 * emits w_ij for every lower entry, and
 *   q_i = (e_i - w_i)' K (e_i - w_i), G_ii = q_i^-1/2, G_ij = -w_ij G_ii,
 * so z = G' G r is SPD for every w (w = 0 is Jacobi).  Training minimises
 * sum_i log q_i (the Kaporin functional of G K G').
 *
 * Pattern: lower entries (col <= row, diagonal last; lpos = CSR position of
 * each) and upper entries (col >= row) with umap = lower index of the
 * transposed entry; each has (nnz + n) / 2 entries. */
int lapy_spai_param_count(void);
size_t lapy_spai_pattern_workspace_bytes(int64_t n);
int lapy_spai_pattern(int64_t n, const int32_t* indptr, const int32_t* indices, int64_t nnz,
                      int32_t* lptr, int32_t* lcol, int32_t* lpos, int32_t* uptr, int32_t* ucol,
                      int32_t* umap, void* work, size_t ws_bytes, void* stream);
/* Edge features (6 floats per lower entry): -A_ij, |v_i - v_j| / h, m_i / h^2,
 * m_j / h^2, log(t / h^2), sigma, with m the lumped mass (row sums of M, or M
 * itself when m_is_diag) and per-segment t, sigma, h (device arrays, nseg).
 * mass_work: n doubles of scratch. */
int lapy_spai_features(int64_t n, int nseg, const int32_t* seg_row, const void* v, int coords_f32,
                       const int32_t* indptr, const double* a_vals, const double* m_vals,
                       int m_is_diag, const int32_t* lptr, const int32_t* lcol, const int32_t* lpos,
                       const double* t_seg, const double* sigma_seg, const double* h_seg,
                       double* mass_work, float* feat, void* stream);
/* w_out[e] = network(feat[e]) for ne entries; weights: lapy_spai_param_count() bf16. */
int lapy_spai_forward(int64_t ne, const float* feat, const void* weights_bf16, float* w_out, void* stream);
/* G on the lower pattern (FP32), log q_i per row and dL/dw per entry (either
 * output may be NULL); k_vals: K (FP64) on the CSR pattern. */
int lapy_spai_factor(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                     const int32_t* lptr, const int32_t* lcol, const int32_t* lpos, const float* w,
                     float* g_lower, double* logq, float* dldw, void* stream);
/* G' values on the upper pattern: g_upper[u] = g_lower[umap[u]] (m upper entries). */
int lapy_spai_transpose_values(int64_t m, const int32_t* umap, const float* g_lower, float* g_upper,
                               void* stream);
/* grad = scale * sum_e dldw[e] * d network(feat[e]) / d parameters (FP32,
 * straight through the BF16 rounding), reduced in a fixed order. */
size_t lapy_spai_backward_workspace_bytes(int64_t ne);
int lapy_spai_backward(int64_t ne, const float* feat, const void* weights_bf16, const float* dldw,
                       float scale, float* grad, void* work, size_t ws_bytes, void* stream);
/* One Adam step on the FP32 master parameters; refreshes the BF16 copy. */
int lapy_spai_adam(int nparam, float* theta, const float* grad, float* m, float* v, void* weights_bf16,
                   float lr, float beta1, float beta2, float eps, int step, void* stream);
int lapy_spai_weights_to_bf16(int nparam, const float* theta, void* weights_bf16, void* stream);
/* lapy_pcg_solve (mixed precision) with z = G' (G r) instead of Jacobi. */
size_t lapy_spai_pcg_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row, int ncol);
int lapy_spai_pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                        int64_t nnz, int nseg, const int32_t* seg_row, int ncol, const double* b,
                        double* x, double rtol, int maxiter, double inner_rtol, const int32_t* lptr,
                        const int32_t* lcol, const float* g_lower, const int32_t* uptr,
                        const int32_t* ucol, const float* g_upper, int32_t* status_out,
                        double* relres_out, int64_t* iters_out, void* ws, size_t ws_bytes, void* stream);

/* ---- heat-method geodesics (lapy/diffgeo.py) ----------------------------
 * Gradient per element of nf vertex functions f (row-major n x nf) into
 * out (m x nf x 3): tria_compute_gradient (diffgeo.py:222-300) and
 * tet_compute_gradient (diffgeo.py:846-922). */
int lapy_tria_gradient(const void* v, int coords_f32, const int32_t* t, int64_t m,
                       const double* f, int nf, double* out, void* stream);
int lapy_tet_gradient(const void* v, int coords_f32, const int32_t* t, int64_t m,
                      const double* f, int nf, double* out, void* stream);
/* In-place g / ||g|| of `rows` 3-vectors, zero vectors -> 0
 * (diffgeo.py:153-154, the nan_to_num normalisation). */
int lapy_normalize_rows3(int64_t rows, int reserved, double* g, void* stream);
/* Integrated divergence at vertices (diffgeo.py:303-387 and :925-1006) of
 * tfunc (m x nf x 3); the vertex sums walk the assembly map's diagonal runs
 * (diag_pos from lapy_csr_diag_index, seg_ptr/seg_src from the symbolic
 * step).  work: m * npe * nf doubles. */
int lapy_tria_divergence(const void* v, int coords_f32, const int32_t* t, int64_t m,
                         int64_t n, const int32_t* diag_pos, const int32_t* seg_ptr,
                         const int32_t* seg_src, const double* tfunc, int nf, double* out,
                         double* work, void* stream);
int lapy_tet_divergence(const void* v, int coords_f32, const int32_t* t, int64_t m,
                        int64_t n, const int32_t* diag_pos, const int32_t* seg_ptr,
                        const int32_t* seg_src, const double* tfunc, int nf, double* out,
                        double* work, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LAPY_GB300_H */
