// Persistent block/batched PCG and the FP64 iterative-refinement driver.
#pragma once
#include <vector>
#include "common.cuh"

namespace lapy {

// Work decomposition of a block-diagonal batch (one segment = one mesh).
//
// chunks  rows grouped into pieces that never cross a segment (used by the
//         segmented GEMM / norm kernels, one CTA per chunk)
// units   32-row blocks inside a segment (one row per lane of a warp)
// vwarps  "virtual warps" of the persistent PCG: each owns a contiguous,
//         row-balanced range of units
// pieces  a virtual warp's unit range cut at segment boundaries; every piece
//         owns one partial-sum slot, so a segment's dot products are the sum
//         of its (few) pieces' partials, in a fixed order
constexpr int kChunkScratch = 16;  // partial sums per chunk (columns of a segmented dot product)
struct ChunkTable {
  int nseg = 0;
  int nchunk = 0;
  int32_t* chunk_row = nullptr;  // device, nchunk + 1
  int32_t* chunk_seg = nullptr;  // device, nchunk
  int32_t* seg_chunk = nullptr;  // device, nseg + 1
  int32_t* seg_row = nullptr;    // device, nseg + 1
  double* scratch = nullptr;     // device, nchunk * kChunkScratch: per-chunk partial sums
  int nunit = 0, npiece = 0, nvw = 0;
  int32_t* unit_row = nullptr;    // device, nunit + 1
  int32_t* piece_unit = nullptr;  // device, npiece + 1
  int32_t* piece_seg = nullptr;   // device, npiece
  int32_t* vw_piece = nullptr;    // device, nvw + 1
  int32_t* seg_piece = nullptr;   // device, nseg + 1
  // Virtual CTAs: groups of 8 consecutive virtual warps (a CTA's worth).  A
  // segment's partial sums are folded into one reduction slot per virtual
  // CTA holding a piece of it: slots [seg_slot[s], seg_slot[s+1]) belong to
  // the virtual CTAs seg_vc0[s], seg_vc0[s] + 1, ...
  int nvc = 0, nslot = 0;
  int32_t* vc_piece = nullptr;    // device, nvc + 1
  int32_t* seg_slot = nullptr;    // device, nseg + 1
  int32_t* seg_vc0 = nullptr;     // device, nseg
  std::vector<int32_t> h_seg_row;
  std::vector<int32_t> h_chunk_row, h_chunk_seg, h_seg_chunk;
  std::vector<int32_t> h_unit_row, h_piece_unit, h_piece_seg, h_vw_piece, h_seg_piece;
  std::vector<int32_t> h_vc_piece, h_seg_slot, h_seg_vc0;
};

// Plan chunks (and the PCG's warp plan) for the given segments (host);
// chunks hold 32..max_rows rows.  Returns the chunk count.
int plan_chunks(const int32_t* seg_row, int nseg, int target_chunks, ChunkTable* ct, int max_rows = 1024);
// Bytes of device memory the table needs.
size_t chunk_table_bytes(const ChunkTable& ct);
// Place the table into `mem` and upload it (synchronous on `stream`).
int upload_chunk_table(ChunkTable* ct, void* mem, cudaStream_t stream);

enum PcgPrecond { kPrecJacobi = 0, kPrecFactored = 1, kPrecTwoLevel = 2, kPrecIC0 = 3 };

// Coarse rows per coarse-solve task: 8 warps x 4 rows; a warp computes
// kCoarseRowsPerPass of them at a time (block widths up to 4).
constexpr int kCoarseTaskRows = 16;
constexpr int kCoarseGroupTasks = 4;  // tasks per dynamically scheduled group (one staging)
constexpr int kWarpsPerCta = 8;
#ifndef LAPY_COARSE_RW
#define LAPY_COARSE_RW 2
#endif
constexpr int kCoarseRowsPerPass = LAPY_COARSE_RW;

// Sliced-ELL copy of a CSR matrix: one slice per 32-row unit of a chunk
// table, entries stored slot-major inside a slice (element k of the slice's
// row `lane` at slice_ptr[u] + 32 k + lane), rows padded to the slice's
// longest row with zero values (column = a row of the slice).  Lane j of a
// warp reads its row with fully coalesced loads and no per-row pointers.
template <typename V>
struct SellMatrix {
  const int32_t* slice_ptr = nullptr;  // nunit + 1 element offsets
  const int32_t* col = nullptr;
  const V* val = nullptr;
};
// Workspace reserved for a SELL copy: values and columns for up to
// pad * nnz + 64 entries per unit (full mesh matrices pad by a few percent;
// the triangular halves of a factor pad much more: their row lengths vary).
size_t sell_bytes_bound(int64_t nnz, const ChunkTable& ct, int elem_size, double pad = 1.5);
// Build the SELL copy into `mem`; *fits = false (and no copy) when the padded
// matrix exceeds the reserved space.
template <typename V>
int build_sell(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals, const ChunkTable& ct,
               void* mem, size_t bytes, SellMatrix<V>* out, bool* fits, cudaStream_t stream);

// Preconditioner description.  Jacobi: z = dinv .* r.  Factored:
// z = Gt * (G * r) with G, Gt CSR on the mesh pattern (SPD by construction).
// Two-level: z = dinv .* r + W (W'KW)^-1 W' r with W the 0/1 aggregation
// matrix of each segment (disjoint aggregates) and the inverse dense per
// segment; SPD as the sum of an SPD and a semi-definite term.
template <typename V>
struct PcgPrecondDesc {
  int kind = kPrecJacobi;
  const V* dinv = nullptr;
  const int32_t* g_ptr = nullptr;
  const int32_t* g_idx = nullptr;
  const V* g_val = nullptr;
  const int32_t* gt_ptr = nullptr;
  const int32_t* gt_idx = nullptr;
  const V* gt_val = nullptr;
  SellMatrix<V> g_sell, gt_sell;      // optional SELL copies of G and G' (val == nullptr: CSR)
  int nagg = 0;                       // aggregates over all segments
  const int32_t* agg = nullptr;       // n: aggregate of each row (-1: none)
  const int32_t* agg_ptr = nullptr;   // nagg + 1: member rows of each aggregate
  const int32_t* agg_row = nullptr;   //   (CSR, rows ascending)
  int agg_contig = 0;                 // aggregate g is the row range [agg_ptr[g], agg_ptr[g+1])
  // IC(0): z = L^-T L^-1 r with L on the system's own CSR pattern (lower
  // part L, upper part the mirror L[j][i]); dinv holds 1 / L[i][i]; rows in
  // forward / backward level order (level l: [ptr[l], ptr[l+1]))
  const V* ic_val = nullptr;
  const int32_t* ic_diag = nullptr;
  int ic_nlev_f = 0, ic_nlev_b = 0;
  const int32_t* ic_lev_f_ptr = nullptr;
  const int32_t* ic_lev_f_row = nullptr;
  const int32_t* ic_lev_b_ptr = nullptr;
  const int32_t* ic_lev_b_row = nullptr;
  const int32_t* agg_sid = nullptr;   // nagg: segment of each aggregate
  const int32_t* seg_agg = nullptr;   // nseg + 1: aggregate range of each segment
  // (W'KW)^-1 of segment s = kscale[s] v v' + R, v = kvec[seg_agg[s] ..] the
  // unit eigenvector of the smallest eigenvalue of W'KW (FP32) and R the
  // remainder, stored in BF16 (row-major, rows padded to ld = nc rounded up
  // to 8, pad entries zero): with the dominant mode of the inverse kept
  // apart, 16-bit storage of the rest leaves the preconditioner SPD
  const int64_t* kinv_off = nullptr;  // nseg: offset of the segment's nc x ld remainder
  const uint16_t* kinv = nullptr;     // BF16 remainders
  const float* kvec = nullptr;        // nagg: v, per segment
  const float* kscale = nullptr;      // nseg: c = v' (W'KW)^-1 v
  // coarse-solve tasks: coarse rows [task_g0[t], task_g1[t]) (global
  // indices, at most kCoarseTaskRows, one segment); virtual CTA v runs tasks
  // [vc_task[v], vc_task[v+1]), contiguous and of about equal cost
  int ntask = 0;
  const int32_t* task_seg = nullptr;  // ntask
  const int32_t* task_g0 = nullptr;   // ntask
  const int32_t* task_g1 = nullptr;   // ntask
  const int32_t* vc_task = nullptr;   // nvc + 1
  // Task groups for dynamic scheduling (launches without reduction slots):
  // up to kCoarseGroupTasks consecutive tasks of one segment, listed by
  // decreasing modelled cost; CTAs take the next group from a counter.
  int ngroup = 0;
  const int32_t* grp_t0 = nullptr;    // ngroup: first task
  const int32_t* grp_t1 = nullptr;    // ngroup: one past the last task
  // coarse work split over the PCG's virtual CTAs: aggregates
  // [vc_agg[v], vc_agg[v+1]) (contiguous, about equal cost) go to virtual
  // CTA v; segment s owns the reduction slots [seg_aslot[s], seg_aslot[s+1])
  // of the virtual CTAs seg_avc0[s], seg_avc0[s] + 1, ...
  int nvc = 0, naslot = 0, max_seg_agg = 0;
  const int32_t* vc_agg = nullptr;     // nvc + 1
  const int32_t* seg_aslot = nullptr;  // nseg + 1
  const int32_t* seg_avc0 = nullptr;   // nseg
};

// Launch-level knobs of the persistent PCG (autotuned per device and batch
// shape; the defaults are the measured choice for batched mesh spectra).
// fold_pieces / fold_aggs: fold partial sums into per-CTA reduction slots
// when a segment has more pieces / coarse unknowns than this; ctas_per_sm:
// resident CTAs per SM to launch (1 .. 5, the kernel's register budget).
struct PcgTuning {
  int fold_pieces = 64;
  int fold_aggs = 1024;
  int ctas_per_sm = 5;
};

// Scratch needed by one persistent PCG solve of n rows x p columns (nagg:
// coarse unknowns of the two-level preconditioner, 0 otherwise).
size_t pcg_workspace_bytes(int64_t n, int p, const ChunkTable& ct, int elem_size, int precond, int64_t nagg = 0);

// Per-(segment, column) outcome codes written to `state`:
//   > 0  converged after that many iterations (1-based)
//   0    x = 0 was exact (zero right-hand side)
//   < 0  LAPY_ERR_NOCONV / LAPY_ERR_BREAKDOWN / LAPY_ERR_NAN
// `sell` (may be null) is a SELL copy of the same matrix; when given, the
// SpMM phase reads it instead of the CSR arrays.
template <typename V>
int pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals,
              const SellMatrix<V>* sell, const PcgPrecondDesc<V>& pc, int p, const ChunkTable& ct,
              const V* B, V* X, double rtol, int maxiter, int32_t* state_dev, void* ws, size_t ws_bytes,
              cudaStream_t stream, int* iters_out, const PcgTuning* tuning = nullptr);

// Mixed-precision PCG with reliable updates: FP32 Jacobi-PCG iterations
// (k32 / sell) whose correction is folded into the FP64 solution X, and
// whose residual is replaced by the FP64 residual B - K64 X, every time the
// FP32 residual of a (segment, column) has fallen by `delta` (checked every
// `ru_every` iterations).  The CG direction is kept across updates, so the
// Krylov recurrence is never restarted.  A column converges when its FP64
// residual reaches rtol * ||B||.  X32: n x p FP32 scratch.
int pcg_solve_ru(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k64, const float* k32,
                 const SellMatrix<float>* sell, const float* dinv32, int p, const ChunkTable& ct, const double* B,
                 double* X, float* X32, double rtol, double delta, int ru_every, int maxiter, int32_t* state_dev,
                 void* ws, size_t ws_bytes, cudaStream_t stream, int* iters_out, int* updates_out);

}  // namespace lapy
