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
struct ChunkTable {
  int nseg = 0;
  int nchunk = 0;
  int32_t* chunk_row = nullptr;  // device, nchunk + 1
  int32_t* chunk_seg = nullptr;  // device, nchunk
  int32_t* seg_chunk = nullptr;  // device, nseg + 1
  int32_t* seg_row = nullptr;    // device, nseg + 1
  int nunit = 0, npiece = 0, nvw = 0;
  int32_t* unit_row = nullptr;    // device, nunit + 1
  int32_t* piece_unit = nullptr;  // device, npiece + 1
  int32_t* piece_seg = nullptr;   // device, npiece
  int32_t* vw_piece = nullptr;    // device, nvw + 1
  int32_t* seg_piece = nullptr;   // device, nseg + 1
  std::vector<int32_t> h_seg_row;
  std::vector<int32_t> h_chunk_row, h_chunk_seg, h_seg_chunk;
  std::vector<int32_t> h_unit_row, h_piece_unit, h_piece_seg, h_vw_piece, h_seg_piece;
};

// Plan chunks (and the PCG's warp plan) for the given segments (host);
// returns the chunk count.
int plan_chunks(const int32_t* seg_row, int nseg, int target_chunks, ChunkTable* ct);
// Bytes of device memory the table needs.
size_t chunk_table_bytes(const ChunkTable& ct);
// Place the table into `mem` and upload it (synchronous on `stream`).
int upload_chunk_table(ChunkTable* ct, void* mem, cudaStream_t stream);

enum PcgPrecond { kPrecJacobi = 0, kPrecFactored = 1 };

// Preconditioner description.  Jacobi: z = dinv .* r.  Factored:
// z = Gt * (G * r) with G, Gt CSR on the mesh pattern (SPD by construction).
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
};

// Scratch needed by one persistent PCG solve of n rows x p columns.
size_t pcg_workspace_bytes(int64_t n, int p, const ChunkTable& ct, int elem_size, int precond);

// Per-(segment, column) outcome codes written to `state`:
//   > 0  converged after that many iterations (1-based)
//   0    x = 0 was exact (zero right-hand side)
//   < 0  LAPY_ERR_NOCONV / LAPY_ERR_BREAKDOWN / LAPY_ERR_NAN
template <typename V>
int pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals,
              const PcgPrecondDesc<V>& pc, int p, const ChunkTable& ct, const V* B, V* X,
              double rtol, int maxiter, int32_t* state_dev, void* ws, size_t ws_bytes,
              cudaStream_t stream, int* iters_out);

}  // namespace lapy
