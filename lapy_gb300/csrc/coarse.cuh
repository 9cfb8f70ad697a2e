// Two-level (aggregation) preconditioner for the batched PCG.
#pragma once
#include "pcg.cuh"

namespace lapy {

// Aggregates are grown by breadth-first search on the matrix graph of each
// segment up to a target size (kAggTarget rows, grown for segments above
// 0.8 kCoarseMaxDim * kAggTarget rows so the coarse dimension stays bounded);
// aggregates below a quarter of the target are merged into their most
// strongly connected neighbour.  A segment whose aggregates average fewer
// than kAggMinAvg / kAggTarget of the target gets no coarse space (its
// preconditioner stays Jacobi).
constexpr int kAggTarget = 64;
constexpr int kAggMinAvg = 40;
// Largest coarse dimension per segment that the dense inverse handles.
constexpr int kCoarseMaxDim = 2048;

// Upper bounds used to size the caller's workspace: aggregates over all
// segments, and bytes of device memory for the two-level data.
int64_t two_level_max_aggs(const int32_t* seg_row, int nseg);
size_t two_level_bytes(int64_t n, const int32_t* seg_row, int nseg, int nvc);

// Build the coarse space of K (CSR on the device, FP64 values) for the
// segments seg_row (host): aggregation on the host, Galerkin matrix W'KW and
// its dense inverse (FP64 Cholesky, stored FP32) on the device, and the
// split of the coarse work over the nvc virtual CTAs of the PCG's warp plan.
// Fills the two-level fields of `pc` (which keeps its Jacobi diagonal).
// `lab_in` (host, may be null): aggregate labels already planned
// (plan_aggregate_order), used instead of aggregating here.
int build_two_level(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k64,
                    const int32_t* seg_row, int nseg, int nvc, void* mem, size_t bytes,
                    PcgPrecondDesc<float>* pc, cudaStream_t stream, const int32_t* lab_in = nullptr,
                    int agg_target = kAggTarget);

// Row order of a batch (host, pattern on the host) that makes every
// aggregate a contiguous row range: each segment is aggregated as
// build_two_level does, its aggregates are ordered breadth-first over the
// aggregate graph, and the rows of an aggregate keep their relative order.
// perm[new] = old (rows stay in their segment); lab_new[new] = local
// aggregate id in the new order (-1 for segments without a coarse space,
// whose rows keep their order).  Neighbouring rows thereby sit in the same
// or nearby aggregates, so the gathers of a sparse product stay close.
// agg_target: rows per aggregate (at least kAggTarget, which the workspace
// bounds assume).
int plan_aggregate_order(int64_t n, const int32_t* hptr, const int32_t* hidx, const int32_t* seg_row, int nseg,
                         int32_t* perm, int32_t* lab_new, int agg_target = kAggTarget);

}  // namespace lapy
