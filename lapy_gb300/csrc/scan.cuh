// Device-wide exclusive prefix sum of int32 counts (deterministic, 3 passes).
#pragma once
#include "common.cuh"

namespace lapy {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// Scratch (in int32 units) needed for a scan of n elements.
inline int64_t scan_scratch_elems(int64_t n) { return (int64_t)lapy_ceil_div(n, kScanTile) + 1; }

// out[0..n] = exclusive scan of in[0..n-1]; out[n] = total.  `scratch` holds
// scan_scratch_elems(n) int32.  Totals must fit int32 (checked by callers).
int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* scratch,
                       cudaStream_t stream);

}  // namespace lapy
