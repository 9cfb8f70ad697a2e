// Two-level (aggregation) preconditioner: coarse space of a block-diagonal
// batch.
//
// Host: each segment's rows are grouped into connected aggregates by
// breadth-first growth on the matrix graph (deterministic: rows are visited
// in index order, neighbours in CSR order; segments are independent and run
// on a fixed set of host threads).  Device: the Galerkin matrix W'KW of every
// segment (one thread per coarse row, fixed summation order) and its dense
// inverse (one CTA per segment: FP64 Cholesky, triangular inverse, B'B),
// split into its dominant rank-1 term (FP32) and a BF16 remainder for the
// per-iteration coarse product of the PCG.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>
#include <cuda_bf16.h>
#include "coarse.cuh"

namespace lapy {

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// Aggregate size for a segment of `rows` rows: kAggTarget, grown for large
// segments so that the coarse dimension stays below about 0.8 kCoarseMaxDim.
static int seg_target(int64_t rows, int agg_target = kAggTarget) {
  return (int)std::max<int64_t>(std::max(agg_target, kAggTarget),
                                (rows * 5 + 4 * kCoarseMaxDim - 1) / (4 * kCoarseMaxDim));
}
// Largest accepted coarse dimension: aggregates average at least 5/8 of the target.
static int64_t seg_cap(int64_t rows) {
  if (rows <= 0) return 0;
  const int64_t min_avg = std::max<int64_t>(1, (int64_t)seg_target(rows) * kAggMinAvg / kAggTarget);
  return (rows + min_avg - 1) / min_avg;
}

int64_t two_level_max_aggs(const int32_t* seg_row, int nseg) {
  int64_t t = 0;
  for (int s = 0; s < nseg; ++s) t += std::min<int64_t>(seg_cap(seg_row[s + 1] - seg_row[s]), kCoarseMaxDim);
  return t;
}

__host__ __device__ static inline int64_t pad8(int64_t c) { return (c + 7) & ~int64_t(7); }

// Bounds over all segments: coarse entries (square blocks), padded BF16
// entries (rows rounded up to 8), and coarse-solve tasks.
static void coarse_bounds(const int32_t* seg_row, int nseg, int64_t* ne, int64_t* ne_pad, int64_t* ntask) {
  *ne = *ne_pad = *ntask = 0;
  for (int s = 0; s < nseg; ++s) {
    const int64_t c = std::min<int64_t>(seg_cap(seg_row[s + 1] - seg_row[s]), kCoarseMaxDim);
    *ne += c * c;
    *ne_pad += c * pad8(c);
    *ntask += (c + kCoarseTaskRows - 1) / kCoarseTaskRows;
  }
}

size_t two_level_bytes(int64_t n, const int32_t* seg_row, int nseg, int nvc) {
  const int64_t na = two_level_max_aggs(seg_row, nseg);
  int64_t ne, ne_pad, nt;
  coarse_bounds(seg_row, nseg, &ne, &ne_pad, &nt);
  return a256(4 * (size_t)n) * 2 + a256(4 * (size_t)(na + 1)) + a256(4 * (size_t)na) +
         a256(4 * (size_t)(nseg + 1)) + a256(8 * (size_t)(nseg + 1)) + a256(2 * (size_t)ne_pad) +
         2 * a256(8 * (size_t)ne) + a256(4 * (size_t)nseg) + a256(4 * (size_t)(std::max(nvc, 1) + 1)) * 2 +
         a256(4 * (size_t)(nseg + 1)) + a256(4 * (size_t)std::max(nseg, 1)) + a256(4 * (size_t)na) +
         a256(4 * (size_t)std::max(nseg, 1)) + 5 * a256(4 * (size_t)std::max<int64_t>(nt, 1)) +
         a256(8 * (size_t)(nseg + 1)) + 2048;
}

// ---- host aggregation -------------------------------------------------------
// Labels rows [r0, r1) with local aggregate ids 0..nc-1 (lab: global array).
// Scratch reused across the segments one host thread aggregates (no
// allocation per aggregate once the vectors have grown).
struct AggScratch {
  std::vector<int32_t> queue, parent, conn_ids, conn_cnt, remap;
  std::vector<std::vector<int32_t>> members;
};

static int aggregate_segment(int32_t r0, int32_t r1, const int32_t* indptr, const int32_t* indices,
                             int32_t* lab, int agg_target, AggScratch& sc) {
  const int32_t len = r1 - r0;
  if (len <= 0) return 0;
  const int target = seg_target(len, agg_target);
  for (int32_t v = r0; v < r1; ++v) lab[v] = -1;
  std::vector<int32_t>& queue = sc.queue;
  queue.reserve(target);
  int32_t id = 0;
  for (int32_t v = r0; v < r1; ++v) {
    if (lab[v] >= 0) continue;
    queue.clear();
    queue.push_back(v);
    lab[v] = id;
    int cnt = 1;
    for (size_t qi = 0; qi < queue.size() && cnt < target; ++qi) {
      const int32_t u = queue[qi];
      for (int32_t k = indptr[u]; k < indptr[u + 1] && cnt < target; ++k) {
        const int32_t w = indices[k];
        if (w < r0 || w >= r1 || lab[w] >= 0) continue;
        lab[w] = id;
        queue.push_back(w);
        ++cnt;
      }
    }
    ++id;
  }
  // merge aggregates below target / 4 rows into the neighbour aggregate
  // with the most connecting entries (ties: the smaller id)
  std::vector<std::vector<int32_t>>& members = sc.members;
  if ((int32_t)members.size() < id) members.resize(id);
  for (int32_t a = 0; a < id; ++a) members[a].clear();
  for (int32_t v = r0; v < r1; ++v) members[lab[v]].push_back(v);
  std::vector<int32_t>& parent = sc.parent;
  parent.resize(id);
  for (int32_t a = 0; a < id; ++a) parent[a] = a;
  auto find = [&](int32_t a) {
    while (parent[a] != a) a = parent[a] = parent[parent[a]];
    return a;
  };
  std::vector<int32_t>& conn_ids = sc.conn_ids;
  std::vector<int32_t>& conn_cnt = sc.conn_cnt;
  for (int32_t a = 0; a < id; ++a) {
    if (parent[a] != a || (int)members[a].size() >= target / 4) continue;
    conn_ids.clear();
    conn_cnt.clear();
    for (int32_t u : members[a]) {
      for (int32_t k = indptr[u]; k < indptr[u + 1]; ++k) {
        const int32_t w = indices[k];
        if (w < r0 || w >= r1) continue;
        const int32_t b = find(lab[w]);
        if (b == a) continue;
        size_t t = 0;
        while (t < conn_ids.size() && conn_ids[t] != b) ++t;
        if (t == conn_ids.size()) {
          conn_ids.push_back(b);
          conn_cnt.push_back(0);
        }
        ++conn_cnt[t];
      }
    }
    if (conn_ids.empty()) continue;  // an isolated component stays on its own
    size_t best = 0;
    for (size_t t = 1; t < conn_ids.size(); ++t)
      if (conn_cnt[t] > conn_cnt[best] || (conn_cnt[t] == conn_cnt[best] && conn_ids[t] < conn_ids[best]))
        best = t;
    const int32_t b = conn_ids[best];
    parent[a] = b;
    members[b].insert(members[b].end(), members[a].begin(), members[a].end());
    members[a].clear();
  }
  // compact: ids in order of each aggregate's first row
  std::vector<int32_t>& remap = sc.remap;
  remap.assign(id, -1);
  int32_t nc = 0;
  for (int32_t v = r0; v < r1; ++v) {
    const int32_t a = find(lab[v]);
    if (remap[a] < 0) remap[a] = nc++;
    lab[v] = remap[a];
  }
  if (nc > std::min<int64_t>(seg_cap(len), kCoarseMaxDim)) {
    for (int32_t v = r0; v < r1; ++v) lab[v] = -1;
    return 0;
  }
  return nc;
}

// ---- device kernels ---------------------------------------------------------
// Row g - seg_agg[s] of segment s's Galerkin matrix: sum of K over the
// aggregate's rows, accumulated per coarse column in row / CSR order.
__global__ void coarse_galerkin_kernel(int nagg, const int32_t* __restrict__ agg, const int32_t* __restrict__ agg_ptr,
                                       const int32_t* __restrict__ agg_row, const int32_t* __restrict__ agg_sid,
                                       const int32_t* __restrict__ seg_agg, const int64_t* __restrict__ off,
                                       const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                       const double* __restrict__ k64, double* __restrict__ kc) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nagg) return;
  const int s = agg_sid[g];
  const int base = seg_agg[s];
  const int nc = seg_agg[s + 1] - base;
  double* row = kc + off[s] + (int64_t)(g - base) * nc;
  for (int32_t m = agg_ptr[g]; m < agg_ptr[g + 1]; ++m) {
    const int32_t i = agg_row[m];
    for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
      const int32_t b = agg[indices[k]] - base;
      if (b >= 0 && b < nc) row[b] += k64[k];
    }
  }
}

constexpr int kInvThreads = 1024;
// Power iterations for the dominant eigenvector of the coarse inverse: the
// smallest eigenvalue of W'KW is the shifted constant mode, separated from
// the next by two to four orders of magnitude on mesh systems, so a few
// iterations give it to working precision; the split below stays exact for
// any v (R is formed from the same v), only the size of R depends on it.
constexpr int kPowerIters = 12;

__device__ __forceinline__ uint16_t to_bf16_bits(double x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn((float)x));
}

// In-place inverse of one SPD block A (nc x nc, row-major, FP64) per CTA:
// A = L L' (lower triangle), B = L^-1 kept transposed in the strict upper
// triangle with its diagonal in shared memory, then F = A^-1 = B'B (FP64,
// full) into `full`.  Then the dominant eigenpair of F by power iteration,
// v (unit) and c = v'Fv, and the split F = c v v' + R: v and c in FP32, R in
// BF16 (rows padded to ld = nc rounded up to 8).  A non-positive pivot leaves
// the segment's block zero (no coarse correction: the preconditioner falls
// back to Jacobi there).
__global__ void __launch_bounds__(kInvThreads) coarse_inverse_kernel(const int32_t* __restrict__ seg_agg,
                                                                     const int64_t* __restrict__ off,
                                                                     const int64_t* __restrict__ off_pad,
                                                                     double* __restrict__ kc,
                                                                     double* __restrict__ full,
                                                                     uint16_t* __restrict__ out,
                                                                     float* __restrict__ kvec,
                                                                     float* __restrict__ kscale,
                                                                     int* __restrict__ failed) {
  __shared__ double col[kCoarseMaxDim];
  __shared__ double diagb[kCoarseMaxDim];
  __shared__ double red[32];
  __shared__ int ok;
  const int s = blockIdx.x;
  const int base = seg_agg[s];
  const int nc = seg_agg[s + 1] - base;
  if (nc <= 0) return;
  const int64_t ld = pad8(nc);
  double* A = kc + off[s];
  double* F = full + off[s];
  uint16_t* O = out + off_pad[s];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = kInvThreads / 32;
  if (tid == 0) ok = 1;
  __syncthreads();
  // Cholesky, right-looking; the pivot column is staged in shared memory
  for (int k = 0; k < nc; ++k) {
    if (tid == 0) {
      const double piv = A[(int64_t)k * nc + k];
      if (!(piv > 0.0) || !isfinite(piv)) ok = 0;
      const double d = ok ? sqrt(piv) : 1.0;
      A[(int64_t)k * nc + k] = d;
      col[k] = d;
    }
    __syncthreads();
    if (!ok) break;
    const double d = col[k];
    for (int i = k + 1 + tid; i < nc; i += kInvThreads) {
      const double l = A[(int64_t)i * nc + k] / d;
      A[(int64_t)i * nc + k] = l;
      col[i] = l;
    }
    __syncthreads();
    for (int i = k + 1 + warp; i < nc; i += nwarp) {
      const double ci = col[i];
      double* Ai = A + (int64_t)i * nc;
      for (int j = k + 1 + lane; j <= i; j += 32) Ai[j] -= ci * col[j];
    }
    __syncthreads();
  }
  if (!ok) {
    for (int64_t t = tid; t < (int64_t)nc * ld; t += kInvThreads) O[t] = 0;
    for (int i = tid; i < nc; i += kInvThreads) kvec[base + i] = 0.0f;
    if (tid == 0) {
      kscale[s] = 0.0f;
      failed[s] = 1;
    }
    return;
  }
  // B = L^-1: row c of U (= column c of B) lives in A[c][c+1..nc), B[c][c] in diagb
  for (int c = tid; c < nc; c += kInvThreads) diagb[c] = 1.0;
  for (int c = warp; c < nc; c += nwarp)
    for (int i = c + 1 + lane; i < nc; i += 32) A[(int64_t)c * nc + i] = 0.0;
  __syncthreads();
  for (int j = 0; j < nc; ++j) {
    // stage column j of L and scale row j of B by 1 / L[j][j]
    for (int i = j + tid; i < nc; i += kInvThreads) col[i] = A[(int64_t)i * nc + j];
    __syncthreads();
    const double inv = 1.0 / col[j];
    for (int c = tid; c < j; c += kInvThreads) A[(int64_t)c * nc + j] *= inv;
    if (tid == 0) diagb[j] *= inv;
    __syncthreads();
    // B[i][c] -= L[i][j] B[j][c] for i > j, c <= j
    for (int c = warp; c <= j; c += nwarp) {
      const double bjc = (c < j) ? A[(int64_t)c * nc + j] : diagb[j];
      double* Uc = A + (int64_t)c * nc;
      for (int i = j + 1 + lane; i < nc; i += 32) Uc[i] -= col[i] * bjc;
    }
    __syncthreads();
  }
  // A^-1 [a][b] = sum_{i >= max(a,b)} B[i][a] B[i][b]   (rows a, b of U);
  // one warp per row a, pairs b >= a
  for (int a = warp; a < nc; a += nwarp) {
    const double* Ua = A + (int64_t)a * nc;
    for (int b = a; b < nc; ++b) {
      const double* Ub = A + (int64_t)b * nc;
      double acc = 0.0;
      for (int i = b + lane; i < nc; i += 32) {
        const double ua = (i == a) ? diagb[a] : Ua[i];
        const double ub = (i == b) ? diagb[b] : Ub[i];
        acc += ua * ub;
      }
      acc = warp_sum(acc);
      if (lane == 0) {
        F[(int64_t)a * nc + b] = acc;
        F[(int64_t)b * nc + a] = acc;
      }
    }
  }
  // dominant eigenvector of F: v <- F v / ||F v|| (v in col, F v in diagb)
  double* v = col;
  double* y = diagb;
  auto matvec = [&]() {  // y = F v, one warp per row
    __syncthreads();
    for (int a = warp; a < nc; a += nwarp) {
      const double* Fa = F + (int64_t)a * nc;
      double acc = 0.0;
      for (int b = lane; b < nc; b += 32) acc += Fa[b] * v[b];
      acc = warp_sum(acc);
      if (lane == 0) y[a] = acc;
    }
    __syncthreads();
  };
  for (int i = tid; i < nc; i += kInvThreads) v[i] = 1.0;
  for (int it = 0; it < kPowerIters; ++it) {
    matvec();
    double part = 0.0;
    for (int i = tid; i < nc; i += kInvThreads) part += y[i] * y[i];
    const double nrm = sqrt(block_sum(part, red));
    for (int i = tid; i < nc; i += kInvThreads) v[i] = y[i] / nrm;
  }
  matvec();
  double part = 0.0;
  for (int i = tid; i < nc; i += kInvThreads) part += v[i] * y[i];
  const double c = block_sum(part, red);  // v'Fv
  for (int i = tid; i < nc; i += kInvThreads) kvec[base + i] = (float)v[i];
  if (tid == 0) kscale[s] = (float)c;
  // R = F - c v v' in BF16, rows padded with zeros to ld
  for (int a = warp; a < nc; a += nwarp) {
    const double* Fa = F + (int64_t)a * nc;
    uint16_t* Oa = O + (int64_t)a * ld;
    const double cva = c * v[a];
    for (int b = lane; b < ld; b += 32) Oa[b] = (b < nc) ? to_bf16_bits(Fa[b] - cva * v[b]) : (uint16_t)0;
  }
}

// Segments largest first: host threads take them from a shared counter
// (mesh sizes differ by 64x between levels; a fixed round-robin split left
// threads idle).  Every segment writes its own rows only, so the result does
// not depend on which thread ran it.
static std::vector<int32_t> largest_first(const int32_t* seg_row, int nseg) {
  std::vector<int32_t> order(nseg);
  for (int s = 0; s < nseg; ++s) order[s] = s;
  std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
    return seg_row[a + 1] - seg_row[a] > seg_row[b + 1] - seg_row[b];
  });
  return order;
}

static int host_threads(int nseg) {
  return std::max(1, std::min<int>(nseg, std::min(16u, std::max(1u, std::thread::hardware_concurrency()))));
}

int plan_aggregate_order(int64_t n, const int32_t* hptr, const int32_t* hidx, const int32_t* seg_row, int nseg,
                         int32_t* perm, int32_t* lab_new, int agg_target) {
  // labels of this call's rows (aggregate_segment sets every row of its
  // segment); the storage is kept per calling thread across calls, like the
  // caller's copies, and handed to the workers as a plain pointer
  thread_local std::vector<int32_t> lab_store;
  if ((int64_t)lab_store.size() < n) lab_store.resize(n);
  int32_t* const lab = lab_store.data();
  const int nthr = host_threads(nseg);
  const std::vector<int32_t> sorder = largest_first(seg_row, nseg);
  std::atomic<int> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < nthr; ++t)
    pool.emplace_back([&]() {
      std::vector<int32_t> order, first, cnt, fill, agg_order, agg_rank;
      AggScratch sc;
      for (int i = next.fetch_add(1); i < nseg; i = next.fetch_add(1)) {
        const int s = sorder[i];
        const int32_t r0 = seg_row[s], r1 = seg_row[s + 1];
        const int nc = aggregate_segment(r0, r1, hptr, hidx, lab, agg_target, sc);
        if (nc <= 0) {  // no coarse space: rows keep their order, no aggregate
          for (int32_t v = r0; v < r1; ++v) {
            perm[v] = v;
            lab_new[v] = -1;
          }
          continue;
        }
        // aggregates in breadth-first order over the aggregate graph (from
        // the aggregate of the segment's first row; neighbours in the order
        // their member rows and CSR entries are met), so that neighbouring
        // aggregates get nearby numbers
        cnt.assign(nc + 1, 0);
        for (int32_t v = r0; v < r1; ++v) ++cnt[lab[v] + 1];
        for (int g = 0; g < nc; ++g) cnt[g + 1] += cnt[g];
        order.resize(r1 - r0);
        fill.assign(cnt.begin(), cnt.end() - 1);
        for (int32_t v = r0; v < r1; ++v) order[fill[lab[v]]++] = v;  // members, rows ascending
        agg_rank.assign(nc, -1);
        agg_order.clear();
        for (int seed = 0; seed < nc; ++seed) {
          if (agg_rank[seed] >= 0) continue;
          agg_rank[seed] = (int32_t)agg_order.size();
          agg_order.push_back(seed);
          for (size_t qi = agg_order.size() - 1; qi < agg_order.size(); ++qi) {
            const int g = agg_order[qi];
            for (int32_t m = cnt[g]; m < cnt[g + 1]; ++m) {
              const int32_t u = order[m];
              for (int32_t k = hptr[u]; k < hptr[u + 1]; ++k) {
                const int32_t w = hidx[k];
                if (w < r0 || w >= r1) continue;
                const int32_t h = lab[w];
                if (h >= 0 && agg_rank[h] < 0) {
                  agg_rank[h] = (int32_t)agg_order.size();
                  agg_order.push_back(h);
                }
              }
            }
          }
        }
        int32_t pos = r0;
        for (int i = 0; i < nc; ++i) {
          const int g = agg_order[i];
          for (int32_t m = cnt[g]; m < cnt[g + 1]; ++m) {
            perm[pos] = order[m];
            lab_new[pos] = i;
            ++pos;
          }
        }
      }
    });
  for (auto& th : pool) th.join();
  return LAPY_OK;
}

int build_two_level(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k64,
                    const int32_t* seg_row, int nseg, int nvc, void* mem, size_t bytes,
                    PcgPrecondDesc<float>* pc, cudaStream_t stream, const int32_t* lab_in, int agg_target) {
  nvc = std::max(nvc, 1);
  if (bytes < two_level_bytes(n, seg_row, nseg, nvc)) return LAPY_ERR_WORKSPACE;
  std::vector<int32_t> lab(n, -1), nc(nseg, 0);
  bool contiguous = false;
  if (lab_in) {
    // labels given (local aggregate ids, rows of an aggregate contiguous and
    // aggregates numbered in row order)
    std::copy(lab_in, lab_in + n, lab.begin());
    contiguous = true;
    for (int s = 0; s < nseg; ++s) {
      int32_t mx = -1;
      for (int32_t v = seg_row[s]; v < seg_row[s + 1]; ++v) {
        if (lab[v] < mx || lab[v] > mx + 1) contiguous = false;
        mx = std::max(mx, lab[v]);
      }
      nc[s] = mx + 1;
    }
  } else {
    // pattern to the host, aggregation there
    std::vector<int32_t> hptr(n + 1);
    LAPY_CUDA_TRY(cudaMemcpyAsync(hptr.data(), indptr, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost, stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
    const int64_t nnz = hptr[n];
    std::vector<int32_t> hidx(nnz);
    LAPY_CUDA_TRY(cudaMemcpyAsync(hidx.data(), indices, 4 * (size_t)nnz, cudaMemcpyDeviceToHost, stream));
    LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
    const int nthr = host_threads(nseg);
    const std::vector<int32_t> sorder = largest_first(seg_row, nseg);
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < nthr; ++t)
      pool.emplace_back([&]() {
        AggScratch sc;
        for (int i = next.fetch_add(1); i < nseg; i = next.fetch_add(1)) {
          const int s = sorder[i];
          nc[s] = aggregate_segment(seg_row[s], seg_row[s + 1], hptr.data(), hidx.data(), lab.data(), agg_target,
                                    sc);
        }
      });
    for (auto& th : pool) th.join();
  }
  std::vector<int32_t> seg_agg(nseg + 1, 0);
  std::vector<int64_t> off(nseg + 1, 0), off_pad(nseg + 1, 0);
  for (int s = 0; s < nseg; ++s) {
    seg_agg[s + 1] = seg_agg[s] + nc[s];
    off[s + 1] = off[s] + (int64_t)nc[s] * nc[s];
    off_pad[s + 1] = off_pad[s] + (int64_t)nc[s] * pad8(nc[s]);
  }
  const int nagg = seg_agg[nseg];
  std::vector<int32_t> agg(n, -1), agg_sid(nagg), agg_ptr(nagg + 1, 0), agg_row;
  for (int s = 0; s < nseg; ++s)
    for (int32_t v = seg_row[s]; v < seg_row[s + 1]; ++v)
      if (lab[v] >= 0) agg[v] = seg_agg[s] + lab[v];
  for (int s = 0; s < nseg; ++s)
    for (int g = seg_agg[s]; g < seg_agg[s + 1]; ++g) agg_sid[g] = s;
  for (int64_t v = 0; v < n; ++v)
    if (agg[v] >= 0) ++agg_ptr[agg[v] + 1];
  for (int g = 0; g < nagg; ++g) agg_ptr[g + 1] += agg_ptr[g];
  agg_row.resize(agg_ptr[nagg]);
  {
    std::vector<int32_t> fill(agg_ptr.begin(), agg_ptr.end() - 1);
    for (int64_t v = 0; v < n; ++v)
      if (agg[v] >= 0) agg_row[fill[agg[v]]++] = (int32_t)v;
  }

  // coarse-solve tasks (up to kCoarseTaskRows coarse rows of one segment),
  // split over the virtual CTAs in contiguous ranges of about equal time.  A
  // task's time (ns) is modelled as a fixed part (its descriptor loads), a
  // latency per warp pass (each warp computes kCoarseRowsPerPass rows per
  // pass) plus one per 128-entry row group the pass streams, and, for the
  // first task of a segment, the staging of the segment's residual (three
  // CTA barriers).  The constants are a non-negative least-squares fit of
  // per-CTA busy times measured with device timers on 512 meshes (levels
  // 3-6): the BF16 bytes themselves did not matter, the dependent round
  // trips did, so small segments' tasks cost several times what their bytes
  // suggest.  Tasks of 16 rows (one pass) keep the split fine-grained: with
  // 32-row tasks one level-6 task was a fifth of a virtual CTA's share and
  // the busiest CTA ran a third longer than the mean.  The aggregates of a virtual CTA's tasks
  // are also its share of the restriction, and the reduction slots of each
  // segment's coarse partial sums follow from that split.
  std::vector<int32_t> task_seg, task_g0, task_g1;
  std::vector<double> task_cost;
  for (int s = 0; s < nseg; ++s)
    for (int g = seg_agg[s]; g < seg_agg[s + 1]; g += kCoarseTaskRows) {
      const int g1 = std::min(g + kCoarseTaskRows, seg_agg[s + 1]);
      task_seg.push_back(s);
      task_g0.push_back(g);
      task_g1.push_back(g1);
      const int rows = g1 - g;
      const double passes = (double)((rows + kWarpsPerCta * kCoarseRowsPerPass - 1) /
                                     (kWarpsPerCta * kCoarseRowsPerPass));
      const double groups = (double)((pad8(nc[s]) + 127) / 128);
      const bool first = g == seg_agg[s];
      task_cost.push_back(1900.0 + (first ? 1600.0 : 0.0) + passes * (800.0 + 800.0 * groups));
    }
  const int ntask = (int)task_seg.size();
  // groups of up to kCoarseGroupTasks consecutive tasks of one segment, in
  // decreasing order of modelled cost (the cheap groups of small segments
  // last, where they even out the CTAs' finishing times)
  std::vector<int32_t> grp_t0, grp_t1;
  {
    std::vector<std::pair<double, int>> order;
    std::vector<int32_t> g0v, g1v;
    for (int t = 0; t < ntask;) {
      int t1 = t + 1;
      while (t1 < ntask && t1 - t < kCoarseGroupTasks && task_seg[t1] == task_seg[t]) ++t1;
      double c = 0.0;
      for (int q = t; q < t1; ++q) c += task_cost[q];
      order.push_back({-c, (int)g0v.size()});
      g0v.push_back(t);
      g1v.push_back(t1);
      t = t1;
    }
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<double, int>& x, const std::pair<double, int>& y) { return x.first < y.first; });
    for (const auto& o : order) {
      grp_t0.push_back(g0v[o.second]);
      grp_t1.push_back(g1v[o.second]);
    }
  }
  const int ngroup = (int)grp_t0.size();
  std::vector<int32_t> vc_task(nvc + 1, 0);
  {
    double total = 0.0;
    for (double c : task_cost) total += c;
    double acc = 0.0;
    int v = 1;
    for (int t = 0; t < ntask; ++t) {
      acc += task_cost[t];
      while (v < nvc && acc >= total * v / nvc) vc_task[v++] = t + 1;
    }
    while (v <= nvc) vc_task[v++] = ntask;
  }
  std::vector<int32_t> vc_agg(nvc + 1, 0), seg_aslot(nseg + 1, 0), seg_avc0(std::max(nseg, 1), 0);
  {
    for (int v = 0; v <= nvc; ++v) vc_agg[v] = vc_task[v] < ntask ? task_g0[vc_task[v]] : nagg;
    auto vc_of = [&](int32_t g) {
      return (int)(std::upper_bound(vc_agg.begin(), vc_agg.end(), g) - vc_agg.begin()) - 1;
    };
    for (int s = 0; s < nseg; ++s) {
      int ns = 0;
      if (nc[s] > 0) {
        seg_avc0[s] = vc_of(seg_agg[s]);
        ns = vc_of(seg_agg[s + 1] - 1) - seg_avc0[s] + 1;
      }
      seg_aslot[s + 1] = seg_aslot[s] + ns;
    }
  }

  // device layout
  char* w = (char*)(((uintptr_t)mem + 255) & ~uintptr_t(255));
  const int64_t na_max = two_level_max_aggs(seg_row, nseg);
  int64_t ne_max, ne_pad_max, nt_max;
  coarse_bounds(seg_row, nseg, &ne_max, &ne_pad_max, &nt_max);
  if (nagg > na_max || off[nseg] > ne_max || off_pad[nseg] > ne_pad_max || ntask > nt_max) {
    lapy_set_last_message("two-level: coarse space exceeds its bound");
    return LAPY_ERR_WORKSPACE;
  }
  int32_t* d_agg = (int32_t*)w; w += a256(4 * (size_t)n);
  int32_t* d_row = (int32_t*)w; w += a256(4 * (size_t)n);
  int32_t* d_ptr = (int32_t*)w; w += a256(4 * (size_t)(na_max + 1));
  int32_t* d_sid = (int32_t*)w; w += a256(4 * (size_t)na_max);
  int32_t* d_seg = (int32_t*)w; w += a256(4 * (size_t)(nseg + 1));
  int64_t* d_off = (int64_t*)w; w += a256(8 * (size_t)(nseg + 1));
  uint16_t* d_kinv = (uint16_t*)w; w += a256(2 * (size_t)ne_pad_max);
  double* d_kc = (double*)w; w += a256(8 * (size_t)ne_max);
  double* d_full = (double*)w; w += a256(8 * (size_t)ne_max);
  int32_t* d_vca = (int32_t*)w; w += a256(4 * (size_t)(nvc + 1));
  int32_t* d_asl = (int32_t*)w; w += a256(4 * (size_t)(nseg + 1));
  int32_t* d_av0 = (int32_t*)w; w += a256(4 * (size_t)std::max(nseg, 1));
  float* d_kvec = (float*)w; w += a256(4 * (size_t)na_max);
  float* d_kscale = (float*)w; w += a256(4 * (size_t)std::max(nseg, 1));
  int32_t* d_tseg = (int32_t*)w; w += a256(4 * (size_t)std::max<int64_t>(nt_max, 1));
  int32_t* d_tg0 = (int32_t*)w; w += a256(4 * (size_t)std::max<int64_t>(nt_max, 1));
  int32_t* d_tg1 = (int32_t*)w; w += a256(4 * (size_t)std::max<int64_t>(nt_max, 1));
  int32_t* d_vct = (int32_t*)w; w += a256(4 * (size_t)(nvc + 1));
  int32_t* d_gt0 = (int32_t*)w; w += a256(4 * (size_t)std::max<int64_t>(nt_max, 1));
  int32_t* d_gt1 = (int32_t*)w; w += a256(4 * (size_t)std::max<int64_t>(nt_max, 1));
  int64_t* d_offp = (int64_t*)w; w += a256(8 * (size_t)(nseg + 1));
  int* d_fail = (int*)w;
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_agg, agg.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, stream));
  if (!agg_row.empty())
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_row, agg_row.data(), 4 * agg_row.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_ptr, agg_ptr.data(), 4 * agg_ptr.size(), cudaMemcpyHostToDevice, stream));
  if (nagg > 0)
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_sid, agg_sid.data(), 4 * (size_t)nagg, cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_seg, seg_agg.data(), 4 * seg_agg.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_off, off.data(), 8 * off.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_vca, vc_agg.data(), 4 * vc_agg.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_asl, seg_aslot.data(), 4 * seg_aslot.size(), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_av0, seg_avc0.data(), 4 * seg_avc0.size(), cudaMemcpyHostToDevice, stream));
  if (ntask > 0) {
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_tseg, task_seg.data(), 4 * (size_t)ntask, cudaMemcpyHostToDevice, stream));
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_tg0, task_g0.data(), 4 * (size_t)ntask, cudaMemcpyHostToDevice, stream));
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_tg1, task_g1.data(), 4 * (size_t)ntask, cudaMemcpyHostToDevice, stream));
  }
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_vct, vc_task.data(), 4 * vc_task.size(), cudaMemcpyHostToDevice, stream));
  if (ngroup > 0) {
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_gt0, grp_t0.data(), 4 * (size_t)ngroup, cudaMemcpyHostToDevice, stream));
    LAPY_CUDA_TRY(cudaMemcpyAsync(d_gt1, grp_t1.data(), 4 * (size_t)ngroup, cudaMemcpyHostToDevice, stream));
  }
  LAPY_CUDA_TRY(cudaMemcpyAsync(d_offp, off_pad.data(), 8 * off_pad.size(), cudaMemcpyHostToDevice, stream));
  if (off[nseg] > 0) LAPY_CUDA_TRY(cudaMemsetAsync(d_kc, 0, 8 * (size_t)off[nseg], stream));
  LAPY_CUDA_TRY(cudaMemsetAsync(d_fail, 0, 4 * (size_t)nseg, stream));
  if (nagg > 0) {
    coarse_galerkin_kernel<<<lapy_ceil_div(nagg, 128), 128, 0, stream>>>(nagg, d_agg, d_ptr, d_row, d_sid, d_seg, d_off,
                                                                         indptr, indices, k64, d_kc);
    LAPY_TRY(lapy_check_launch("coarse_galerkin_kernel"));
    coarse_inverse_kernel<<<nseg, kInvThreads, 0, stream>>>(d_seg, d_off, d_offp, d_kc, d_full, d_kinv, d_kvec,
                                                            d_kscale, d_fail);
    LAPY_TRY(lapy_check_launch("coarse_inverse_kernel"));
  }
  // the host vectors are pageable: the copies complete before they go away
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  pc->kind = kPrecTwoLevel;
  pc->nagg = nagg;
  pc->agg = d_agg;
  pc->agg_ptr = d_ptr;
  pc->agg_row = d_row;
  pc->agg_sid = d_sid;
  pc->seg_agg = d_seg;
  pc->agg_contig = contiguous ? 1 : 0;
  pc->kinv_off = d_offp;
  pc->kinv = d_kinv;
  pc->kvec = d_kvec;
  pc->kscale = d_kscale;
  pc->ntask = ntask;
  pc->task_seg = d_tseg;
  pc->task_g0 = d_tg0;
  pc->task_g1 = d_tg1;
  pc->vc_task = d_vct;
  pc->ngroup = ngroup;
  pc->grp_t0 = d_gt0;
  pc->grp_t1 = d_gt1;
  pc->nvc = nvc;
  pc->naslot = seg_aslot[nseg];
  pc->max_seg_agg = nseg > 0 ? *std::max_element(nc.begin(), nc.end()) : 0;
  pc->vc_agg = d_vca;
  pc->seg_aslot = d_asl;
  pc->seg_avc0 = d_av0;
  return LAPY_OK;
}

}  // namespace lapy

extern "C" int lapy_aggregate_order(int64_t n, const int32_t* indptr, const int32_t* indices, const int32_t* seg_row,
                                    int nseg, int agg_target, int32_t* perm, int32_t* labels) {
  using namespace lapy;
  if (n < 0 || nseg < 0 || !seg_row || (n > 0 && (!indptr || !indices || !perm || !labels)) ||
      agg_target < kAggTarget || agg_target > 1024) {
    lapy_set_last_message("aggregate_order: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (seg_row[0] != 0 || seg_row[nseg] != n) {
    lapy_set_last_message("aggregate_order: segment rows must span [0, n)");
    return LAPY_ERR_INVALID;
  }
  for (int s = 0; s < nseg; ++s)
    if (seg_row[s + 1] < seg_row[s]) {
      lapy_set_last_message("aggregate_order: segment rows must not decrease");
      return LAPY_ERR_INVALID;
    }
  if (n == 0) return LAPY_OK;
  return plan_aggregate_order(n, indptr, indices, seg_row, nseg, perm, labels, agg_target);
}
