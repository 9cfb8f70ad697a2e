// Persistent cooperative PCG over a block-diagonal batch of CSR systems.
//
// One cooperative launch runs the whole solve, warp-centric: the rows are cut
// into 32-row units (one row per lane), every virtual warp owns a contiguous,
// row-balanced range of units, and that range is split at segment (mesh)
// boundaries into pieces.  A piece accumulates its dot-product partials in
// registers and writes one slot per column; after a grid barrier, any warp
// that needs a segment's scalar sums that segment's few slots in a fixed
// order (bitwise reproducible).  Warps never wait for one another except at
// the grid barriers: three per iteration with the Jacobi preconditioner, five
// with the factored one z = Gt (G r).  Convergence is tracked per (segment,
// column): converged columns freeze and converged segments skip their rows.
// The SpMM stages each unit's contiguous slice of the matrix in the warp's
// part of shared memory with coalesced loads before the per-row gathers.
// Barriers spin with a bound (common.cuh).
#include <climits>
#include <type_traits>
#include <cmath>
#include <cstring>
#include "pcg.cuh"
#include "blas.cuh"
#include "scan.cuh"

namespace lapy {

constexpr int32_t kActive = INT32_MAX;
constexpr int kPcgThreads = 256;
constexpr int kWarps = kPcgThreads / 32;
constexpr int kUnit = 32;
constexpr int kStageWarp = 384;   // staged nonzeros per warp (values + column indices)
constexpr int kSellShort = 8;     // SELL slices up to this width take the all-loads-first path
constexpr int kPlanCtasPerSm = 5; // resident CTAs per SM the warp plan assumes (48 registers)



static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

int plan_chunks(const int32_t* seg_row, int nseg, int target_chunks, ChunkTable* ct, int max_rows) {
  const int64_t total = seg_row[nseg] - seg_row[0];
  int64_t cr = (total + std::max(1, target_chunks) - 1) / std::max(1, target_chunks);
  cr = std::max<int64_t>(32, std::min<int64_t>(std::max(32, max_rows), cr));
  cr = (cr + 31) / 32 * 32;
  ct->nseg = nseg;
  ct->h_seg_row.assign(seg_row, seg_row + nseg + 1);
  ct->h_chunk_row.clear();
  ct->h_chunk_seg.clear();
  ct->h_seg_chunk.assign(nseg + 1, 0);
  std::vector<int32_t> unit_seg;
  ct->h_unit_row.clear();
  for (int s = 0; s < nseg; ++s) {
    ct->h_seg_chunk[s] = (int32_t)ct->h_chunk_seg.size();
    const int64_t r0 = seg_row[s], r1 = seg_row[s + 1];
    const int64_t len = r1 - r0;
    const int64_t nc = std::max<int64_t>(1, (len + cr - 1) / cr);
    for (int64_t k = 0; k < nc; ++k) {
      ct->h_chunk_row.push_back((int32_t)(r0 + len * k / nc));
      ct->h_chunk_seg.push_back(s);
    }
    for (int64_t r = r0; r < r1; r += kUnit) {
      ct->h_unit_row.push_back((int32_t)r);
      unit_seg.push_back(s);
    }
  }
  ct->h_seg_chunk[nseg] = (int32_t)ct->h_chunk_seg.size();
  ct->h_chunk_row.push_back(seg_row[nseg]);
  ct->nchunk = (int)ct->h_chunk_seg.size();
  ct->h_unit_row.push_back(seg_row[nseg]);
  ct->nunit = (int)unit_seg.size();

  // virtual warps: contiguous unit ranges with about total/nvw rows each;
  // ranges that received no unit are dropped, so every virtual warp (and
  // every virtual CTA below) holds at least one piece
  const int nvw0 = std::max(1, std::min(ct->nunit, kPlanCtasPerSm * kWarps * lapy_num_sms()));
  std::vector<int32_t> ub;
  ub.reserve(nvw0 + 1);
  ub.push_back(0);
  for (int w = 1; w <= nvw0; ++w) {
    const int64_t target = seg_row[0] + total * w / nvw0;
    int32_t b = (int32_t)(std::lower_bound(ct->h_unit_row.begin(), ct->h_unit_row.begin() + ct->nunit,
                                           (int32_t)target) - ct->h_unit_row.begin());
    if (w == nvw0) b = ct->nunit;
    if (b > ub.back()) ub.push_back(b);
  }
  if (ub.size() == 1) ub.push_back(ct->nunit);  // no units at all: one empty virtual warp
  const int nvw = (int)ub.size() - 1;
  ct->nvw = nvw;
  ct->h_piece_unit.clear();
  ct->h_piece_seg.clear();
  ct->h_vw_piece.assign(nvw + 1, 0);
  for (int w = 0; w < nvw; ++w) {
    ct->h_vw_piece[w] = (int32_t)ct->h_piece_seg.size();
    for (int32_t u = ub[w]; u < ub[w + 1]; ++u) {
      if (u == ub[w] || unit_seg[u] != unit_seg[u - 1]) {
        ct->h_piece_unit.push_back(u);
        ct->h_piece_seg.push_back(unit_seg[u]);
      }
    }
  }
  ct->npiece = (int)ct->h_piece_seg.size();
  ct->h_vw_piece[nvw] = ct->npiece;
  ct->h_piece_unit.push_back(ct->nunit);
  ct->h_seg_piece.assign(nseg + 1, ct->npiece);
  for (int p = ct->npiece - 1; p >= 0; --p) ct->h_seg_piece[ct->h_piece_seg[p]] = p;
  for (int s = nseg - 1; s >= 0; --s)  // segments without rows: empty piece range
    if (ct->h_seg_piece[s] > ct->h_seg_piece[s + 1]) ct->h_seg_piece[s] = ct->h_seg_piece[s + 1];

  // virtual CTAs and the reduction slots of every segment
  const int nvc = (nvw + kWarps - 1) / kWarps;
  ct->nvc = nvc;
  ct->h_vc_piece.resize(nvc + 1);
  for (int v = 0; v <= nvc; ++v) ct->h_vc_piece[v] = ct->h_vw_piece[std::min(v * kWarps, nvw)];
  std::vector<int32_t> piece_vc(ct->npiece);
  for (int w = 0; w < nvw; ++w)
    for (int32_t q = ct->h_vw_piece[w]; q < ct->h_vw_piece[w + 1]; ++q) piece_vc[q] = w / kWarps;
  ct->h_seg_slot.assign(nseg + 1, 0);
  ct->h_seg_vc0.assign(nseg, 0);
  for (int s = 0; s < nseg; ++s) {
    const int32_t q0 = ct->h_seg_piece[s], q1 = ct->h_seg_piece[s + 1];
    int ns = 0;
    if (q0 < q1) {
      ct->h_seg_vc0[s] = piece_vc[q0];
      ns = piece_vc[q1 - 1] - piece_vc[q0] + 1;
    }
    ct->h_seg_slot[s + 1] = ct->h_seg_slot[s] + ns;
  }
  ct->nslot = ct->h_seg_slot[nseg];
  return ct->nchunk;
}

size_t chunk_table_bytes(const ChunkTable& ct) {
  return a256(4 * (size_t)(ct.nchunk + 1)) + a256(4 * (size_t)ct.nchunk) + a256(4 * (size_t)(ct.nseg + 1)) * 3 +
         a256(4 * (size_t)(ct.nunit + 1)) + a256(4 * (size_t)(ct.npiece + 1)) + a256(4 * (size_t)ct.npiece) +
         a256(4 * (size_t)(ct.nvw + 1)) + a256(4 * (size_t)(ct.nvc + 1)) + a256(4 * (size_t)(ct.nseg + 1)) +
         a256(4 * (size_t)std::max(ct.nseg, 1)) + a256(8 * (size_t)kChunkScratch * std::max(ct.nchunk, 1));
}

int upload_chunk_table(ChunkTable* ct, void* mem, cudaStream_t stream) {
  char* p = (char*)mem;
  auto put = [&](int32_t** dst, const std::vector<int32_t>& src) -> int {
    *dst = (int32_t*)p;
    p += a256(4 * src.size());
    LAPY_CUDA_TRY(cudaMemcpyAsync(*dst, src.data(), 4 * src.size(), cudaMemcpyHostToDevice, stream));
    return LAPY_OK;
  };
  LAPY_TRY(put(&ct->chunk_row, ct->h_chunk_row));
  LAPY_TRY(put(&ct->chunk_seg, ct->h_chunk_seg));
  LAPY_TRY(put(&ct->seg_chunk, ct->h_seg_chunk));
  LAPY_TRY(put(&ct->seg_row, ct->h_seg_row));
  LAPY_TRY(put(&ct->unit_row, ct->h_unit_row));
  LAPY_TRY(put(&ct->piece_unit, ct->h_piece_unit));
  LAPY_TRY(put(&ct->piece_seg, ct->h_piece_seg));
  LAPY_TRY(put(&ct->vw_piece, ct->h_vw_piece));
  LAPY_TRY(put(&ct->seg_piece, ct->h_seg_piece));
  LAPY_TRY(put(&ct->vc_piece, ct->h_vc_piece));
  LAPY_TRY(put(&ct->seg_slot, ct->h_seg_slot));
  LAPY_TRY(put(&ct->seg_vc0, ct->h_seg_vc0));
  ct->scratch = (double*)p;
  p += a256(8 * (size_t)kChunkScratch * std::max(ct->nchunk, 1));
  // pageable sources: the copies must complete before the host vectors change
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}

// Scalar (dot product) type: FP32 for FP32 iterations, FP64 for FP64 ones.
template <typename V>
using ScalarOf = typename std::conditional<sizeof(V) == 4, float, double>::type;

template <typename V>
struct PcgArgs {
  using S = ScalarOf<V>;
  int64_t n;
  const int32_t* indptr;
  const int32_t* indices;
  const V* vals;
  SellMatrix<V> sell;
  int use_sell;
  PcgPrecondDesc<V> pc;
  const int32_t* unit_row;
  const int32_t* piece_unit;
  const int32_t* piece_seg;
  const int32_t* vw_piece;
  const int32_t* seg_piece;
  const int32_t* vc_piece;  // virtual CTAs (8 virtual warps) and reduction slots
  const int32_t* seg_slot;
  const int32_t* seg_vc0;
  int nvw;
  int npiece;
  int nseg;
  int nvc;
  int nslot;
  int fold;  // fold partial sums into reduction slots (segments with many pieces)
  const V* B;
  V* X;
  V* R;
  V* P;
  V* Q;
  V* Z;
  V* T;
  S* part;            // [3][npiece][NP]  pq, rz, rr
  S* slot;            // [3][nslot][NP]   the same folded per virtual CTA
  S* aslot;           // [naslot][NP]     csl folded per virtual CTA (two-level)
  S* rc;              // [nagg][NP] restricted residual W'r   (two-level)
  S* yc;              // [nagg][NP] coarse solution (W'KW)^-1 W'r
  S* csl;             // [nagg][NP] rc .* yc (coarse part of r'z)
  S* rc_part;         // [2][npiece][NP] partial rc of aggregates that straddle pieces
  int32_t* rc_cnt;    // [nagg] arrivals at a straddling aggregate (zero between phases)
  unsigned* cq;       // [2] coarse task-group counters, used by alternate coarse phases
  S* rz;              // [2][nseg][NP]
  S* bb;              // [nseg][NP]
  int32_t* state;     // [2][nseg][NP]
  int32_t* state_out; // [nseg][NP]
  int* iters;         // [1]
  unsigned long long* work;  // [2] rows and nonzeros processed by the SpMM phase
  S rtol2;
  int maxiter;
  GridBarrier bar;
  // reliable updates (RU variant): FP64 right-hand side, solution and matrix;
  // X above is then the FP32 correction accumulated since the last update
  const double* B64;   // n x NP
  double* X64;         // n x NP
  const double* K64;   // FP64 values on indptr / indices
  double* part64;      // [npiece][NP]  partial ||b - K x||^2
  double* slot64;      // [nslot][NP]   the same folded per virtual CTA
  S* rref;             // [nseg][NP]    squared residual at the last update
  int32_t* ru_col;     // [2][nseg][NP] update requests (by parity)
  unsigned* ru_flag;   // [2]           any request (by parity)
  unsigned* n_updates; // [1]           update sweeps performed
  double rtol2_64;
  S delta2;
  int ru_every;
  unsigned long long* phase_ns;  // [kPcgPhases] device time per phase (profile mode), or null
  unsigned long long* cwork;     // [1] BF16 bytes of the coarse inverse streamed by the coarse solves
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// NP consecutive values of row `row` (vectorised: rows are NP * sizeof(V)
// aligned because every buffer starts on a 256-byte boundary).
template <typename V, int NP>
__device__ __forceinline__ void load_row(const V* __restrict__ base, int64_t row, V (&out)[NP]) {
  const V* p = base + row * NP;
  if constexpr (sizeof(V) == 4 && NP % 4 == 0) {
#pragma unroll
    for (int j = 0; j < NP / 4; ++j) {
      const float4 v = reinterpret_cast<const float4*>(p)[j];
      out[4 * j] = v.x; out[4 * j + 1] = v.y; out[4 * j + 2] = v.z; out[4 * j + 3] = v.w;
    }
  } else if constexpr (sizeof(V) == 4 && NP == 2) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    out[0] = v.x; out[1] = v.y;
  } else if constexpr (sizeof(V) == 8 && NP % 2 == 0) {
#pragma unroll
    for (int j = 0; j < NP / 2; ++j) {
      const double2 v = reinterpret_cast<const double2*>(p)[j];
      out[2 * j] = v.x; out[2 * j + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < NP; ++j) out[j] = p[j];
  }
}

template <typename V, int NP>
__device__ __forceinline__ void store_row(V* __restrict__ base, int64_t row, const V (&v)[NP]) {
  V* p = base + row * NP;
  if constexpr (sizeof(V) == 4 && NP % 4 == 0) {
#pragma unroll
    for (int j = 0; j < NP / 4; ++j)
      reinterpret_cast<float4*>(p)[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
  } else if constexpr (sizeof(V) == 4 && NP == 2) {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  } else if constexpr (sizeof(V) == 8 && NP % 2 == 0) {
#pragma unroll
    for (int j = 0; j < NP / 2; ++j) reinterpret_cast<double2*>(p)[j] = make_double2(v[2 * j], v[2 * j + 1]);
  } else {
#pragma unroll
    for (int j = 0; j < NP; ++j) p[j] = v[j];
  }
}

// Sum of a segment's piece slots for every column; afterwards each lane holds
// all NP totals in tot[] (fixed summation order).  FP32 throughout: the
// iteration's vectors are FP32, and FP64 arithmetic is scarce on this part.
// The slots [p0, p1) form one contiguous array of (p1 - p0) * NP values; when
// NP spans two or more 16-byte vectors, lanes stream it as vectors (a lane
// always lands on the same VEC columns), two vectors in flight per lane, so
// a segment of a few hundred pieces costs a few memory round trips; narrower
// rows keep one value per lane with four loads in flight (fewer registers).
template <int NP, typename S>
__device__ __forceinline__ void seg_totals(const S* __restrict__ part, int p0, int p1, S (&tot)[NP]) {
  const int lane = threadIdx.x & 31;
  constexpr int VEC = 16 / (int)sizeof(S);
  if constexpr (NP % VEC == 0 && NP >= 2 * VEC && NP <= 32 * VEC) {
    using Vec = typename std::conditional<sizeof(S) == 4, float4, double2>::type;
    const Vec* base = reinterpret_cast<const Vec*>(part + (int64_t)p0 * NP);
    const int nv = (p1 - p0) * (NP / VEC);
    S acc[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) acc[j] = S(0);
    auto add = [&](const Vec& v) {
      if constexpr (sizeof(S) == 4) {
        acc[0] += v.x; acc[1] += v.y; acc[2 % VEC] += v.z; acc[3 % VEC] += v.w;
      } else {
        acc[0] += v.x; acc[1 % VEC] += v.y;
      }
    };
    int i = lane;
    for (; i + 32 < nv; i += 64) {
      const Vec v0 = base[i], v1 = base[i + 32];
      add(v0); add(v1);
    }
    if (i < nv) add(base[i]);
    // lanes l and l' hold the same columns when l = l' mod NP / VEC
#pragma unroll
    for (int o = 16; o >= NP / VEC && o > 0; o >>= 1) {
#pragma unroll
      for (int j = 0; j < VEC; ++j) acc[j] += __shfl_xor_sync(0xffffffffu, acc[j], o);
    }
#pragma unroll
    for (int q = 0; q < NP; ++q) tot[q] = __shfl_sync(0xffffffffu, acc[q % VEC], q / VEC);
  } else {
    constexpr int SPAN = (NP <= 32) ? 32 / NP : 1;
    S acc = S(0);
    int p = p0 + lane / NP;
    for (; p + 3 * SPAN < p1; p += 4 * SPAN) {
      const S a0 = part[(int64_t)p * NP + (lane % NP)], a1 = part[(int64_t)(p + SPAN) * NP + (lane % NP)];
      const S a2 = part[(int64_t)(p + 2 * SPAN) * NP + (lane % NP)];
      const S a3 = part[(int64_t)(p + 3 * SPAN) * NP + (lane % NP)];
      acc += (a0 + a1) + (a2 + a3);
    }
    for (; p < p1; p += SPAN) acc += part[(int64_t)p * NP + (lane % NP)];
#pragma unroll
    for (int o = 16; o >= NP; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
#pragma unroll
    for (int q = 0; q < NP; ++q) tot[q] = __shfl_sync(0xffffffffu, acc, q);
  }
}

// Warp-reduce per-lane column partials and store them to dst[0..NP).
template <int NP, typename S>
__device__ __forceinline__ void warp_store_partials(const S (&acc)[NP], S* dst) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    const S v = warp_sum(acc[q]);
    if (lane == q) dst[q] = v;
  }
}

// Y = Mat * Xin on the 32 rows [ur0, ur1) of one unit (lane = row): the unit's
// contiguous slice of values and column indices is staged in the warp's part
// of shared memory with coalesced loads, then each lane gathers the NP-wide
// rows of Xin.  Slices longer than the staging space read the matrix directly.
// With DOT, dacc[q] += Wdot(row, q) * Y(row, q).
template <typename V, int NP, bool DOT>
__device__ __forceinline__ void unit_spmm(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                          const V* __restrict__ val, const V* __restrict__ Xin,
                                          V* __restrict__ Y, const V* __restrict__ Wdot, int ur0, int ur1,
                                          V* __restrict__ wval, int32_t* __restrict__ widx,
                                          ScalarOf<V> (&dacc)[NP]) {
  const int lane = threadIdx.x & 31;
  const int32_t k0 = ptr[ur0], k1 = ptr[ur1];
  const bool staged = (k1 - k0) <= kStageWarp;
  __syncwarp();  // the previous unit's slice is no longer read
  if (staged) {
    for (int32_t e = lane; e < k1 - k0; e += 32) {
      wval[e] = val[k0 + e];
      widx[e] = idx[k0 + e];
    }
  }
  __syncwarp();
  const int row = ur0 + lane;
  if (row < ur1) {
    const int32_t kb = ptr[row], ke = ptr[row + 1];
    V acc[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) acc[q] = V(0);
#pragma unroll 4
    for (int32_t k = kb; k < ke; ++k) {
      const V a = staged ? wval[k - k0] : val[k];
      const int32_t c = staged ? widx[k - k0] : idx[k];
      V xr[NP];
      load_row<V, NP>(Xin, c, xr);
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += a * xr[q];
    }
    store_row<V, NP>(Y, row, acc);
    if (DOT) {
      V w[NP];
      load_row<V, NP>(Wdot, row, w);
#pragma unroll
      for (int q = 0; q < NP; ++q) dacc[q] += w[q] * acc[q];
    }
  }
}

// Y = Mat * Xin on unit u (rows [ur0, ur1), lane = row) from the SELL copy.
template <typename V, int NP, bool DOT>
__device__ __forceinline__ void sell_unit_spmm(const SellMatrix<V>& M, const V* __restrict__ Xin,
                                               V* __restrict__ Y, const V* __restrict__ Wdot, int u, int ur0,
                                               int ur1, ScalarOf<V> (&dacc)[NP]) {
  const int lane = threadIdx.x & 31;
  const int32_t base = M.slice_ptr[u];
  const int w = (M.slice_ptr[u + 1] - base) >> 5;
  const int32_t* __restrict__ cp = M.col + base + lane;
  const V* __restrict__ vp = M.val + base + lane;
  V acc[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) acc[q] = V(0);
  if (w <= kSellShort) {
    // short slices (mesh rows: up to 7 entries): every value and column
    // index of the slice is requested at once, then every gather, so the
    // unit costs two dependent memory round trips
    V av[kSellShort];
    int32_t cv[kSellShort];
#pragma unroll
    for (int k = 0; k < kSellShort; ++k) {
      av[k] = (k < w) ? __ldg(vp + 32 * k) : V(0);
      cv[k] = (k < w) ? __ldg(cp + 32 * k) : 0;
    }
#pragma unroll
    for (int k = 0; k < kSellShort; ++k) {
      if (k < w) {
        V xr[NP];
        load_row<V, NP>(Xin, cv[k], xr);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] += av[k] * xr[q];
      }
    }
  } else {
#pragma unroll 4
    for (int k = 0; k < w; ++k) {
      const V a = __ldg(vp + 32 * k);
      const int32_t c = __ldg(cp + 32 * k);
      V xr[NP];
      load_row<V, NP>(Xin, c, xr);
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += a * xr[q];
    }
  }
  const int row = ur0 + lane;
  if (row < ur1) {
    store_row<V, NP>(Y, row, acc);
    if (DOT) {
      V wv[NP];
      load_row<V, NP>(Wdot, row, wv);
#pragma unroll
      for (int q = 0; q < NP; ++q) dacc[q] += wv[q] * acc[q];
    }
  }
}

// Asynchronous 16-byte global -> shared copies (completion tracked per
// thread in commit groups).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Y = Mat * Xin over the units [u0, u1) of one piece from the FP32 SELL copy,
// software-pipelined: while the warp gathers for unit u, the values and
// column indices of unit u + 1 are already being copied into the other of
// the warp's two shared-memory slots (cp.async), so a unit costs about one
// memory round trip (its gathers).  Slices wider than kSellShort are read
// directly.  `buf`: the warp's 2 * kSellShort * 32 values then as many column
// indices.  With DOT, dacc[q] += Wdot(row, q) * Y(row, q).
template <int NP, bool DOT>
__device__ __forceinline__ void sell_piece_spmm(const SellMatrix<float>& M, const float* __restrict__ Xin,
                                                float* __restrict__ Y, const float* __restrict__ Wdot,
                                                const int32_t* __restrict__ unit_row, int u0, int u1,
                                                float* __restrict__ buf, float (&dacc)[NP]) {
  constexpr int kSlot = kSellShort * 32;
  const int lane = threadIdx.x & 31;
  float* sval = buf;
  int32_t* scol = reinterpret_cast<int32_t*>(buf + 2 * kSlot);
  // issue the copies of unit u's slice into slot `slot` (nothing for wide slices)
  auto issue = [&](int32_t base, int w, int slot) {
    if (w <= kSellShort) {
      const int n16 = w * 8;  // 16-byte pieces per array (32 entries = 8 pieces per slice column)
      for (int c = lane; c < n16; c += 32) {
        cp_async16(sval + slot * kSlot + 4 * c, M.val + base + 4 * c);
        cp_async16(scol + slot * kSlot + 4 * c, M.col + base + 4 * c);
      }
    }
    cp_async_commit();
  };
  int32_t b0 = M.slice_ptr[u0], b1 = M.slice_ptr[u0 + 1];
  int32_t b2 = (u0 + 1 < u1) ? M.slice_ptr[u0 + 2] : b1;
  issue(b0, (b1 - b0) >> 5, 0);
  for (int u = u0; u < u1; ++u) {
    const int slot = (u - u0) & 1;
    const int w = (b1 - b0) >> 5;
    // next unit's slice into the other slot (every lane has finished reading
    // it: the __syncwarp at the end of the previous iteration)
    if (u + 1 < u1) issue(b1, (b2 - b1) >> 5, slot ^ 1);
    else cp_async_commit();
    const int32_t b3 = (u + 2 < u1) ? M.slice_ptr[u + 3] : b2;
    float acc[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) acc[q] = 0.f;
    if (w <= kSellShort) {
      cp_async_wait_prev();  // this unit's group (all but the newest) is complete
      __syncwarp();          // ... for every lane's copies
      const float* sv = sval + slot * kSlot + lane;
      const int32_t* sc = scol + slot * kSlot + lane;
#pragma unroll
      for (int k = 0; k < kSellShort; ++k) {
        if (k < w) {
          float xr[NP];
          load_row<float, NP>(Xin, sc[32 * k], xr);
          const float av = sv[32 * k];
#pragma unroll
          for (int q = 0; q < NP; ++q) acc[q] += av * xr[q];
        }
      }
    } else {
      const int32_t* __restrict__ cp = M.col + b0 + lane;
      const float* __restrict__ vp = M.val + b0 + lane;
#pragma unroll 4
      for (int k = 0; k < w; ++k) {
        const float a = __ldg(vp + 32 * k);
        const int32_t c = __ldg(cp + 32 * k);
        float xr[NP];
        load_row<float, NP>(Xin, c, xr);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] += a * xr[q];
      }
    }
    const int row = unit_row[u] + lane;
    if (row < unit_row[u + 1]) {
      store_row<float, NP>(Y, row, acc);
      if (DOT) {
        float wv[NP];
        load_row<float, NP>(Wdot, row, wv);
#pragma unroll
        for (int q = 0; q < NP; ++q) dacc[q] += wv[q] * acc[q];
      }
    }
    __syncwarp();  // the slot just read may be refilled next iteration
    b0 = b1;
    b1 = b2;
    b2 = b3;
  }
  cp_async_wait_prev();
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// Reduction slots.  After the warps of a CTA have stored the partial sums of
// their pieces (and after a __syncthreads), the CTA folds them into one slot
// per (segment, virtual CTA), one warp per segment, in piece order; consumers
// then sum a segment's slots, at most one per CTA that holds rows of it,
// instead of one per piece.
template <typename V, int NP, typename S>
__device__ __forceinline__ void fold_pieces(const PcgArgs<V>& a, const S* __restrict__ part,
                                            S* __restrict__ slots) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int vc = blockIdx.x; vc < a.nvc; vc += gridDim.x) {
    const int p0 = a.vc_piece[vc], p1 = a.vc_piece[vc + 1];
    if (p0 >= p1) continue;
    const int s0 = a.piece_seg[p0], s1 = a.piece_seg[p1 - 1];
    for (int s = s0 + warp; s <= s1; s += kWarps) {
      const int pa = max(a.seg_piece[s], p0), pb = min(a.seg_piece[s + 1], p1);
      if (pa >= pb) continue;
      S tot[NP];
      seg_totals<NP>(part, pa, pb, tot);
      S* dst = slots + (int64_t)(a.seg_slot[s] + vc - a.seg_vc0[s]) * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q)
        if (lane == q) dst[q] = tot[q];
    }
  }
}

// Visit the aggregates (coarse unknowns) this warp handles; s is the
// aggregate's segment.  Folding launches take those of the CTA's virtual
// CTAs (contiguous ranges of equal aggregate counts, every kWarps-th one
// starting at the warp's index), so that their partial sums fold into the
// CTA's slots; the others deal all aggregates round-robin over all warps.
#define FOR_MY_AGGS(a, ...)                                                                 \
  if ((a).fold) {                                                                          \
    for (int vc = blockIdx.x; vc < (a).pc.nvc; vc += gridDim.x) {                          \
      for (int g = (a).pc.vc_agg[vc] + (int)(threadIdx.x >> 5); g < (a).pc.vc_agg[vc + 1]; \
           g += kWarps) {                                                                  \
        const int s = (a).pc.agg_sid[g];                                                   \
        __VA_ARGS__                                                                        \
      }                                                                                    \
    }                                                                                      \
  } else {                                                                                 \
    for (int g = blockIdx.x * kWarps + (int)(threadIdx.x >> 5); g < (a).pc.nagg;           \
         g += gridDim.x * kWarps) {                                                        \
      const int s = (a).pc.agg_sid[g];                                                     \
      __VA_ARGS__                                                                          \
    }                                                                                      \
  }

// Column totals of segment s: from its reduction slots when the launch
// folds, else straight from the partial sums of its pieces (of its
// aggregates, for the coarse term).
template <typename V, int NP, typename S>
__device__ __forceinline__ void piece_totals(const PcgArgs<V>& a, const S* __restrict__ part,
                                             const S* __restrict__ slots, int s, S (&tot)[NP]) {
  if (a.fold) seg_totals<NP>(slots, a.seg_slot[s], a.seg_slot[s + 1], tot);
  else seg_totals<NP>(part, a.seg_piece[s], a.seg_piece[s + 1], tot);
}
template <typename V, int NP, typename S>
__device__ __forceinline__ void coarse_totals(const PcgArgs<V>& a, int s, S (&tot)[NP]) {
  if (a.fold) seg_totals<NP>(a.aslot, a.pc.seg_aslot[s], a.pc.seg_aslot[s + 1], tot);
  else seg_totals<NP>(a.csl, a.pc.seg_agg[s], a.pc.seg_agg[s + 1], tot);
}

// Fold the per-aggregate csl values of the CTA's virtual CTAs into one slot
// per (segment, virtual CTA), one warp per segment (after a __syncthreads).
template <typename V, int NP, typename S>
__device__ __forceinline__ void fold_aggs(const PcgArgs<V>& a, const S* __restrict__ csl,
                                          S* __restrict__ slots) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int vc = blockIdx.x; vc < a.pc.nvc; vc += gridDim.x) {
    const int g0 = a.pc.vc_agg[vc], g1 = a.pc.vc_agg[vc + 1];
    if (g0 >= g1) continue;
    const int s0 = a.pc.agg_sid[g0], s1 = a.pc.agg_sid[g1 - 1];
    for (int s = s0 + warp; s <= s1; s += kWarps) {
      const int ga = max(a.pc.seg_agg[s], g0), gb = min(a.pc.seg_agg[s + 1], g1);
      if (ga >= gb) continue;
      S tot[NP];
      seg_totals<NP>(csl, ga, gb, tot);
      S* dst = slots + (int64_t)(a.pc.seg_aslot[s] + vc - a.pc.seg_avc0[s]) * NP;
#pragma unroll
      for (int q = 0; q < NP; ++q)
        if (lane == q) dst[q] = tot[q];
    }
  }
}

// Two-level preconditioner, restriction: rc = W' R for the aggregates of
// segments with an active column (all == true: every aggregate), one warp
// per aggregate.
template <typename V, int NP>
__device__ __forceinline__ void coarse_restrict(const PcgArgs<V>& a, const int32_t* st, bool all) {
  using S = ScalarOf<V>;
  const int lane = threadIdx.x & 31;
  FOR_MY_AGGS(a, {
    if (!all) {
      bool act = false;
_Pragma("unroll")
      for (int q = 0; q < NP; ++q) act |= st[s * NP + q] == kActive;
      if (!act) continue;
    }
    S acc[NP];
_Pragma("unroll")
    for (int q = 0; q < NP; ++q) acc[q] = S(0);
    for (int32_t m = a.pc.agg_ptr[g] + lane; m < a.pc.agg_ptr[g + 1]; m += 32) {
      V r[NP];
      load_row<V, NP>(a.R, a.pc.agg_contig ? m : a.pc.agg_row[m], r);
_Pragma("unroll")
      for (int q = 0; q < NP; ++q) acc[q] += (S)r[q];
    }
_Pragma("unroll")
    for (int q = 0; q < NP; ++q) {
      const S v = warp_sum(acc[q]);
      if (lane == q) a.rc[(int64_t)g * NP + q] = v;
    }
  })
}

// Restriction fused into the update phase (aggregates are contiguous row
// ranges): piece p has summed its rows of aggregate g into acc (per lane).
// An aggregate inside the piece's rows is written to rc directly.  One that
// straddles pieces pa..pb leaves one partial per piece: the piece it starts in
// writes its tail slot (2 pa + 1), every later piece its head slot (2 p); the
// last of them to arrive (a counter per aggregate) sums the partials in piece
// order, so the result does not depend on the arrival order, writes rc and
// clears the counter.  head / tail: g is the piece's first aggregate and
// began in an earlier piece / its last one and goes on in a later piece.
// Called by the whole warp.
template <typename V, int NP, typename S>
__device__ __forceinline__ void restrict_flush(const PcgArgs<V>& a, int p, int g, bool head, bool tail,
                                               const S (&acc)[NP]) {
  const int lane = threadIdx.x & 31;
  S tot[NP];
#pragma unroll
  for (int q = 0; q < NP; ++q) tot[q] = warp_sum(acc[q]);
  if (!head && !tail) {
#pragma unroll
    for (int q = 0; q < NP; ++q)
      if (lane == q) a.rc[(int64_t)g * NP + q] = tot[q];
    return;
  }
  const int slot = 2 * p + (head ? 0 : 1);
#pragma unroll
  for (int q = 0; q < NP; ++q)
    if (lane == q) a.rc_part[(int64_t)slot * NP + q] = tot[q];
  __threadfence();
  __syncwarp();
  int pa = p, pb = p, last = 0;
  if (lane == 0) {
    const int ga = a.pc.agg_ptr[g], gb = a.pc.agg_ptr[g + 1];
    while (a.unit_row[a.piece_unit[pa]] > ga) --pa;
    while (a.unit_row[a.piece_unit[pb + 1]] < gb) ++pb;
    last = atomicAdd(a.rc_cnt + g, 1) == pb - pa;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  pa = __shfl_sync(0xffffffffu, pa, 0);
  pb = __shfl_sync(0xffffffffu, pb, 0);
  __threadfence();
  if (lane < NP) {
    S sum = S(0);
    for (int pp = pa; pp <= pb; ++pp) sum += __ldcg(a.rc_part + (int64_t)(2 * pp + (pp == pa ? 1 : 0)) * NP + lane);
    a.rc[(int64_t)g * NP + lane] = sum;
  }
  if (lane == 0) a.rc_cnt[g] = 0;
}

// BF16 element e (0..3) of four packed in a uint2 (element 0 in the low half
// of .x): a BF16 value is the upper 16 bits of the FP32 with the same value.
__device__ __forceinline__ float bf16x4_elem(const uint2& w, int e) {
  const unsigned word = (e < 2) ? w.x : w.y;
  return __uint_as_float((e & 1) ? (word & 0xffff0000u) : (word << 16));
}

// Rows of the coarse product for one warp: acc[r][q] += sum_j R[r][j] x[j][q]
// over j < jend (a multiple of 4), for the nr <= RW rows starting at kr (row
// stride ld, a multiple of 8).  Lane l streams entries 4l .. 4l+3 of every
// 128, one 8-byte load per row, the next group's loads issued before the
// current group is used (two groups of RW loads in flight per lane; a third
// measured no faster and spilled more); each x
// value read serves RW rows.  SWZ: x is the staged copy in shared memory,
// entry j at (j % 4) * (ld / 4) + j / 4, so that the 32 lanes read 32
// consecutive entries (no bank conflicts); otherwise x is rc in global
// memory, entry j at j.
template <int NP, int RW, bool SWZ>
__device__ __forceinline__ void coarse_rows(const uint16_t* __restrict__ kr, int ld, int jend, int nr,
                                            const float* x, float (&acc)[RW][NP]) {
  const int lane = threadIdx.x & 31;
  const int l4 = ld >> 2;
  const uint2* __restrict__ kq = reinterpret_cast<const uint2*>(kr);  // 4 entries per uint2
  uint2 w[RW];
#pragma unroll
  for (int r = 0; r < RW; ++r)
    w[r] = (r < nr && 4 * lane < jend) ? __ldg(kq + r * l4 + lane) : make_uint2(0u, 0u);
  for (int j4 = lane; 4 * j4 < jend; j4 += 32) {
    const int jn = j4 + 32;
    uint2 wn[RW];
#pragma unroll
    for (int r = 0; r < RW; ++r) wn[r] = (r < nr && 4 * jn < jend) ? __ldg(kq + r * l4 + jn) : make_uint2(0u, 0u);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      float xv[NP];
      load_row<float, NP>(x, SWZ ? e * l4 + j4 : 4 * j4 + e, xv);
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const float kv = bf16x4_elem(w[r], e);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[r][q] = fmaf(kv, xv[q], acc[r][q]);
      }
    }
#pragma unroll
    for (int r = 0; r < RW; ++r) w[r] = wn[r];
  }
}

// Two-level preconditioner, coarse solve: yc = (W'KW)^-1 rc per segment and
// csl = rc .* yc, with (W'KW)^-1 = c v v' + R (R in BF16).  CTA-wide tasks
// of up to kCoarseTaskRows coarse rows of one segment: the CTA stages the
// segment's rc (zero-padded to ld) and v'rc in shared memory when they fit
// (`stage`, shared with the SpMM staging buffer), then every warp computes
// RW rows at a time; otherwise each warp reads rc from global memory (only
// below nc) and forms v'rc itself.
template <typename V, int NP>
__device__ __forceinline__ void coarse_solve(const PcgArgs<V>& a, const int32_t* st, bool all, float* stage,
                                             int stage_floats, unsigned long long& cbytes, unsigned* ctr) {
  static_assert(sizeof(V) == 4, "the two-level preconditioner runs FP32 iterations");
  // rows per warp pass (each staged residual value read from shared memory
  // serves that many rows; bounded by the 48-register budget)
  constexpr int RW = (NP <= 4) ? kCoarseRowsPerPass : 1;
  static_assert(kWarps == kWarpsPerCta, "coarse task plan and kernel disagree on the CTA size");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ float s_vrc[NP];
  __shared__ float s_red[kWarps][NP];
  __shared__ int s_grab;
  int staged = -1;
  // task ranges: groups taken from the counter (every CTA until the list is
  // exhausted), or the CTA's virtual CTAs' static ranges when the launch
  // folds partial sums per virtual CTA
  const bool dyn = !a.fold && a.pc.ngroup > 0;
  int vc = blockIdx.x;
  for (;;) {
    int t0, t1;
    if (dyn) {
      if (threadIdx.x == 0) s_grab = (int)atomicAdd(ctr, 1u);
      __syncthreads();
      const int gi = s_grab;
      __syncthreads();  // every thread has read s_grab before it changes
      if (gi >= a.pc.ngroup) break;
      t0 = a.pc.grp_t0[gi];
      t1 = a.pc.grp_t1[gi];
    } else {
      if (vc >= a.pc.nvc) break;
      t0 = a.pc.vc_task[vc];
      t1 = a.pc.vc_task[vc + 1];
      vc += gridDim.x;
    }
    for (int t = t0; t < t1; ++t) {
      const int s = a.pc.task_seg[t];
      if (!all) {
        bool act = false;
#pragma unroll
        for (int q = 0; q < NP; ++q) act |= st[s * NP + q] == kActive;
        if (!act) continue;  // the same decision in every thread of the CTA
      }
      const int base = a.pc.seg_agg[s];
      const int nc = a.pc.seg_agg[s + 1] - base;
      const int ld = (nc + 7) & ~7;
      const float* __restrict__ rcs = a.rc + (int64_t)base * NP;
      const float* __restrict__ vs = a.pc.kvec + base;
      const bool use_stage = ld * NP <= stage_floats;
      float vrc[NP];
      if (use_stage) {
        if (s != staged) {
          __syncthreads();  // every warp is done with the previous segment
          float part[NP];
#pragma unroll
          for (int q = 0; q < NP; ++q) part[q] = 0.f;
          const int l4 = ld >> 2;
          for (int j = threadIdx.x; j < ld; j += blockDim.x) {
            float xv[NP];
            if (j < nc) {
              load_row<float, NP>(rcs, j, xv);
              const float vj = vs[j];
#pragma unroll
              for (int q = 0; q < NP; ++q) part[q] = fmaf(vj, xv[q], part[q]);
            } else {
#pragma unroll
              for (int q = 0; q < NP; ++q) xv[q] = 0.f;
            }
            store_row<float, NP>(stage, (j & 3) * l4 + (j >> 2), xv);
          }
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const float w = warp_sum(part[q]);
            if (lane == 0) s_red[warp][q] = w;
          }
          __syncthreads();
          if (threadIdx.x < NP) {
            float tot = 0.f;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) tot += s_red[w][threadIdx.x];
            s_vrc[threadIdx.x] = tot;
          }
          __syncthreads();
          staged = s;
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) vrc[q] = s_vrc[q];
      } else {
        float part[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) part[q] = 0.f;
        for (int j = lane; j < nc; j += 32) {
          float xv[NP];
          load_row<float, NP>(rcs, j, xv);
          const float vj = vs[j];
#pragma unroll
          for (int q = 0; q < NP; ++q) part[q] = fmaf(vj, xv[q], part[q]);
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) vrc[q] = warp_sum(part[q]);
      }
      const int g0 = a.pc.task_g0[t], g1 = a.pc.task_g1[t];
      const float c = a.pc.kscale[s];
      if (threadIdx.x == 0) cbytes += 2ull * (unsigned long long)(g1 - g0) * (unsigned long long)ld;
      const uint16_t* kseg = a.pc.kinv + a.pc.kinv_off[s];
      for (int r0 = g0 + warp * RW; r0 < g1; r0 += kWarps * RW) {
        const int nr = min(RW, g1 - r0);
        const uint16_t* kr = kseg + (int64_t)(r0 - base) * ld;
        // the epilogue's operands of the lane that writes (row r0 + lane / NP,
        // column lane % NP), loaded before the row stream so that their round
        // trip overlaps it
        const int my_r = lane / NP;
        const bool my_ok = lane < RW * NP && my_r < nr;
        const float my_rc = my_ok ? a.rc[(int64_t)(r0 + my_r) * NP + lane % NP] : 0.f;
        const float my_cv = my_ok ? c * vs[r0 + my_r - base] : 0.f;
        float acc[RW][NP];
#pragma unroll
        for (int r = 0; r < RW; ++r)
#pragma unroll
          for (int q = 0; q < NP; ++q) acc[r][q] = 0.f;
        if (use_stage) {
          coarse_rows<NP, RW, true>(kr, ld, ld, nr, stage, acc);
        } else {
          // rc is read only below nc (what follows may be another segment's)
          const int body = nc & ~3;
          coarse_rows<NP, RW, false>(kr, ld, body, nr, rcs, acc);
          for (int j = body + lane; j < nc; j += 32) {
            float xv[NP];
            load_row<float, NP>(rcs, j, xv);
#pragma unroll
            for (int r = 0; r < RW; ++r) {
              const float kv = (r < nr) ? __uint_as_float((unsigned)kr[r * ld + j] << 16) : 0.f;
#pragma unroll
              for (int q = 0; q < NP; ++q) acc[r][q] = fmaf(kv, xv[q], acc[r][q]);
            }
          }
        }
#pragma unroll
        for (int r = 0; r < RW; ++r) {
          const int g = r0 + r;
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            const float sum = warp_sum(acc[r][q]);
            if (r < nr && lane == r * NP + q) {
              const float y = sum + my_cv * vrc[q];
              a.yc[(int64_t)g * NP + q] = y;
              a.csl[(int64_t)g * NP + q] = y * my_rc;
            }
          }
        }
      }
    }
  }
  if (a.fold) {
    __syncthreads();
    fold_aggs<V, NP>(a, a.csl, a.aslot);
  }
}

// z = dinv .* r (+ the coarse correction W yc for the two-level preconditioner)
template <typename V, int NP, int PC>
__device__ __forceinline__ void apply_diag_coarse(const PcgArgs<V>& a, int row, const V (&r)[NP], V (&z)[NP]) {
  const V d = a.pc.dinv[row];
#pragma unroll
  for (int q = 0; q < NP; ++q) z[q] = d * r[q];
  if constexpr (PC == kPrecTwoLevel) {
    const int g = a.pc.agg[row];
    if (g >= 0) {
#pragma unroll
      for (int q = 0; q < NP; ++q) z[q] += (V)a.yc[(int64_t)g * NP + q];
    }
  }
}

// Row `row` of Mat * Xin for the calling lane (unit u, lane = row): from the
// SELL copy when present, else the CSR arrays.  No warp synchronisation: lanes
// of rows past the unit's end may call it and ignore the result.
template <typename V, int NP>
__device__ __forceinline__ void row_apply(const SellMatrix<V>& sm, const int32_t* __restrict__ ptr,
                                          const int32_t* __restrict__ idx, const V* __restrict__ val,
                                          const V* __restrict__ Xin, int u, int row, bool valid, V (&acc)[NP]) {
#pragma unroll
  for (int q = 0; q < NP; ++q) acc[q] = V(0);
  if (sm.val) {
    const int lane = threadIdx.x & 31;
    const int32_t base = sm.slice_ptr[u];
    const int w = (sm.slice_ptr[u + 1] - base) >> 5;
#pragma unroll 4
    for (int k = 0; k < w; ++k) {
      const V a = __ldg(sm.val + base + 32 * k + lane);
      V xr[NP];
      load_row<V, NP>(Xin, __ldg(sm.col + base + 32 * k + lane), xr);
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += a * xr[q];
    }
  } else if (valid) {
    for (int32_t k = ptr[row]; k < ptr[row + 1]; ++k) {
      const V a = val[k];
      V xr[NP];
      load_row<V, NP>(Xin, idx[k], xr);
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += a * xr[q];
    }
  }
}

// T = G R on the piece's rows; returns the partial ||T||^2 (= r' G'G r) per column.
template <typename V, int NP>
__device__ __forceinline__ void factor_first_half(const PcgArgs<V>& a, int u0, int u1, ScalarOf<V> (&acc)[NP]) {
  const int lane = threadIdx.x & 31;
  for (int u = u0; u < u1; ++u) {
    const int row = a.unit_row[u] + lane;
    const bool valid = row < a.unit_row[u + 1];
    V t[NP];
    row_apply<V, NP>(a.pc.g_sell, a.pc.g_ptr, a.pc.g_idx, a.pc.g_val, a.R, u, row, valid, t);
    if (valid) {
      store_row<V, NP>(a.T, row, t);
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += t[q] * t[q];
    }
  }
}

// IC(0) preconditioner: T = L^-1 R level by level (one thread per row, a
// grid barrier after each level), then Z = L^-T T over the backward levels.
// Every row is solved (rows of converged segments too: their R is frozen).
template <typename V, int NP>
__device__ __forceinline__ bool ic0_apply_grid(const PcgArgs<V>& a) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int l = 0; l < a.pc.ic_nlev_f; ++l) {
    for (int32_t t = a.pc.ic_lev_f_ptr[l] + tid; t < a.pc.ic_lev_f_ptr[l + 1]; t += nth) {
      const int32_t i = a.pc.ic_lev_f_row[t];
      const int32_t kd = a.pc.ic_diag[i];
      V acc[NP];
      load_row<V, NP>(a.R, i, acc);
      for (int32_t k = a.indptr[i]; k < kd; ++k) {
        const V lv = a.pc.ic_val[k];
        V y[NP];
        load_row<V, NP>(a.T, a.indices[k], y);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] -= lv * y[q];
      }
      const V d = a.pc.dinv[i];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] *= d;
      store_row<V, NP>(a.T, i, acc);
    }
    if (!grid_sync(a.bar)) return false;
  }
  for (int l = 0; l < a.pc.ic_nlev_b; ++l) {
    for (int32_t t = a.pc.ic_lev_b_ptr[l] + tid; t < a.pc.ic_lev_b_ptr[l + 1]; t += nth) {
      const int32_t i = a.pc.ic_lev_b_row[t];
      const int32_t kd = a.pc.ic_diag[i];
      V acc[NP];
      load_row<V, NP>(a.T, i, acc);
      for (int32_t k = kd + 1; k < a.indptr[i + 1]; ++k) {
        const V lv = a.pc.ic_val[k];
        V z[NP];
        load_row<V, NP>(a.Z, a.indices[k], z);
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] -= lv * z[q];
      }
      const V d = a.pc.dinv[i];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] *= d;
      store_row<V, NP>(a.Z, i, acc);
    }
    if (!grid_sync(a.bar)) return false;
  }
  return true;
}

// Partial r'z of a piece's rows (z = Z, the preconditioned residual).
template <typename V, int NP>
__device__ __forceinline__ void piece_rz(const PcgArgs<V>& a, int u0, int u1, ScalarOf<V> (&acc)[NP]) {
  const int lane = threadIdx.x & 31;
  for (int u = u0; u < u1; ++u) {
    const int row = a.unit_row[u] + lane;
    if (row < a.unit_row[u + 1]) {
      V r[NP], z[NP];
      load_row<V, NP>(a.R, row, r);
      load_row<V, NP>(a.Z, row, z);
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] += r[q] * z[q];
    }
  }
}

// Loop over this warp's pieces: s = segment, [u0, u1) = units of the piece.
#define FOR_MY_PIECES(a, ...)                                                               \
  for (int vw = gw; vw < (a).nvw; vw += nw) {                                                \
    for (int p = (a).vw_piece[vw]; p < (a).vw_piece[vw + 1]; ++p) {                          \
      const int s = (a).piece_seg[p];                                                        \
      const int u0 = (a).piece_unit[p], u1 = (a).piece_unit[p + 1];                          \
      (void)s; (void)u0; (void)u1;                                                           \
      __VA_ARGS__                                                                            \
    }                                                                                        \
  }

template <typename V, int NP, int PC, bool RU>
__global__ void __launch_bounds__(kPcgThreads, kPlanCtasPerSm) pcg_kernel(PcgArgs<V> a) {
  using S = ScalarOf<V>;
  // one buffer: the SpMM's staged slices (values, then column indices) or,
  // in the coarse phase, a segment's restricted residual
  constexpr int kStageBytes =
      kWarps * (kStageWarp * (int)(sizeof(V) + sizeof(int32_t)) > 2 * kSellShort * 32 * 8
                    ? kStageWarp * (int)(sizeof(V) + sizeof(int32_t))
                    : 2 * kSellShort * 32 * 8);
  __shared__ __align__(16) unsigned char stage_raw[kStageBytes];
  V* sval_all = reinterpret_cast<V*>(stage_raw);
  int32_t* sidx_all = reinterpret_cast<int32_t*>(stage_raw + kWarps * kStageWarp * sizeof(V));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gw = blockIdx.x * kWarps + warp, nw = gridDim.x * kWarps;
  V* wval = sval_all + warp * kStageWarp;
  int32_t* widx = sidx_all + warp * kStageWarp;
  // the warp's two SELL slots (FP32 iterations)
  float* wslots = reinterpret_cast<float*>(stage_raw) + warp * (2 * kSellShort * 32 * 2);
  S* part_pq = a.part;
  S* part_rz = a.part + (int64_t)a.npiece * NP;
  S* part_rr = a.part + 2 * (int64_t)a.npiece * NP;
  S* slot_pq = a.slot;
  S* slot_rz = a.slot + (int64_t)a.nslot * NP;
  S* slot_rr = a.slot + 2 * (int64_t)a.nslot * NP;
  constexpr bool kDiagPC = PC == kPrecJacobi || PC == kPrecTwoLevel;  // z = dinv .* r (+ coarse term)
  // CTA flag "a column of one of my segments is still active", summed over
  // the grid by the barriers that close the initialisation and phase C
  __shared__ int s_act;
  __shared__ unsigned s_seen;
  if (threadIdx.x == 0) s_act = 0;
  // rows and nonzeros this warp streamed through the SpMM phase; coarse
  // inverse bytes this CTA streamed (thread 0)
  unsigned long long w_rows = 0, w_nnz = 0, c_bytes = 0;
  // profile mode: thread 0 of CTA 0 adds the device time between consecutive
  // barrier exits to the phase that just ended (a barrier exit marks the
  // moment the slowest CTA finished the phase)
  const bool timer = a.phase_ns != nullptr && blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long t_mark = timer ? globaltimer_ns() : 0ull;
  auto mark = [&](int ph) {
    if (timer) {
      const unsigned long long now = globaltimer_ns();
      a.phase_ns[ph] += now - t_mark;
      t_mark = now;
    }
  };

  // ---- phase 0: X = 0, R = B, P = M^-1 R (Jacobi); partial b'b and r'z
  FOR_MY_PIECES(a, {
    S bb[NP], rz[NP];
#pragma unroll
    for (int q = 0; q < NP; ++q) { bb[q] = S(0); rz[q] = S(0); }
    for (int u = u0; u < u1; ++u) {
      const int row = a.unit_row[u] + lane;
      if (row < a.unit_row[u + 1]) {
        V b[NP], z[NP], zero[NP];
        if constexpr (RU) {
          double b64[NP], z64[NP];
          load_row<double, NP>(a.B64, row, b64);
#pragma unroll
          for (int q = 0; q < NP; ++q) { b[q] = (V)b64[q]; z64[q] = 0.0; }
          store_row<double, NP>(a.X64, row, z64);
        } else {
          load_row<V, NP>(a.B, row, b);
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) zero[q] = V(0);
        store_row<V, NP>(a.X, row, zero);
        store_row<V, NP>(a.R, row, b);
        if (kDiagPC) {
          const V d = a.pc.dinv[row];
#pragma unroll
          for (int q = 0; q < NP; ++q) { z[q] = d * b[q]; rz[q] += b[q] * z[q]; }
          if (PC == kPrecJacobi) store_row<V, NP>(a.P, row, z);
        }
#pragma unroll
        for (int q = 0; q < NP; ++q) bb[q] += b[q] * b[q];
      }
    }
    warp_store_partials<NP>(bb, part_rr + (int64_t)p * NP);
    if (kDiagPC) warp_store_partials<NP>(rz, part_rz + (int64_t)p * NP);
  })
  if (a.fold) {
    __syncthreads();
    fold_pieces<V, NP>(a, part_rr, slot_rr);
    if (kDiagPC) fold_pieces<V, NP>(a, part_rz, slot_rz);
  }
  if constexpr (PC == kPrecTwoLevel) {
    if (!grid_sync(a.bar)) return;
    coarse_restrict<V, NP>(a, nullptr, true);
    if (!grid_sync(a.bar)) return;
    coarse_solve<V, NP>(a, nullptr, true, reinterpret_cast<float*>(stage_raw), kStageBytes / 4, c_bytes, a.cq);
  }
  if constexpr (PC == kPrecIC0) {  // Z = (L L')^-1 R, r'z; P = Z below
    if (!grid_sync(a.bar)) return;
    if (!ic0_apply_grid<V, NP>(a)) return;
    FOR_MY_PIECES(a, {
      S acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = S(0);
      piece_rz<V, NP>(a, u0, u1, acc);
      warp_store_partials<NP>(acc, part_rz + (int64_t)p * NP);
    })
    if (a.fold) {
      __syncthreads();
      fold_pieces<V, NP>(a, part_rz, slot_rz);
    }
  }
  if constexpr (PC == kPrecFactored) {  // r'z = ||G r||^2; P = G'(G r) below
    if (!grid_sync(a.bar)) return;
    FOR_MY_PIECES(a, {
      S acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = S(0);
      factor_first_half<V, NP>(a, u0, u1, acc);
      warp_store_partials<NP>(acc, part_rz + (int64_t)p * NP);
    })
    if (a.fold) {
      __syncthreads();
      fold_pieces<V, NP>(a, part_rz, slot_rz);
    }
  }
  if (!grid_sync(a.bar)) return;
  // the first iteration's coarse phase takes groups from counter 1
  if (PC == kPrecTwoLevel && blockIdx.x == 0 && threadIdx.x == 0) a.cq[1] = 0u;
  // ---- segment initialisation (the warp holding a segment's first piece publishes)
  FOR_MY_PIECES(a, {
    if constexpr (PC == kPrecFactored) {
      for (int u = u0; u < u1; ++u) {
        const int row = a.unit_row[u] + lane;
        const bool valid = row < a.unit_row[u + 1];
        V z[NP];
        row_apply<V, NP>(a.pc.gt_sell, a.pc.gt_ptr, a.pc.gt_idx, a.pc.gt_val, a.T, u, row, valid, z);
        if (valid) store_row<V, NP>(a.P, row, z);
      }
    }
    if constexpr (PC == kPrecIC0) {
      for (int u = u0; u < u1; ++u) {
        const int row = a.unit_row[u] + lane;
        if (row < a.unit_row[u + 1]) {
          V z[NP];
          load_row<V, NP>(a.Z, row, z);
          store_row<V, NP>(a.P, row, z);
        }
      }
    }
    if constexpr (PC == kPrecTwoLevel) {
      for (int u = u0; u < u1; ++u) {
        const int row = a.unit_row[u] + lane;
        if (row < a.unit_row[u + 1]) {
          V r[NP], z[NP];
          load_row<V, NP>(a.R, row, r);
          apply_diag_coarse<V, NP, PC>(a, row, r, z);
          store_row<V, NP>(a.P, row, z);
        }
      }
    }
    if (a.seg_piece[s] == p) {
      S bb[NP], rz[NP];
      piece_totals<V, NP>(a, part_rr, slot_rr, s, bb);
      piece_totals<V, NP>(a, part_rz, slot_rz, s, rz);
      if constexpr (PC == kPrecTwoLevel) {
        S c[NP];
        coarse_totals<V, NP>(a, s, c);
#pragma unroll
        for (int q = 0; q < NP; ++q) rz[q] += c[q];
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        if (lane == q) {
          int32_t st;
          if (!isfinite(bb[q]) || !isfinite(rz[q])) st = LAPY_ERR_NAN;
          else if (bb[q] == S(0)) st = 0;
          else if (!(rz[q] > S(0))) st = LAPY_ERR_BREAKDOWN;
          else st = kActive;
          a.bb[s * NP + q] = bb[q];
          a.rz[s * NP + q] = rz[q];
          if (RU) a.rref[s * NP + q] = bb[q];
          a.state[s * NP + q] = st;
          if (st == kActive) s_act = 1;
        }
      }
    }
  })
  if (!grid_sync(a.bar, &s_act, &s_seen)) return;
  mark(0);
  unsigned seen_prev = s_seen, nact = s_seen;

  int it = 0;
  for (;; ++it) {
    const int par = it & 1;
    const int32_t* st_cur = a.state + par * (int64_t)a.nseg * NP;
    int32_t* st_nxt = a.state + (par ^ 1) * (int64_t)a.nseg * NP;
    const S* rz_cur = a.rz + par * (int64_t)a.nseg * NP;
    S* rz_nxt = a.rz + (par ^ 1) * (int64_t)a.nseg * NP;
    if (nact == 0 || it >= a.maxiter) break;

    // ---- reliable update of the columns flagged in the previous phase C:
    // X64 += X (FP32 correction), X = 0; then R = b - K64 X64 in FP64
    bool ru_now = false;
    const int32_t* ru_req = nullptr;
    if constexpr (RU) {
      ru_req = a.ru_col + par * (int64_t)a.nseg * NP;
      ru_now = *((volatile unsigned*)&a.ru_flag[par]) != 0u;
      if (ru_now) {
        FOR_MY_PIECES(a, {
          bool fl[NP];
          bool anyf = false;
#pragma unroll
          for (int q = 0; q < NP; ++q) { fl[q] = ru_req[s * NP + q] != 0; anyf |= fl[q]; }
          if (anyf) {
            for (int u = u0; u < u1; ++u) {
              const int row = a.unit_row[u] + lane;
              if (row < a.unit_row[u + 1]) {
                V x[NP];
                double x64[NP];
                load_row<V, NP>(a.X, row, x);
                load_row<double, NP>(a.X64, row, x64);
#pragma unroll
                for (int q = 0; q < NP; ++q)
                  if (fl[q]) { x64[q] += (double)x[q]; x[q] = V(0); }
                store_row<double, NP>(a.X64, row, x64);
                store_row<V, NP>(a.X, row, x);
              }
            }
          }
        })
        if (!grid_sync(a.bar)) return;
        FOR_MY_PIECES(a, {
          bool fl[NP];
          bool anyf = false;
#pragma unroll
          for (int q = 0; q < NP; ++q) { fl[q] = ru_req[s * NP + q] != 0; anyf |= fl[q]; }
          double rr[NP];
          S rz[NP];
#pragma unroll
          for (int q = 0; q < NP; ++q) { rr[q] = 0.0; rz[q] = S(0); }
          if (anyf) {
            for (int u = u0; u < u1; ++u) {
              const int row = a.unit_row[u] + lane;
              if (row < a.unit_row[u + 1]) {
                double acc[NP], b64[NP];
#pragma unroll
                for (int q = 0; q < NP; ++q) acc[q] = 0.0;
                const int32_t kb = a.indptr[row], ke = a.indptr[row + 1];
                for (int32_t k = kb; k < ke; ++k) {
                  const double v = __ldg(a.K64 + k);
                  double xr[NP];
                  load_row<double, NP>(a.X64, __ldg(a.indices + k), xr);
#pragma unroll
                  for (int q = 0; q < NP; ++q) acc[q] = fma(v, xr[q], acc[q]);
                }
                load_row<double, NP>(a.B64, row, b64);
                V r[NP];
                load_row<V, NP>(a.R, row, r);
                const V d = a.pc.dinv[row];
#pragma unroll
                for (int q = 0; q < NP; ++q) {
                  if (fl[q]) {
                    const double r64 = b64[q] - acc[q];
                    rr[q] += r64 * r64;
                    r[q] = (V)r64;
                    rz[q] += r[q] * (d * r[q]);
                  }
                }
                store_row<V, NP>(a.R, row, r);
              }
            }
          }
          warp_store_partials<NP>(rr, a.part64 + (int64_t)p * NP);
          warp_store_partials<NP>(rz, part_rz + (int64_t)p * NP);
        })
        if (a.fold) {
          __syncthreads();
          fold_pieces<V, NP>(a, a.part64, a.slot64);
          fold_pieces<V, NP>(a, part_rz, slot_rz);
        }
        if (!grid_sync(a.bar)) return;
        mark(2);
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.n_updates, 1u);
      }
    }

    // ---- phase A: Q = K P, partial p'q
    if (RU && blockIdx.x == 0 && threadIdx.x == 0) a.ru_flag[par ^ 1] = 0u;
    FOR_MY_PIECES(a, {
      bool colact[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) colact[q] = st_cur[s * NP + q] == kActive;
      if constexpr (RU) {
        const bool first = a.seg_piece[s] == p;
        if (first && lane < NP) a.ru_col[(par ^ 1) * (int64_t)a.nseg * NP + s * NP + lane] = 0;
        bool fl[NP];
        bool anyf = false;
#pragma unroll
        for (int q = 0; q < NP; ++q) { fl[q] = ru_now && ru_req[s * NP + q] != 0; anyf |= fl[q]; }
        if (anyf) {
          // the true residual decides convergence; otherwise CG continues with
          // the same direction P and the new r'z
          double rr64[NP];
          S rzt[NP];
          piece_totals<V, NP>(a, a.part64, a.slot64, s, rr64);
          piece_totals<V, NP>(a, part_rz, slot_rz, s, rzt);
#pragma unroll
          for (int q = 0; q < NP; ++q) {
            if (!(fl[q] && colact[q])) continue;
            int32_t st = kActive;
            if (!isfinite(rr64[q]) || !isfinite(rzt[q])) st = LAPY_ERR_NAN;
            else if (rr64[q] <= a.rtol2_64 * (double)a.bb[s * NP + q]) st = it > 0 ? it : 1;
            else if (!(rzt[q] > S(0))) st = LAPY_ERR_BREAKDOWN;
            colact[q] = st == kActive;
            if (first && lane == q) {
              const_cast<int32_t*>(st_cur)[s * NP + q] = st;
              if (st == kActive) {
                const_cast<S*>(rz_cur)[s * NP + q] = rzt[q];
                a.rref[s * NP + q] = (S)rr64[q];
              }
            }
          }
        }
      }
      bool mine = false;
#pragma unroll
      for (int q = 0; q < NP; ++q) mine |= (lane == q) && colact[q];
      const bool any = __any_sync(0xffffffffu, mine);
      S acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = S(0);
      if (any) {
        if (a.use_sell) {
          if constexpr (sizeof(V) == 4) {
            sell_piece_spmm<NP, true>(a.sell, a.P, a.Q, a.P, a.unit_row, u0, u1, wslots, acc);
          } else {
            for (int u = u0; u < u1; ++u)
              sell_unit_spmm<V, NP, true>(a.sell, a.P, a.Q, a.P, u, a.unit_row[u], a.unit_row[u + 1], acc);
          }
        } else {
          for (int u = u0; u < u1; ++u)
            unit_spmm<V, NP, true>(a.indptr, a.indices, a.vals, a.P, a.Q, a.P, a.unit_row[u], a.unit_row[u + 1],
                                   wval, widx, acc);
        }
        if (lane == 0) {
          const int r0 = a.unit_row[u0], r1 = a.unit_row[u1];
          w_rows += (unsigned long long)(r1 - r0);
          w_nnz += (unsigned long long)(a.indptr[r1] - a.indptr[r0]);
        }
      }
      warp_store_partials<NP>(acc, part_pq + (int64_t)p * NP);
    })
    if (a.fold) {
      __syncthreads();
      fold_pieces<V, NP>(a, part_pq, slot_pq);
    }
    if (!grid_sync(a.bar)) return;
    mark(1);

    // ---- phase B: alpha, X += alpha P, R -= alpha Q, partial r'r (and r'z for Jacobi)
    FOR_MY_PIECES(a, {
      S pq[NP];
      piece_totals<V, NP>(a, part_pq, slot_pq, s, pq);
      V alpha[NP];
      bool act[NP];
      bool any = false;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        act[q] = st_cur[s * NP + q] == kActive && pq[q] > S(0) && isfinite(pq[q]);
        alpha[q] = act[q] ? (V)(rz_cur[s * NP + q] / pq[q]) : V(0);
        any |= act[q];
      }
      S rr[NP], rz[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) { rr[q] = S(0); rz[q] = S(0); }
      // fused restriction: every piece of a segment with an active column
      // sums its rows of each aggregate (the same decision in all of them)
      bool rseg = false;
      if constexpr (PC == kPrecTwoLevel) {
        if (a.pc.agg_contig) {
#pragma unroll
          for (int q = 0; q < NP; ++q) rseg |= st_cur[s * NP + q] == kActive;
        }
      }
      if (any || rseg) {
        int cg = -1;  // aggregate being summed (warp-uniform)
        S cacc[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) cacc[q] = S(0);
        // the piece's first and last aggregates, and whether they go on
        // beyond the piece (rows of other segments carry other labels)
        int gF = -1, gL = -1;
        bool hs = false, ts = false;
        if constexpr (PC == kPrecTwoLevel) {
          if (rseg) {
            const int r0 = a.unit_row[u0], r1 = a.unit_row[u1];
            gF = a.pc.agg[r0];
            gL = a.pc.agg[r1 - 1];
            hs = r0 > 0 && a.pc.agg[r0 - 1] == gF;
            ts = r1 < a.n && a.pc.agg[r1] == gL;
          }
        }
        for (int u = u0; u < u1; ++u) {
          const int row = a.unit_row[u] + lane;
          const bool valid = row < a.unit_row[u + 1];
          V r[NP];
          if (valid) {
            V x[NP], pv[NP], qv[NP];
            load_row<V, NP>(a.X, row, x);
            load_row<V, NP>(a.P, row, pv);
            load_row<V, NP>(a.Q, row, qv);
            load_row<V, NP>(a.R, row, r);
            const V d = kDiagPC ? a.pc.dinv[row] : V(0);
#pragma unroll
            for (int q = 0; q < NP; ++q) {
              if (act[q]) {
                x[q] = x[q] + alpha[q] * pv[q];
                r[q] = r[q] - alpha[q] * qv[q];
              }
              rr[q] += r[q] * r[q];
              if (kDiagPC) rz[q] += r[q] * (d * r[q]);
            }
            store_row<V, NP>(a.X, row, x);
            store_row<V, NP>(a.R, row, r);
          } else {
#pragma unroll
            for (int q = 0; q < NP; ++q) r[q] = V(0);
          }
          if constexpr (PC == kPrecTwoLevel) {
            if (rseg) {
              // the unit's rows cover aggregates gl..gh, each a lane range
              const int g = valid ? a.pc.agg[row] : -1;
              const int gl = __shfl_sync(0xffffffffu, g, 0);
              const int gh = __shfl_sync(0xffffffffu, g, a.unit_row[u + 1] - a.unit_row[u] - 1);
              for (int gg = gl; gg >= 0 && gg <= gh; ++gg) {
                if (gg != cg) {
                  if (cg >= 0)
                    restrict_flush<V, NP>(a, p, cg, hs && cg == gF, ts && cg == gL && !(hs && cg == gF), cacc);
                  cg = gg;
#pragma unroll
                  for (int q = 0; q < NP; ++q) cacc[q] = S(0);
                }
                if (g == gg) {
#pragma unroll
                  for (int q = 0; q < NP; ++q) cacc[q] += (S)r[q];
                }
              }
            }
          }
        }
        if constexpr (PC == kPrecTwoLevel) {
          if (rseg && cg >= 0)
            restrict_flush<V, NP>(a, p, cg, hs && cg == gF, ts && cg == gL && !(hs && cg == gF), cacc);
        }
      }
      warp_store_partials<NP>(rr, part_rr + (int64_t)p * NP);
      if (kDiagPC) warp_store_partials<NP>(rz, part_rz + (int64_t)p * NP);
    })
    if (a.fold) {
      __syncthreads();
      fold_pieces<V, NP>(a, part_rr, slot_rr);
      if (kDiagPC) fold_pieces<V, NP>(a, part_rz, slot_rz);
    }
    if (!grid_sync(a.bar)) return;
    mark(2);

    if constexpr (PC == kPrecTwoLevel) {
      // ---- phases R, G: coarse correction of the new residual (the
      // restriction ran in phase B when aggregates are row ranges)
      if (!a.pc.agg_contig) {
        coarse_restrict<V, NP>(a, st_cur, false);
        if (!grid_sync(a.bar)) return;
      }
      mark(3);
      // coarse phase k = it + 1 takes groups from counter k % 2; the other
      // one is cleared in the direction phase for phase k + 1
      coarse_solve<V, NP>(a, st_cur, false, reinterpret_cast<float*>(stage_raw), kStageBytes / 4, c_bytes,
                          a.cq + ((it + 1) & 1));
      if (!grid_sync(a.bar)) return;
      mark(4);
    }

    if constexpr (PC == kPrecIC0) {
      // ---- phase B2: Z = (L L')^-1 R by level-scheduled solves, then r'z
      if (!ic0_apply_grid<V, NP>(a)) return;
      FOR_MY_PIECES(a, {
        S acc[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] = S(0);
        piece_rz<V, NP>(a, u0, u1, acc);
        warp_store_partials<NP>(acc, part_rz + (int64_t)p * NP);
      })
      if (a.fold) {
        __syncthreads();
        fold_pieces<V, NP>(a, part_rz, slot_rz);
      }
      if (!grid_sync(a.bar)) return;
      mark(3);
    }

    if constexpr (PC == kPrecFactored) {
      // ---- phase B2: T = G R and r'z = ||T||^2 (G'T is applied in phase C)
      FOR_MY_PIECES(a, {
        S acc[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) acc[q] = S(0);
        bool anyact = false;
#pragma unroll
        for (int q = 0; q < NP; ++q) anyact |= st_cur[s * NP + q] == kActive;
        if (anyact) factor_first_half<V, NP>(a, u0, u1, acc);
        warp_store_partials<NP>(acc, part_rz + (int64_t)p * NP);
      })
      if (a.fold) {
        __syncthreads();
        fold_pieces<V, NP>(a, part_rz, slot_rz);
      }
      if (!grid_sync(a.bar)) return;
      mark(3);
    }

    // ---- phase C: convergence, beta, P = Z + beta P
    if (PC == kPrecTwoLevel && blockIdx.x == 0 && threadIdx.x == 0) a.cq[it & 1] = 0u;
    FOR_MY_PIECES(a, {
      S pq[NP], rzn[NP], rr[NP];
      piece_totals<V, NP>(a, part_pq, slot_pq, s, pq);
      piece_totals<V, NP>(a, part_rz, slot_rz, s, rzn);
      piece_totals<V, NP>(a, part_rr, slot_rr, s, rr);
      if constexpr (PC == kPrecTwoLevel) {
        S c[NP];
        coarse_totals<V, NP>(a, s, c);
#pragma unroll
        for (int q = 0; q < NP; ++q) rzn[q] += c[q];
      }
      V beta[NP];
      bool act[NP];
      bool any = false;
      const bool first = a.seg_piece[s] == p;
      const bool ru_slot = RU && ((it + 1) % a.ru_every == 0);
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        const int32_t st0 = st_cur[s * NP + q];
        int32_t st = st0;
        bool req = false;
        if (st0 == kActive) {
          if (!(pq[q] > S(0)) || !isfinite(pq[q])) st = LAPY_ERR_BREAKDOWN;
          else if (!isfinite(rr[q]) || !isfinite(rzn[q])) st = LAPY_ERR_NAN;
          else if (RU) {
            // the FP32 residual fell by delta (or to the tolerance): request an
            // FP64 update at the next update slot
            req = (ru_slot && (rr[q] <= a.rtol2 * a.bb[s * NP + q] || rr[q] <= a.delta2 * a.rref[s * NP + q])) ||
                  rr[q] == S(0);
            if (!(rzn[q] > S(0)) && !req) st = LAPY_ERR_BREAKDOWN;
          } else if (rr[q] <= a.rtol2 * a.bb[s * NP + q]) st = it + 1;
          else if (!(rzn[q] > S(0))) st = LAPY_ERR_BREAKDOWN;
        }
        act[q] = st == kActive;
        beta[q] = (act[q] && rzn[q] > S(0)) ? (V)(rzn[q] / rz_cur[s * NP + q]) : V(0);
        any |= act[q];
        if (first && lane == q) {
          st_nxt[s * NP + q] = st;
          rz_nxt[s * NP + q] = rzn[q];
          if (act[q]) s_act = 1;
          if (RU && req) {
            a.ru_col[(par ^ 1) * (int64_t)a.nseg * NP + s * NP + q] = 1;
            atomicOr(&a.ru_flag[par ^ 1], 1u);
          }
        }
      }
      if constexpr (PC == kPrecTwoLevel) {
        if (!any) continue;
        // z = dinv .* r + yc[agg]: the next unit's row range and aggregate
        // labels are loaded one unit ahead, so the coarse value is not a
        // second dependent round trip after the label
        int rb = a.unit_row[u0], re = a.unit_row[u0 + 1];
        int gn = rb + lane < re ? a.pc.agg[rb + lane] : -1;
        for (int u = u0; u < u1; ++u) {
          const int row = rb + lane;
          const bool valid = row < re;
          const int g = gn;
          rb = re;
          if (u + 1 < u1) {
            re = a.unit_row[u + 2];
            gn = rb + lane < re ? a.pc.agg[rb + lane] : -1;
          }
          if (valid) {
            V r[NP], z[NP], pv[NP];
            load_row<V, NP>(a.R, row, r);
            load_row<V, NP>(a.P, row, pv);
            const V d = a.pc.dinv[row];
            V y[NP];
            if (g >= 0) load_row<V, NP>(a.yc, g, y);
#pragma unroll
            for (int q = 0; q < NP; ++q) z[q] = d * r[q] + (g >= 0 ? y[q] : V(0));
#pragma unroll
            for (int q = 0; q < NP; ++q)
              if (act[q]) pv[q] = z[q] + beta[q] * pv[q];
            store_row<V, NP>(a.P, row, pv);
          }
        }
      } else if (any) {  // Jacobi, IC(0), learned factor
        for (int u = u0; u < u1; ++u) {
          const int row = a.unit_row[u] + lane;
          if (row < a.unit_row[u + 1]) {
            V z[NP], pv[NP];
            if (kDiagPC) {
              V r[NP];
              load_row<V, NP>(a.R, row, r);
              apply_diag_coarse<V, NP, PC>(a, row, r, z);
            } else if constexpr (PC == kPrecIC0) {
              load_row<V, NP>(a.Z, row, z);
            } else {
              row_apply<V, NP>(a.pc.gt_sell, a.pc.gt_ptr, a.pc.gt_idx, a.pc.gt_val, a.T, u, row, true, z);
            }
            load_row<V, NP>(a.P, row, pv);
#pragma unroll
            for (int q = 0; q < NP; ++q)
              if (act[q]) pv[q] = z[q] + beta[q] * pv[q];
            store_row<V, NP>(a.P, row, pv);
          }
        }
      }
    })
    if (!grid_sync(a.bar, &s_act, &s_seen)) return;
    mark(5);
    nact = s_seen - seen_prev;
    seen_prev = s_seen;
  }

  // ---- publish the final state (the warp holding a segment's first piece)
  const int par = it & 1;
  const int32_t* st_fin = a.state + par * (int64_t)a.nseg * NP;
  FOR_MY_PIECES(a, {
    if (RU) {  // corrections not yet folded in (columns stopped between updates)
      for (int u = u0; u < u1; ++u) {
        const int row = a.unit_row[u] + lane;
        if (row < a.unit_row[u + 1]) {
          V x[NP];
          double x64[NP];
          load_row<V, NP>(a.X, row, x);
          load_row<double, NP>(a.X64, row, x64);
#pragma unroll
          for (int q = 0; q < NP; ++q) x64[q] += (double)x[q];
          store_row<double, NP>(a.X64, row, x64);
        }
      }
    }
    if (a.seg_piece[s] == p && lane < NP) {
      int32_t st = st_fin[s * NP + lane];
      if (st == kActive) st = LAPY_ERR_NOCONV;
      a.state_out[s * NP + lane] = st;
    }
  })
  if (blockIdx.x == 0 && threadIdx.x == 0) a.iters[0] = it;
  mark(6);
  if (lane == 0 && w_rows != 0) {
    atomicAdd(&a.work[0], w_rows);
    atomicAdd(&a.work[1], w_nnz);
  }
  if (threadIdx.x == 0 && c_bytes != 0) atomicAdd(a.cwork, c_bytes);
}

// ---- sliced-ELL construction ---------------------------------------------
__global__ void sell_width_kernel(int nunit, const int32_t* __restrict__ unit_row, const int32_t* __restrict__ indptr,
                                  int32_t* __restrict__ slice_elems) {
  const int u = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (u >= nunit) return;
  const int r = unit_row[u] + lane;
  const int len = (r < unit_row[u + 1]) ? indptr[r + 1] - indptr[r] : 0;
  const int w = warp_max(len);
  if (lane == 0) slice_elems[u] = 32 * w;
}

template <typename V>
__global__ void sell_fill_kernel(int nunit, const int32_t* __restrict__ unit_row, const int32_t* __restrict__ indptr,
                                 const int32_t* __restrict__ indices, const V* __restrict__ vals,
                                 const int32_t* __restrict__ slice_ptr, int32_t* __restrict__ col,
                                 V* __restrict__ val) {
  const int u = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (u >= nunit) return;
  const int r0 = unit_row[u];
  const int r = r0 + lane;
  const bool valid = r < unit_row[u + 1];
  const int32_t kb = valid ? indptr[r] : 0, len = valid ? indptr[r + 1] - kb : 0;
  const int32_t base = slice_ptr[u];
  const int w = (slice_ptr[u + 1] - base) >> 5;
  for (int k = 0; k < w; ++k) {
    const int32_t pos = base + 32 * k + lane;
    if (k < len) {
      col[pos] = indices[kb + k];
      val[pos] = vals[kb + k];
    } else {
      col[pos] = valid ? r : r0;
      val[pos] = V(0);
    }
  }
}

size_t sell_bytes_bound(int64_t nnz, const ChunkTable& ct, int elem_size, double pad) {
  const size_t elems = (size_t)(pad * (double)nnz) + 64 * (size_t)ct.nunit;
  return a256(4 * (size_t)(ct.nunit + 1)) + a256(4 * (size_t)scan_scratch_elems(ct.nunit + 1)) +
         a256(4 * (size_t)(ct.nunit + 1)) + a256(4 * elems) + a256((size_t)elem_size * elems) + 256;
}

template <typename V>
int build_sell(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals, const ChunkTable& ct,
               void* mem, size_t bytes, SellMatrix<V>* out, bool* fits, cudaStream_t stream) {
  (void)n;
  *fits = false;
  if (bytes < sell_bytes_bound(0, ct, sizeof(V))) return LAPY_OK;
  char* w = (char*)(((uintptr_t)mem + 255) & ~uintptr_t(255));
  char* end = (char*)mem + bytes;
  int32_t* counts = (int32_t*)w; w += a256(4 * (size_t)(ct.nunit + 1));
  int32_t* scratch = (int32_t*)w; w += a256(4 * (size_t)scan_scratch_elems(ct.nunit + 1));
  int32_t* slice_ptr = (int32_t*)w; w += a256(4 * (size_t)(ct.nunit + 1));
  const unsigned blocks = lapy_ceil_div((int64_t)ct.nunit * 32, 256);
  sell_width_kernel<<<blocks, 256, 0, stream>>>(ct.nunit, ct.unit_row, indptr, counts);
  LAPY_TRY(lapy_check_launch("sell_width_kernel"));
  LAPY_TRY(exclusive_scan_i32(counts, slice_ptr, ct.nunit, scratch, stream));
  int32_t total = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&total, slice_ptr + ct.nunit, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  const size_t need = a256(4 * (size_t)total) + a256(sizeof(V) * (size_t)total);
  if ((size_t)(end - w) < need || total < 0) return LAPY_OK;  // too much padding: the CSR path is used
  int32_t* col = (int32_t*)w; w += a256(4 * (size_t)total);
  V* val = (V*)w;
  sell_fill_kernel<V><<<blocks, 256, 0, stream>>>(ct.nunit, ct.unit_row, indptr, indices, vals, slice_ptr, col, val);
  LAPY_TRY(lapy_check_launch("sell_fill_kernel"));
  out->slice_ptr = slice_ptr;
  out->col = col;
  out->val = val;
  *fits = true;
  return LAPY_OK;
}

template int build_sell<float>(int64_t, const int32_t*, const int32_t*, const float*, const ChunkTable&, void*,
                               size_t, SellMatrix<float>*, bool*, cudaStream_t);
template int build_sell<double>(int64_t, const int32_t*, const int32_t*, const double*, const ChunkTable&, void*,
                                size_t, SellMatrix<double>*, bool*, cudaStream_t);

size_t pcg_workspace_bytes(int64_t n, int p, const ChunkTable& ct, int elem_size, int precond, int64_t nagg) {
  const size_t vec = a256((size_t)n * p * elem_size);
  size_t b = vec * (precond == kPrecFactored ? 4 : precond == kPrecIC0 ? 5 : 3);  // R P Q (+ T, + Z)
  b += a256(sizeof(double) * 3 * (size_t)ct.npiece * p);
  b += a256(sizeof(double) * 3 * (size_t)ct.nslot * p);
  b += a256(sizeof(double) * (size_t)ct.nslot * p);
  b += a256(sizeof(double) * 2 * (size_t)ct.nseg * p);
  b += a256(sizeof(double) * (size_t)ct.nseg * p);
  b += a256(sizeof(int32_t) * 2 * (size_t)ct.nseg * p);
  b += a256(256);  // control words and the barrier word
  // reliable updates: FP64 partials, reference residuals, request flags
  b += a256(sizeof(double) * (size_t)ct.npiece * p) + a256(sizeof(double) * (size_t)ct.nseg * p) +
       a256(sizeof(int32_t) * 2 * (size_t)ct.nseg * p);
  if (precond == kPrecTwoLevel) {
    b += 3 * a256(sizeof(double) * (size_t)std::max<int64_t>(nagg, 1) * p);
    b += a256(sizeof(double) * (size_t)(nagg + ct.nvc + 1) * p);  // coarse reduction slots
    b += a256(sizeof(double) * 2 * (size_t)ct.npiece * p) + a256(sizeof(int32_t) * (size_t)std::max<int64_t>(nagg, 1));
  }
  return b + 256;
}

template <typename V, int NP, int PC, bool RU>
static int launch_pcg(PcgArgs<V>& args, int ctas_per_sm, cudaStream_t stream) {
  auto kern = pcg_kernel<V, NP, PC, RU>;
  int per_sm = 0;
  LAPY_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPcgThreads, 0));
  if (per_sm <= 0) {
    lapy_set_last_message("pcg: kernel cannot be resident (occupancy 0)");
    return LAPY_ERR_CUDA;
  }
  per_sm = std::max(1, std::min({per_sm, kPlanCtasPerSm, ctas_per_sm}));
  const int grid = std::max(1, std::min(per_sm * lapy_num_sms(), (args.nvw + kWarps - 1) / kWarps));
  void* kargs[] = {(void*)&args};
  LAPY_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kPcgThreads), kargs, 0, stream));
  return lapy_check_launch("pcg_kernel");
}

template <typename V, int PC, bool RU = false>
static int launch_pcg_np(PcgArgs<V>& args, int p, int ctas_per_sm, cudaStream_t stream) {
  switch (p) {
    case 1: return launch_pcg<V, 1, PC, RU>(args, ctas_per_sm, stream);
    case 2: return launch_pcg<V, 2, PC, RU>(args, ctas_per_sm, stream);
    case 4: return launch_pcg<V, 4, PC, RU>(args, ctas_per_sm, stream);
    case 8: return launch_pcg<V, 8, PC, RU>(args, ctas_per_sm, stream);
    case 16: return launch_pcg<V, 16, PC, RU>(args, ctas_per_sm, stream);
    default:
      lapy_set_last_message("pcg: block width %d not in {1,2,4,8,16}", p);
      return LAPY_ERR_INVALID;
  }
}

// Workspace layout and launch shared by the plain and reliable-update solves.
template <typename V>
static int pcg_run(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals,
                   const SellMatrix<V>* sell, const PcgPrecondDesc<V>& pc, int p, const ChunkTable& ct,
                   const V* B, V* X, double rtol, int maxiter, int32_t* state_dev, void* ws, size_t ws_bytes,
                   cudaStream_t stream, int* iters_out, const double* K64, const double* B64, double* X64,
                   double delta, int ru_every, int* updates_out, const PcgTuning* tuning) {
  const PcgTuning tn = tuning ? *tuning : PcgTuning();
  if (ws_bytes < pcg_workspace_bytes(n, p, ct, sizeof(V), pc.kind, pc.nagg)) return LAPY_ERR_WORKSPACE;
  const bool ru = B64 != nullptr;
  char* w = (char*)(((uintptr_t)ws + 255) & ~uintptr_t(255));
  const size_t vec = a256((size_t)n * p * sizeof(V));
  PcgArgs<V> a{};
  a.n = n;
  a.indptr = indptr;
  a.indices = indices;
  a.vals = vals;
  a.use_sell = sell != nullptr && sell->val != nullptr;
  if (a.use_sell) a.sell = *sell;
  a.pc = pc;
  a.unit_row = ct.unit_row;
  a.piece_unit = ct.piece_unit;
  a.piece_seg = ct.piece_seg;
  a.vw_piece = ct.vw_piece;
  a.seg_piece = ct.seg_piece;
  a.vc_piece = ct.vc_piece;
  a.seg_slot = ct.seg_slot;
  a.seg_vc0 = ct.seg_vc0;
  a.nvc = ct.nvc;
  a.nslot = ct.nslot;
  {
    // fold into reduction slots only when some segment has many pieces (or
    // coarse unknowns): with few, the direct sums are cheaper
    int maxp = 0;
    for (int s = 0; s < ct.nseg; ++s) maxp = std::max(maxp, ct.h_seg_piece[s + 1] - ct.h_seg_piece[s]);
    a.fold = (maxp > tn.fold_pieces || (pc.kind == kPrecTwoLevel && pc.max_seg_agg > tn.fold_aggs)) ? 1 : 0;
  }
  a.nvw = ct.nvw;
  a.npiece = ct.npiece;
  a.nseg = ct.nseg;
  a.B = B;
  a.X = X;
  a.R = (V*)w; w += vec;
  a.P = (V*)w; w += vec;
  a.Q = (V*)w; w += vec;
  a.Z = nullptr;
  a.T = nullptr;
  if (pc.kind == kPrecFactored || pc.kind == kPrecIC0) {
    a.T = (V*)w; w += vec;
  }
  if (pc.kind == kPrecIC0) {
    a.Z = (V*)w; w += vec;
  }
  using S = ScalarOf<V>;
  a.part = (S*)w; w += a256(sizeof(double) * 3 * (size_t)ct.npiece * p);
  a.slot = (S*)w; w += a256(sizeof(double) * 3 * (size_t)ct.nslot * p);
  a.rz = (S*)w; w += a256(sizeof(double) * 2 * (size_t)ct.nseg * p);
  a.bb = (S*)w; w += a256(sizeof(double) * (size_t)ct.nseg * p);
  a.state = (int32_t*)w; w += a256(sizeof(int32_t) * 2 * (size_t)ct.nseg * p);
  // control words: [2] iters, [5] err, [6..9] work (u64 x2), [10..11] ru_flag,
  // [12] updates, [14..27] phase times (u64 x kPcgPhases), [28..29] coarse
  // bytes (u64), [30..31] coarse task-group counters; the barrier word sits
  // alone on the next 128-byte line
  static_assert(14 + 2 * kPcgPhases <= 28, "phase timers overlap the coarse byte counter");
  unsigned* ctl = (unsigned*)w;
  w += a256(256);
  a.iters = (int*)(ctl + 2);
  a.bar.word = (unsigned long long*)(ctl + 32);
  a.bar.err = (int*)(ctl + 5);
  a.work = (unsigned long long*)(ctl + 6);
  a.ru_flag = ctl + 10;
  a.n_updates = ctl + 12;
  a.cwork = (unsigned long long*)(ctl + 28);
  a.cq = ctl + 30;
  a.part64 = (double*)w; w += a256(sizeof(double) * (size_t)ct.npiece * p);
  a.slot64 = (double*)w; w += a256(sizeof(double) * (size_t)ct.nslot * p);
  a.rref = (S*)w; w += a256(sizeof(double) * (size_t)ct.nseg * p);
  a.ru_col = (int32_t*)w; w += a256(sizeof(int32_t) * 2 * (size_t)ct.nseg * p);
  if (pc.kind == kPrecTwoLevel) {
    const size_t cb = a256(sizeof(double) * (size_t)std::max(pc.nagg, 1) * p);
    a.rc = (S*)w; w += cb;
    a.yc = (S*)w; w += cb;
    a.csl = (S*)w; w += cb;
    if ((int64_t)pc.naslot > (int64_t)pc.nagg + ct.nvc + 1) {
      lapy_set_last_message("pcg: coarse reduction slots exceed the workspace bound");
      return LAPY_ERR_WORKSPACE;
    }
    a.aslot = (S*)w; w += a256(sizeof(double) * (size_t)(pc.nagg + ct.nvc + 1) * p);
    a.rc_part = (S*)w; w += a256(sizeof(double) * 2 * (size_t)ct.npiece * p);
    a.rc_cnt = (int32_t*)w; w += a256(sizeof(int32_t) * (size_t)std::max(pc.nagg, 1));
  }
  a.state_out = state_dev;
  a.rtol2 = (S)(rtol * rtol);
  a.rtol2_64 = rtol * rtol;
  a.maxiter = maxiter;
  a.B64 = B64;
  a.X64 = X64;
  a.K64 = K64;
  a.delta2 = (S)(delta * delta);
  a.ru_every = std::max(1, ru_every);
  LAPY_CUDA_TRY(cudaMemsetAsync(ctl, 0, 256, stream));
  // every slot is rewritten by each fold; cleared once so that none is ever
  // read uninitialised
  LAPY_CUDA_TRY(cudaMemsetAsync(a.slot, 0, sizeof(double) * 3 * (size_t)ct.nslot * p, stream));
  if (pc.kind == kPrecTwoLevel) {
    LAPY_CUDA_TRY(cudaMemsetAsync(a.aslot, 0, sizeof(double) * (size_t)std::max(pc.naslot, 1) * p, stream));
    LAPY_CUDA_TRY(cudaMemsetAsync(a.rc_cnt, 0, sizeof(int32_t) * (size_t)std::max(pc.nagg, 1), stream));
  }
  LAPY_CUDA_TRY(cudaMemsetAsync(a.slot64, 0, sizeof(double) * (size_t)ct.nslot * p, stream));
  if (ru) LAPY_CUDA_TRY(cudaMemsetAsync(a.ru_col, 0, sizeof(int32_t) * 2 * (size_t)ct.nseg * p, stream));
  // segments without rows have no piece: they are reported as solved
  LAPY_CUDA_TRY(cudaMemsetAsync(state_dev, 0, sizeof(int32_t) * (size_t)ct.nseg * p, stream));
  int st;
  const bool prof = lapy_profile_enabled();
  a.phase_ns = prof ? (unsigned long long*)(ctl + 14) : nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (prof) {
    LAPY_CUDA_TRY(cudaEventCreate(&e0));
    LAPY_CUDA_TRY(cudaEventCreate(&e1));
    LAPY_CUDA_TRY(cudaEventRecord(e0, stream));
  }
  if (ru) {
    if constexpr (sizeof(V) == 4) {
      if (pc.kind != kPrecJacobi) {
        lapy_set_last_message("pcg: reliable updates need the Jacobi preconditioner");
        return LAPY_ERR_INVALID;
      }
      st = launch_pcg_np<V, kPrecJacobi, true>(a, p, tn.ctas_per_sm, stream);
    } else {
      lapy_set_last_message("pcg: reliable updates run FP32 iterations");
      return LAPY_ERR_INVALID;
    }
  } else if (pc.kind == kPrecFactored) {
    st = launch_pcg_np<V, kPrecFactored>(a, p, tn.ctas_per_sm, stream);
  } else if (pc.kind == kPrecIC0) {
    if constexpr (sizeof(V) == 4) {
      st = launch_pcg_np<V, kPrecIC0>(a, p, tn.ctas_per_sm, stream);
    } else {
      lapy_set_last_message("pcg: the IC(0) preconditioner runs FP32 iterations");
      return LAPY_ERR_INVALID;
    }
  } else if (pc.kind == kPrecTwoLevel) {
    if constexpr (sizeof(V) == 4) {
      st = launch_pcg_np<V, kPrecTwoLevel>(a, p, tn.ctas_per_sm, stream);
    } else {
      lapy_set_last_message("pcg: the two-level preconditioner runs FP32 iterations");
      return LAPY_ERR_INVALID;
    }
  } else {
    st = launch_pcg_np<V, kPrecJacobi>(a, p, tn.ctas_per_sm, stream);
  }
  if (st != LAPY_OK) return st;
  if (prof) LAPY_CUDA_TRY(cudaEventRecord(e1, stream));
  unsigned hctl[32];
  LAPY_CUDA_TRY(cudaMemcpyAsync(hctl, ctl, sizeof(hctl), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (prof) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    unsigned long long rows, nnz;
    memcpy(&rows, &hctl[6], 8);
    memcpy(&nnz, &hctl[8], 8);
    unsigned long long cbytes;
    memcpy(&cbytes, &hctl[28], 8);
    lapy_profile_add_pcg(ms, (long long)hctl[2], (long long)rows, (long long)nnz, p, (int)sizeof(V), pc.kind,
                         (double)cbytes, pc.kind == kPrecTwoLevel && pc.agg_contig != 0);
    double phase_ms[kPcgPhases];
    for (int k = 0; k < kPcgPhases; ++k) {
      unsigned long long ns;
      memcpy(&ns, &hctl[14 + 2 * k], 8);
      phase_ms[k] = (double)ns * 1e-6;
    }
    lapy_profile_add_phases(phase_ms);
  }
  if (hctl[5] != 0) {
    lapy_set_last_message("pcg: grid barrier timed out");
    return LAPY_ERR_TIMEOUT;
  }
  if (iters_out) *iters_out = (int)hctl[2];
  if (updates_out) *updates_out = (int)hctl[12];
  return LAPY_OK;
}

template <typename V>
int pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals,
              const SellMatrix<V>* sell, const PcgPrecondDesc<V>& pc, int p, const ChunkTable& ct,
              const V* B, V* X, double rtol, int maxiter, int32_t* state_dev, void* ws, size_t ws_bytes,
              cudaStream_t stream, int* iters_out, const PcgTuning* tuning) {
  return pcg_run<V>(n, indptr, indices, vals, sell, pc, p, ct, B, X, rtol, maxiter, state_dev, ws, ws_bytes,
                    stream, iters_out, nullptr, nullptr, nullptr, 0.0, 1, nullptr, tuning);
}

int pcg_solve_ru(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k64, const float* k32,
                 const SellMatrix<float>* sell, const float* dinv32, int p, const ChunkTable& ct, const double* B,
                 double* X, float* X32, double rtol, double delta, int ru_every, int maxiter, int32_t* state_dev,
                 void* ws, size_t ws_bytes, cudaStream_t stream, int* iters_out, int* updates_out) {
  PcgPrecondDesc<float> pc;
  pc.kind = kPrecJacobi;
  pc.dinv = dinv32;
  return pcg_run<float>(n, indptr, indices, k32, sell, pc, p, ct, nullptr, X32, rtol, maxiter, state_dev, ws,
                        ws_bytes, stream, iters_out, k64, B, X, delta, ru_every, updates_out, nullptr);
}

template int pcg_solve<float>(int64_t, const int32_t*, const int32_t*, const float*, const SellMatrix<float>*,
                              const PcgPrecondDesc<float>&, int, const ChunkTable&, const float*,
                              float*, double, int, int32_t*, void*, size_t, cudaStream_t, int*,
                              const PcgTuning*);
template int pcg_solve<double>(int64_t, const int32_t*, const int32_t*, const double*, const SellMatrix<double>*,
                               const PcgPrecondDesc<double>&, int, const ChunkTable&, const double*,
                               double*, double, int, int32_t*, void*, size_t, cudaStream_t, int*,
                               const PcgTuning*);

// Standalone FP32 SELL product Y = Mat X (row-major n x NP): the PCG's SpMM
// outside the persistent kernel.  Every warp takes a contiguous range of
// units and runs them through the same cp.async double-buffered slice
// pipeline as the PCG (sell_piece_spmm).
template <int NP>
__global__ void __launch_bounds__(256) sell_spmm_pipe_kernel(SellMatrix<float> M, const int32_t* __restrict__ unit_row,
                                                             int nunit, const float* __restrict__ X,
                                                             float* __restrict__ Y) {
  __shared__ __align__(16) float slots[kWarps][2 * kSellShort * 32 * 2];
  const int warp = threadIdx.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * kWarps + warp, nw = (int64_t)gridDim.x * kWarps;
  const int u0 = (int)(nunit * gw / nw), u1 = (int)(nunit * (gw + 1) / nw);
  if (u0 >= u1) return;
  float dummy[NP];
  sell_piece_spmm<NP, false>(M, X, Y, nullptr, unit_row, u0, u1, slots[warp], dummy);
}

template <int NP>
static int launch_sell_pipe(const SellMatrix<float>& M, const int32_t* unit_row, int nunit, const float* X, float* Y,
                            cudaStream_t stream) {
  int per_sm = 0;
  LAPY_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sell_spmm_pipe_kernel<NP>, 256, 0));
  per_sm = std::max(1, per_sm);
  const int grid = std::max(1, std::min(per_sm * lapy_num_sms(), (nunit + kWarps - 1) / kWarps));
  sell_spmm_pipe_kernel<NP><<<grid, 256, 0, stream>>>(M, unit_row, nunit, X, Y);
  return lapy_check_launch("sell_spmm_pipe_kernel");
}

}  // namespace lapy

// Standalone SELL product: workspace = chunk table, FP32 values, SELL copy.
static size_t sell_f32_layout(int64_t nnz, const lapy::ChunkTable& ct, size_t* off_vals, size_t* off_sell) {
  using namespace lapy;
  size_t off = a256(chunk_table_bytes(ct));
  *off_vals = off;
  off += a256(4 * (size_t)nnz);
  *off_sell = off;
  return off + sell_bytes_bound(nnz, ct, sizeof(float)) + 256;
}

extern "C" size_t lapy_sell_f32_workspace_bytes(int64_t n, int64_t nnz, int nseg, const int32_t* seg_row) {
  using namespace lapy;
  if (n <= 0 || nnz <= 0 || nseg <= 0 || !seg_row) return 0;
  ChunkTable ct;
  plan_chunks(seg_row, nseg, 4 * lapy_num_sms(), &ct);
  size_t a, b;
  return sell_f32_layout(nnz, ct, &a, &b);
}

extern "C" int lapy_sell_f32_build(int64_t n, const int32_t* indptr, const int32_t* indices, const double* vals,
                                   int64_t nnz, int nseg, const int32_t* seg_row, lapy_sell_f32* out, void* work,
                                   size_t ws_bytes, void* stream_) {
  using namespace lapy;
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n <= 0 || nnz <= 0 || nseg <= 0 || !seg_row || !indptr || !indices || !vals || !out || !work) {
    lapy_set_last_message("sell_f32_build: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (seg_row[0] != 0 || seg_row[nseg] != n) {
    lapy_set_last_message("sell_f32_build: segment rows must span [0, n)");
    return LAPY_ERR_INVALID;
  }
  ChunkTable ct;
  plan_chunks(seg_row, nseg, 4 * lapy_num_sms(), &ct);
  size_t off_vals, off_sell;
  const size_t need = sell_f32_layout(nnz, ct, &off_vals, &off_sell);
  if (ws_bytes < need) return LAPY_ERR_WORKSPACE;
  char* base = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  LAPY_TRY(upload_chunk_table(&ct, base, stream));
  float* v32 = (float*)(base + off_vals);
  LAPY_TRY(cast_f64_f32(nnz, vals, v32, stream));
  SellMatrix<float> sm;
  bool fits = false;
  LAPY_TRY(build_sell<float>(n, indptr, indices, v32, ct, base + off_sell, need - off_sell - 256, &sm, &fits, stream));
  if (!fits) {
    lapy_set_last_message("sell_f32_build: the padded matrix exceeds the reserved space");
    return LAPY_ERR_WORKSPACE;
  }
  out->nunit = ct.nunit;
  out->unit_row = ct.unit_row;
  out->slice_ptr = sm.slice_ptr;
  out->col = sm.col;
  out->val = sm.val;
  return LAPY_OK;
}

extern "C" int lapy_sell_f32_spmm(const lapy_sell_f32* m, int ncol, const float* x, float* y, void* stream_) {
  using namespace lapy;
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!m || !m->slice_ptr || !m->col || !m->val || !m->unit_row || m->nunit <= 0 || !x || !y) {
    lapy_set_last_message("sell_f32_spmm: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  SellMatrix<float> sm;
  sm.slice_ptr = m->slice_ptr;
  sm.col = m->col;
  sm.val = m->val;
  switch (ncol) {
    case 1: return launch_sell_pipe<1>(sm, m->unit_row, m->nunit, x, y, stream);
    case 2: return launch_sell_pipe<2>(sm, m->unit_row, m->nunit, x, y, stream);
    case 4: return launch_sell_pipe<4>(sm, m->unit_row, m->nunit, x, y, stream);
    case 8: return launch_sell_pipe<8>(sm, m->unit_row, m->nunit, x, y, stream);
    default:
      lapy_set_last_message("sell_f32_spmm: ncol %d not in {1, 2, 4, 8}", ncol);
      return LAPY_ERR_INVALID;
  }
}

// Consistency of the persistent PCG's warp plan for the given segments (host
// only, no device work): every virtual warp and virtual CTA holds at least one
// piece, every reduction slot of a segment belongs to a virtual CTA that holds
// a piece of it, pieces stay inside their segment, and the 32-row units of the
// pieces cover every row exactly once.
extern "C" int lapy_plan_check(const int32_t* seg_row, int nseg) {
  using namespace lapy;
  if (nseg < 0 || (nseg > 0 && !seg_row)) return LAPY_ERR_INVALID;
  for (int s = 0; s < nseg; ++s)
    if (seg_row[s + 1] < seg_row[s]) return LAPY_ERR_INVALID;
  ChunkTable ct;
  plan_chunks(seg_row, nseg, 4 * lapy_num_sms(), &ct);
  auto fail = [](const char* what) {
    lapy_set_last_message("plan_check: %s", what);
    return LAPY_ERR_INVALID;
  };
  const int64_t total = nseg > 0 ? (int64_t)seg_row[nseg] - seg_row[0] : 0;
  if (total > 0) {
    for (int w = 0; w < ct.nvw; ++w)
      if (ct.h_vw_piece[w + 1] <= ct.h_vw_piece[w]) return fail("a virtual warp holds no piece");
    for (int v = 0; v < ct.nvc; ++v)
      if (ct.h_vc_piece[v + 1] <= ct.h_vc_piece[v]) return fail("a virtual CTA holds no piece");
  }
  if (ct.nvc != (ct.nvw + kWarps - 1) / kWarps || ct.h_vc_piece[ct.nvc] != ct.npiece)
    return fail("virtual CTA table");
  std::vector<int> piece_vc(ct.npiece);
  for (int w = 0; w < ct.nvw; ++w)
    for (int32_t q = ct.h_vw_piece[w]; q < ct.h_vw_piece[w + 1]; ++q) piece_vc[q] = w / kWarps;
  for (int s = 0; s < nseg; ++s) {
    const int32_t q0 = ct.h_seg_piece[s], q1 = ct.h_seg_piece[s + 1];
    const int ns = ct.h_seg_slot[s + 1] - ct.h_seg_slot[s];
    if ((seg_row[s + 1] > seg_row[s]) != (q1 > q0)) return fail("segment without pieces");
    if (q1 <= q0) {
      if (ns != 0) return fail("slots of an empty segment");
      continue;
    }
    std::vector<char> seen(ns, 0);
    for (int32_t q = q0; q < q1; ++q) {
      if (ct.h_piece_seg[q] != s) return fail("piece outside its segment");
      const int k = piece_vc[q] - ct.h_seg_vc0[s];
      if (k < 0 || k >= ns) return fail("piece outside its segment's slots");
      seen[k] = 1;
    }
    for (int k = 0; k < ns; ++k)
      if (!seen[k]) return fail("slot without a piece");
  }
  std::vector<int> cover(total, 0);
  for (int q = 0; q < ct.npiece; ++q)
    for (int32_t u = ct.h_piece_unit[q]; u < ct.h_piece_unit[q + 1]; ++u)
      for (int32_t r = ct.h_unit_row[u]; r < ct.h_unit_row[u + 1]; ++r) cover[r - seg_row[0]]++;
  for (int64_t r = 0; r < total; ++r)
    if (cover[r] != 1) return fail("rows not covered exactly once");
  return LAPY_OK;
}
