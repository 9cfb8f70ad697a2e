// Persistent cooperative PCG over a block-diagonal batch of CSR systems.
//
// One launch runs the whole solve.  Rows are split into chunks that never
// cross a segment (one mesh = one segment).  Dot products are per (segment, column): each chunk writes its
// partial sum, and after a grid barrier every CTA that needs a segment's
// scalar re-reduces that segment's partials in a fixed order, so the result
// is bitwise reproducible.  Chunks are dealt to CTAs round-robin.  Three barriers per iteration (Jacobi), five with
// the factored preconditioner z = Gt (G r).  Convergence is tracked per
// (segment, column); converged columns freeze and fully converged segments
// skip their rows.  Barriers spin with a bound (common.cuh).
#include <climits>
#include <cstring>
#include <cmath>
#include "pcg.cuh"
#include "spmv.cuh"

namespace lapy {

constexpr int32_t kActive = INT32_MAX;
constexpr int kPcgThreads = 256;
// staged nonzeros per tile (values + column indices in shared memory)
constexpr int kStageCap = 3072;

int plan_chunks(const int32_t* seg_row, int nseg, int target_chunks, ChunkTable* ct) {
  const int64_t total = seg_row[nseg] - seg_row[0];
  int64_t cr = (total + std::max(1, target_chunks) - 1) / std::max(1, target_chunks);
  cr = std::max<int64_t>(32, std::min<int64_t>(1024, cr));
  cr = (cr + 31) / 32 * 32;
  ct->nseg = nseg;
  ct->h_seg_row.assign(seg_row, seg_row + nseg + 1);
  ct->h_chunk_row.clear();
  ct->h_chunk_seg.clear();
  ct->h_seg_chunk.assign(nseg + 1, 0);
  for (int s = 0; s < nseg; ++s) {
    ct->h_seg_chunk[s] = (int32_t)ct->h_chunk_seg.size();
    const int64_t r0 = seg_row[s], r1 = seg_row[s + 1];
    const int64_t len = r1 - r0;
    const int64_t nc = std::max<int64_t>(1, (len + cr - 1) / cr);
    for (int64_t k = 0; k < nc; ++k) {
      ct->h_chunk_row.push_back((int32_t)(r0 + len * k / nc));
      ct->h_chunk_seg.push_back(s);
    }
  }
  ct->h_seg_chunk[nseg] = (int32_t)ct->h_chunk_seg.size();
  ct->h_chunk_row.push_back(seg_row[nseg]);
  ct->nchunk = (int)ct->h_chunk_seg.size();
  return ct->nchunk;
}

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

size_t chunk_table_bytes(int nseg, int nchunk) {
  return a256(4 * (size_t)(nchunk + 1)) + a256(4 * (size_t)nchunk) + a256(4 * (size_t)(nseg + 1)) +
         a256(4 * (size_t)(nseg + 1));
}

int upload_chunk_table(ChunkTable* ct, void* mem, cudaStream_t stream) {
  char* p = (char*)mem;
  ct->chunk_row = (int32_t*)p; p += a256(4 * (size_t)(ct->nchunk + 1));
  ct->chunk_seg = (int32_t*)p; p += a256(4 * (size_t)ct->nchunk);
  ct->seg_chunk = (int32_t*)p; p += a256(4 * (size_t)(ct->nseg + 1));
  ct->seg_row = (int32_t*)p;
  LAPY_CUDA_TRY(cudaMemcpyAsync(ct->chunk_row, ct->h_chunk_row.data(), 4 * (ct->nchunk + 1), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(ct->chunk_seg, ct->h_chunk_seg.data(), 4 * ct->nchunk, cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(ct->seg_chunk, ct->h_seg_chunk.data(), 4 * (ct->nseg + 1), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(ct->seg_row, ct->h_seg_row.data(), 4 * (ct->nseg + 1), cudaMemcpyHostToDevice, stream));
  // pageable sources: make sure the copies completed before the vectors change
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}

template <typename V>
struct PcgArgs {
  int64_t n;
  const int32_t* indptr;
  const int32_t* indices;
  const V* vals;
  PcgPrecondDesc<V> pc;
  const int32_t* chunk_row;
  const int32_t* chunk_seg;
  const int32_t* seg_chunk;
  int nchunk;
  int nseg;
  const V* B;
  V* X;
  V* R;
  V* P;
  V* Q;
  V* Z;
  V* T;
  double* part;       // [3][nchunk][NP]  pq, rz, rr
  double* rz;         // [2][nseg][NP]
  double* bb;         // [nseg][NP]
  int32_t* state;     // [2][nseg][NP]
  int32_t* state_out; // [nseg][NP]
  unsigned* active;   // [2]
  int* iters;         // [1]
  unsigned long long* work;  // [2] rows and nonzeros processed by the SpMM phase
  double rtol2;
  int maxiter;
  GridBarrier bar;
};

// Shared scratch of one CTA.
template <int NP>
struct PcgShared {
  double red[kPcgThreads / 32][NP];
  double s0[NP], s1[NP], s2[NP];
  double scal[NP];
  int act[NP];
  int any;
  int seg;
};

// Sum part[c*NP + col] over the chunks of segment s with all threads; thread
// col < NP receives the column total in out[col].  Fixed order -> deterministic.
template <int NP>
__device__ __forceinline__ void seg_reduce(const double* __restrict__ part, int c0, int c1,
                                           PcgShared<NP>& sh, double* out) {
  const int t = threadIdx.x;
  const int col = t % NP;
  double acc = 0.0;
  for (int c = c0 + t / NP; c < c1; c += kPcgThreads / NP) acc += part[(int64_t)c * NP + col];
#pragma unroll
  for (int o = 16; o >= NP; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __syncthreads();
  if ((t & 31) < NP) sh.red[t >> 5][t & 31] = acc;
  __syncthreads();
  if (t < NP) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kPcgThreads / 32; ++w) s += sh.red[w][t];
    out[t] = s;
  }
  __syncthreads();
}

// Reduce a per-thread partial whose column is threadIdx.x % NP over the CTA
// and store it to part[c*NP + col].
template <int NP>
__device__ __forceinline__ void cta_partial_store(double acc, PcgShared<NP>& sh, double* dst) {
  const int t = threadIdx.x;
#pragma unroll
  for (int o = 16; o >= NP; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __syncthreads();
  if ((t & 31) < NP) sh.red[t >> 5][t & 31] = acc;
  __syncthreads();
  if (t < NP) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kPcgThreads / 32; ++w) s += sh.red[w][t];
    dst[t] = s;
  }
  __syncthreads();
}

// Reduce per-thread partials of all NP columns (one row per thread) and store
// them to dst[0..NP).
template <int NP>
__device__ __forceinline__ void cta_rows_partial_store(const double (&acc)[NP], PcgShared<NP>& sh,
                                                       double* dst) {
  const int t = threadIdx.x;
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    const double v = warp_sum(acc[q]);
    if ((t & 31) == 0) sh.red[t >> 5][q] = v;
  }
  __syncthreads();
  if (t < NP) {
    double s = 0.0;
#pragma unroll
    for (int w = 0; w < kPcgThreads / 32; ++w) s += sh.red[w][t];
    dst[t] = s;
  }
  __syncthreads();
}

// NP consecutive values of row `row` (vectorised: rows are NP * sizeof(V)
// aligned because every buffer starts on a 256-byte boundary).
template <typename V, int NP>
__device__ __forceinline__ void load_row(const V* __restrict__ base, int64_t row, V (&out)[NP]) {
  const V* p = base + row * NP;
  if constexpr (sizeof(V) == 4 && NP % 4 == 0) {
#pragma unroll
    for (int j = 0; j < NP / 4; ++j) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(p) + j);
      out[4 * j] = v.x; out[4 * j + 1] = v.y; out[4 * j + 2] = v.z; out[4 * j + 3] = v.w;
    }
  } else if constexpr (sizeof(V) == 4 && NP == 2) {
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    out[0] = v.x; out[1] = v.y;
  } else if constexpr (sizeof(V) == 8 && NP % 2 == 0) {
#pragma unroll
    for (int j = 0; j < NP / 2; ++j) {
      const double2 v = __ldg(reinterpret_cast<const double2*>(p) + j);
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

// Shared-memory-staged SpMM over the rows [r0, r1) of one chunk: tiles of
// kPcgThreads rows; the tile's contiguous slice of values and column indices
// is first copied into shared memory with coalesced loads (every thread keeps
// several independent loads in flight), then each thread forms one row,
// gathering the NP-wide rows of Xin.  Tiles longer than the staging buffer
// read the matrix directly.  With DOT, dacc[q] += Wdot(row, q) * Y(row, q).
template <typename V, int NP, bool DOT>
__device__ __forceinline__ void chunk_spmm(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                           const V* __restrict__ val, const V* __restrict__ Xin,
                                           V* __restrict__ Y, const V* __restrict__ Wdot, int r0, int r1,
                                           V* __restrict__ sval, int32_t* __restrict__ sidx,
                                           double (&dacc)[NP]) {
  const int t = threadIdx.x;
  for (int tr0 = r0; tr0 < r1; tr0 += kPcgThreads) {
    const int tr1 = min(tr0 + kPcgThreads, r1);
    const int32_t k0 = ptr[tr0], k1 = ptr[tr1];
    const bool staged = (k1 - k0) <= kStageCap;
    __syncthreads();  // the previous tile is done with the staging buffer
    if (staged) {
      for (int32_t e = t; e < k1 - k0; e += kPcgThreads) {
        sval[e] = val[k0 + e];
        sidx[e] = idx[k0 + e];
      }
    }
    __syncthreads();
    const int row = tr0 + t;
    if (row < tr1) {
      const int32_t kb = ptr[row], ke = ptr[row + 1];
      V acc[NP];
#pragma unroll
      for (int q = 0; q < NP; ++q) acc[q] = V(0);
#pragma unroll 4
      for (int32_t k = kb; k < ke; ++k) {
        const V a = staged ? sval[k - k0] : val[k];
        const int32_t c = staged ? sidx[k - k0] : idx[k];
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
        for (int q = 0; q < NP; ++q) dacc[q] += (double)(w[q] * acc[q]);
      }
    }
  }
}

template <typename V, int NP, int PC>
__global__ void __launch_bounds__(kPcgThreads) pcg_kernel(PcgArgs<V> a) {
  __shared__ PcgShared<NP> sh;
  extern __shared__ __align__(16) unsigned char stage_raw[];
  V* sval = reinterpret_cast<V*>(stage_raw);
  int32_t* sidx = reinterpret_cast<int32_t*>(stage_raw + sizeof(V) * kStageCap);
  const int t = threadIdx.x;
  // Chunks are dealt round-robin: every CTA holds pieces of many segments,
  // so the work stays balanced while segments converge at different times.
  const int c_begin = blockIdx.x, c_step = gridDim.x;
  const int c_end = a.nchunk;
  double* part_pq = a.part;
  double* part_rz = a.part + (int64_t)a.nchunk * NP;
  double* part_rr = a.part + 2 * (int64_t)a.nchunk * NP;
  const int colt = t % NP;  // fixed column of this thread in element-wise loops
  constexpr int U = 4;      // element-wise unroll: U independent streams per thread

  // ---- phase 0: X = 0, R = B, Z = M^-1 R, P = Z; partial b'b and r'z
  for (int c = c_begin; c < c_end; c += c_step) {
    const int64_t e0 = (int64_t)a.chunk_row[c] * NP, e1 = (int64_t)a.chunk_row[c + 1] * NP;
    double bb = 0.0, rz = 0.0;
    for (int64_t i = e0 + t; i < e1; i += kPcgThreads) {
      const V b = a.B[i];
      a.X[i] = V(0);
      a.R[i] = b;
      bb += (double)b * (double)b;
      if (PC == kPrecJacobi) {
        const V z = a.pc.dinv[i / NP] * b;
        a.P[i] = z;
        rz += (double)b * (double)z;
      }
    }
    cta_partial_store<NP>(bb, sh, part_rr + (int64_t)c * NP);
    if (PC == kPrecJacobi) cta_partial_store<NP>(rz, sh, part_rz + (int64_t)c * NP);
  }
  if (PC == kPrecFactored) {
    if (!grid_sync(a.bar)) return;
    double dummy[NP];
    for (int c = c_begin; c < c_end; c += c_step)
      chunk_spmm<V, NP, false>(a.pc.g_ptr, a.pc.g_idx, a.pc.g_val, a.R, a.T, nullptr, a.chunk_row[c],
                               a.chunk_row[c + 1], sval, sidx, dummy);
    if (!grid_sync(a.bar)) return;
    for (int c = c_begin; c < c_end; c += c_step) {
      double acc[NP];
#pragma unroll
      for (int j = 0; j < NP; ++j) acc[j] = 0.0;
      chunk_spmm<V, NP, true>(a.pc.gt_ptr, a.pc.gt_idx, a.pc.gt_val, a.T, a.Z, a.R, a.chunk_row[c],
                              a.chunk_row[c + 1], sval, sidx, acc);
      cta_rows_partial_store<NP>(acc, sh, part_rz + (int64_t)c * NP);
    }
    if (!grid_sync(a.bar)) return;
    for (int c = c_begin; c < c_end; c += c_step) {
      const int64_t e0 = (int64_t)a.chunk_row[c] * NP, e1 = (int64_t)a.chunk_row[c + 1] * NP;
      for (int64_t i = e0 + t; i < e1; i += kPcgThreads) a.P[i] = a.Z[i];
    }
  }
  if (!grid_sync(a.bar)) return;
  // ---- segment initialisation (first chunk of each segment publishes)
  for (int c = c_begin; c < c_end; c += c_step) {
    const int s = a.chunk_seg[c];
    if (a.seg_chunk[s] != c) continue;
    seg_reduce<NP>(part_rr, a.seg_chunk[s], a.seg_chunk[s + 1], sh, sh.s0);
    seg_reduce<NP>(part_rz, a.seg_chunk[s], a.seg_chunk[s + 1], sh, sh.s1);
    if (t < NP) {
      const double bb = sh.s0[t], rz = sh.s1[t];
      int32_t st;
      if (!isfinite(bb) || !isfinite(rz)) st = LAPY_ERR_NAN;
      else if (bb == 0.0) st = 0;
      else if (!(rz > 0.0)) st = LAPY_ERR_BREAKDOWN;
      else st = kActive;
      a.bb[s * NP + t] = bb;
      a.rz[s * NP + t] = rz;
      a.state[s * NP + t] = st;
      if (st == kActive) atomicAdd(&a.active[0], 1u);
    }
    __syncthreads();
  }
  if (!grid_sync(a.bar)) return;

  int it = 0;
  for (;; ++it) {
    const int par = it & 1;
    const int32_t* st_cur = a.state + par * (int64_t)a.nseg * NP;
    int32_t* st_nxt = a.state + (par ^ 1) * (int64_t)a.nseg * NP;
    const double* rz_cur = a.rz + par * (int64_t)a.nseg * NP;
    double* rz_nxt = a.rz + (par ^ 1) * (int64_t)a.nseg * NP;
    const unsigned nact = *((volatile unsigned*)&a.active[par]);
    if (nact == 0 || it >= a.maxiter) break;

    // ---- phase A: Q = K P, partial p'q
    if (blockIdx.x == 0 && t == 0) a.active[par ^ 1] = 0u;
    if (t == 0) sh.seg = -1;
    __syncthreads();
    for (int c = c_begin; c < c_end; c += c_step) {
      const int s = a.chunk_seg[c];
      if (s != sh.seg) {
        __syncthreads();
        if (t == 0) {
          int any = 0;
          for (int q = 0; q < NP; ++q) any |= (st_cur[s * NP + q] == kActive);
          sh.any = any;
          sh.seg = s;
        }
        __syncthreads();
      }
      if (!sh.any) {
        if (t < NP) part_pq[(int64_t)c * NP + t] = 0.0;
        continue;
      }
      double acc[NP];
#pragma unroll
      for (int j = 0; j < NP; ++j) acc[j] = 0.0;
      chunk_spmm<V, NP, true>(a.indptr, a.indices, a.vals, a.P, a.Q, a.P, a.chunk_row[c], a.chunk_row[c + 1],
                              sval, sidx, acc);
      cta_rows_partial_store<NP>(acc, sh, part_pq + (int64_t)c * NP);
      if (t == 0) {
        const int r0 = a.chunk_row[c], r1 = a.chunk_row[c + 1];
        atomicAdd(&a.work[0], (unsigned long long)(r1 - r0));
        atomicAdd(&a.work[1], (unsigned long long)(a.indptr[r1] - a.indptr[r0]));
      }
    }
    if (!grid_sync(a.bar)) return;

    // ---- phase B: alpha, X += alpha P, R -= alpha Q, partial r'r (and r'z for Jacobi)
    if (t == 0) sh.seg = -1;
    __syncthreads();
    for (int c = c_begin; c < c_end; c += c_step) {
      const int s = a.chunk_seg[c];
      if (s != sh.seg) {
        seg_reduce<NP>(part_pq, a.seg_chunk[s], a.seg_chunk[s + 1], sh, sh.s0);
        if (t < NP) {
          const double pq = sh.s0[t];
          const bool act = st_cur[s * NP + t] == kActive;
          const bool ok = act && pq > 0.0 && isfinite(pq);
          sh.scal[t] = ok ? rz_cur[s * NP + t] / pq : 0.0;
          sh.act[t] = ok;
        }
        if (t == 0) sh.seg = s;
        __syncthreads();
        if (t == 0) {
          int any = 0;
          for (int q = 0; q < NP; ++q) any |= sh.act[q];
          sh.any = any;
        }
        __syncthreads();
      }
      const int64_t e0 = (int64_t)a.chunk_row[c] * NP, e1 = (int64_t)a.chunk_row[c + 1] * NP;
      if (!sh.any) {
        if (t < NP) {
          part_rr[(int64_t)c * NP + t] = 0.0;
          part_rz[(int64_t)c * NP + t] = 0.0;
        }
        continue;
      }
      const V alpha = (V)sh.scal[colt];
      const bool act = sh.act[colt];
      float rr = 0.f, rz = 0.f;
      for (int64_t i0 = e0 + t; i0 < e1; i0 += U * kPcgThreads) {
        V xv[U], pv[U], qv[U], rv[U], dv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = i0 + u * kPcgThreads;
          if (i < e1) {
            rv[u] = a.R[i];
            if (act) { xv[u] = a.X[i]; pv[u] = a.P[i]; qv[u] = a.Q[i]; }
            if (PC == kPrecJacobi) dv[u] = a.pc.dinv[i / NP];
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int64_t i = i0 + u * kPcgThreads;
          if (i < e1) {
            V r = rv[u];
            if (act) {
              a.X[i] = xv[u] + alpha * pv[u];
              r = r - alpha * qv[u];
              a.R[i] = r;
            }
            rr += (float)(r * r);
            if (PC == kPrecJacobi) rz += (float)(r * (dv[u] * r));
          }
        }
      }
      cta_partial_store<NP>((double)rr, sh, part_rr + (int64_t)c * NP);
      if (PC == kPrecJacobi) cta_partial_store<NP>((double)rz, sh, part_rz + (int64_t)c * NP);
    }
    if (!grid_sync(a.bar)) return;

    if (PC == kPrecFactored) {
      // ---- phase B2: T = G R ; phase B3: Z = Gt T, partial r'z
      double dummy[NP];
      for (int c = c_begin; c < c_end; c += c_step)
        chunk_spmm<V, NP, false>(a.pc.g_ptr, a.pc.g_idx, a.pc.g_val, a.R, a.T, nullptr, a.chunk_row[c],
                                 a.chunk_row[c + 1], sval, sidx, dummy);
      if (!grid_sync(a.bar)) return;
      for (int c = c_begin; c < c_end; c += c_step) {
        double acc[NP];
#pragma unroll
        for (int j = 0; j < NP; ++j) acc[j] = 0.0;
        chunk_spmm<V, NP, true>(a.pc.gt_ptr, a.pc.gt_idx, a.pc.gt_val, a.T, a.Z, a.R, a.chunk_row[c],
                                a.chunk_row[c + 1], sval, sidx, acc);
        cta_rows_partial_store<NP>(acc, sh, part_rz + (int64_t)c * NP);
      }
      if (!grid_sync(a.bar)) return;
    }

    // ---- phase C: convergence, beta, P = Z + beta P
    if (t == 0) sh.seg = -1;
    __syncthreads();
    for (int c = c_begin; c < c_end; c += c_step) {
      const int s = a.chunk_seg[c];
      if (s != sh.seg) {
        seg_reduce<NP>(part_pq, a.seg_chunk[s], a.seg_chunk[s + 1], sh, sh.s0);
        seg_reduce<NP>(part_rz, a.seg_chunk[s], a.seg_chunk[s + 1], sh, sh.s1);
        seg_reduce<NP>(part_rr, a.seg_chunk[s], a.seg_chunk[s + 1], sh, sh.s2);
        if (t < NP) {
          const int32_t st0 = st_cur[s * NP + t];
          const double pq = sh.s0[t], rzn = sh.s1[t], rr = sh.s2[t];
          int32_t st = st0;
          if (st0 == kActive) {
            if (!(pq > 0.0) || !isfinite(pq)) st = LAPY_ERR_BREAKDOWN;
            else if (!isfinite(rr) || !isfinite(rzn)) st = LAPY_ERR_NAN;
            else if (rr <= a.rtol2 * a.bb[s * NP + t]) st = it + 1;
            else if (!(rzn > 0.0)) st = LAPY_ERR_BREAKDOWN;
          }
          const bool act = st == kActive;
          sh.scal[t] = act ? rzn / rz_cur[s * NP + t] : 0.0;
          sh.act[t] = act;
          if (a.seg_chunk[s] == c) {  // a segment's first chunk always starts a new run
            st_nxt[s * NP + t] = st;
            rz_nxt[s * NP + t] = rzn;
            if (act) atomicAdd(&a.active[par ^ 1], 1u);
          }
        }
        if (t == 0) sh.seg = s;
        __syncthreads();
        if (t == 0) {
          int any = 0;
          for (int q = 0; q < NP; ++q) any |= sh.act[q];
          sh.any = any;
        }
        __syncthreads();
      }
      if (!sh.any) continue;
      const int64_t e0 = (int64_t)a.chunk_row[c] * NP, e1 = (int64_t)a.chunk_row[c + 1] * NP;
      const V beta = (V)sh.scal[colt];
      if (sh.act[colt]) {
        for (int64_t i0 = e0 + t; i0 < e1; i0 += U * kPcgThreads) {
          V zv[U], pv[U];
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int64_t i = i0 + u * kPcgThreads;
            if (i < e1) {
              zv[u] = (PC == kPrecJacobi) ? a.pc.dinv[i / NP] * a.R[i] : a.Z[i];
              pv[u] = a.P[i];
            }
          }
#pragma unroll
          for (int u = 0; u < U; ++u) {
            const int64_t i = i0 + u * kPcgThreads;
            if (i < e1) a.P[i] = zv[u] + beta * pv[u];
          }
        }
      }
    }
    if (!grid_sync(a.bar)) return;
  }

  // ---- publish the final state (first chunk of each segment)
  const int par = it & 1;
  const int32_t* st_cur = a.state + par * (int64_t)a.nseg * NP;
  for (int c = c_begin; c < c_end; c += c_step) {
    const int s = a.chunk_seg[c];
    if (a.seg_chunk[s] != c) continue;
    if (t < NP) {
      int32_t st = st_cur[s * NP + t];
      if (st == kActive) st = LAPY_ERR_NOCONV;
      a.state_out[s * NP + t] = st;
    }
  }
  if (blockIdx.x == 0 && t == 0) a.iters[0] = it;
}

size_t pcg_workspace_bytes(int64_t n, int p, int nseg, int nchunk, int elem_size, int precond) {
  const size_t vec = a256((size_t)n * p * elem_size);
  size_t b = vec * (precond == kPrecFactored ? 5 : 3);  // R P Q (+ Z T)
  b += a256(sizeof(double) * 3 * (size_t)nchunk * p);
  b += a256(sizeof(double) * 2 * (size_t)nseg * p);
  b += a256(sizeof(double) * (size_t)nseg * p);
  b += a256(sizeof(int32_t) * 2 * (size_t)nseg * p);
  b += a256(64);  // active[2], iters, barrier, work counters
  return b + 256;
}

template <typename V, int NP, int PC>
static int launch_pcg(PcgArgs<V>& args, cudaStream_t stream) {
  auto kern = pcg_kernel<V, NP, PC>;
  const size_t smem = (sizeof(V) + sizeof(int32_t)) * kStageCap;
  int per_sm = 0;
  LAPY_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPcgThreads, smem));
  if (per_sm <= 0) {
    lapy_set_last_message("pcg: kernel cannot be resident (occupancy 0)");
    return LAPY_ERR_CUDA;
  }
  const int grid = std::max(1, std::min(per_sm * lapy_num_sms(), args.nchunk));
  void* kargs[] = {(void*)&args};
  LAPY_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kPcgThreads), kargs, smem, stream));
  return lapy_check_launch("pcg_kernel");
}

template <typename V, int PC>
static int launch_pcg_np(PcgArgs<V>& args, int p, cudaStream_t stream) {
  switch (p) {
    case 1: return launch_pcg<V, 1, PC>(args, stream);
    case 2: return launch_pcg<V, 2, PC>(args, stream);
    case 4: return launch_pcg<V, 4, PC>(args, stream);
    case 8: return launch_pcg<V, 8, PC>(args, stream);
    case 16: return launch_pcg<V, 16, PC>(args, stream);
    default:
      lapy_set_last_message("pcg: block width %d not in {1,2,4,8,16}", p);
      return LAPY_ERR_INVALID;
  }
}

template <typename V>
int pcg_solve(int64_t n, const int32_t* indptr, const int32_t* indices, const V* vals,
              const PcgPrecondDesc<V>& pc, int p, const ChunkTable& ct, const V* B, V* X,
              double rtol, int maxiter, int32_t* state_dev, void* ws, size_t ws_bytes,
              cudaStream_t stream, int* iters_out) {
  if (ws_bytes < pcg_workspace_bytes(n, p, ct.nseg, ct.nchunk, sizeof(V), pc.kind))
    return LAPY_ERR_WORKSPACE;
  char* w = (char*)(((uintptr_t)ws + 255) & ~uintptr_t(255));
  const size_t vec = a256((size_t)n * p * sizeof(V));
  PcgArgs<V> a;
  a.n = n;
  a.indptr = indptr;
  a.indices = indices;
  a.vals = vals;
  a.pc = pc;
  a.chunk_row = ct.chunk_row;
  a.chunk_seg = ct.chunk_seg;
  a.seg_chunk = ct.seg_chunk;
  a.nchunk = ct.nchunk;
  a.nseg = ct.nseg;
  a.B = B;
  a.X = X;
  a.R = (V*)w; w += vec;
  a.P = (V*)w; w += vec;
  a.Q = (V*)w; w += vec;
  a.Z = nullptr;
  a.T = nullptr;
  if (pc.kind == kPrecFactored) {
    a.Z = (V*)w; w += vec;
    a.T = (V*)w; w += vec;
  }
  a.part = (double*)w; w += a256(sizeof(double) * 3 * (size_t)ct.nchunk * p);
  a.rz = (double*)w; w += a256(sizeof(double) * 2 * (size_t)ct.nseg * p);
  a.bb = (double*)w; w += a256(sizeof(double) * (size_t)ct.nseg * p);
  a.state = (int32_t*)w; w += a256(sizeof(int32_t) * 2 * (size_t)ct.nseg * p);
  unsigned* ctl = (unsigned*)w;  // active[2], iters, count, gen, err
  a.active = ctl;
  a.iters = (int*)(ctl + 2);
  a.bar.count = ctl + 3;
  a.bar.gen = ctl + 4;
  a.bar.err = (int*)(ctl + 5);
  a.work = (unsigned long long*)(ctl + 6);
  a.state_out = state_dev;
  a.rtol2 = rtol * rtol;
  a.maxiter = maxiter;
  LAPY_CUDA_TRY(cudaMemsetAsync(ctl, 0, 64, stream));
  int st;
  const bool prof = lapy_profile_enabled();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (prof) {
    LAPY_CUDA_TRY(cudaEventCreate(&e0));
    LAPY_CUDA_TRY(cudaEventCreate(&e1));
    LAPY_CUDA_TRY(cudaEventRecord(e0, stream));
  }
  if (pc.kind == kPrecFactored)
    st = launch_pcg_np<V, kPrecFactored>(a, p, stream);
  else
    st = launch_pcg_np<V, kPrecJacobi>(a, p, stream);
  if (st != LAPY_OK) return st;
  if (prof) LAPY_CUDA_TRY(cudaEventRecord(e1, stream));
  unsigned hctl[10];
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
    lapy_profile_add_pcg(ms, (long long)hctl[2], (long long)rows, (long long)nnz, p, (int)sizeof(V));
  }
  if (hctl[5] != 0) {
    lapy_set_last_message("pcg: grid barrier timed out");
    return LAPY_ERR_TIMEOUT;
  }
  if (iters_out) *iters_out = (int)hctl[2];
  return LAPY_OK;
}

template int pcg_solve<float>(int64_t, const int32_t*, const int32_t*, const float*,
                              const PcgPrecondDesc<float>&, int, const ChunkTable&, const float*,
                              float*, double, int, int32_t*, void*, size_t, cudaStream_t, int*);
template int pcg_solve<double>(int64_t, const int32_t*, const int32_t*, const double*,
                               const PcgPrecondDesc<double>&, int, const ChunkTable&, const double*,
                               double*, double, int, int32_t*, void*, size_t, cudaStream_t, int*);

}  // namespace lapy
