// Learned factorised sparse approximate inverse (per-edge MLP).
//
// For an SPD system K on a symmetric mesh pattern, G is lower triangular on
// the pattern's lower part.  A per-edge network (6 -> 64 -> 64 -> 1, tanh,
// BF16 weights, FP32 accumulation; the forward pass's 64 x 64 layer on the
// tensor pipe) emits w_ij for every strictly lower entry;
// row i then gets
//   q_i = (e_i - w_i)' K (e_i - w_i),  G_ii = q_i^-1/2,  G_ij = -w_ij G_ii,
// so diag(G K G') = 1 and G'G is SPD for every w (w = 0 is Jacobi).  The
// training loss sum_i log q_i is the Kaporin functional of G K G' (its exact
// minimiser is FSAI); dL/dw_ij = (-2 K_ij + 2 sum_k w_ik K_jk) / q_i.
//
// Lower pattern: rows' entries with col <= row in CSR order (diagonal last);
// upper pattern: col >= row (diagonal first), with umap[u] the lower index of
// the transposed entry, so G' values are a gather of G's.
#include <cmath>
#include <cuda_bf16.h>
#include "common.cuh"
#include "scan.cuh"

namespace lapy {

constexpr int kNF = 6, kHid = 64;
constexpr int kOW1 = 0, kOB1 = kOW1 + kHid * kNF, kOW2 = kOB1 + kHid, kOB2 = kOW2 + kHid * kHid,
              kOW3 = kOB2 + kHid, kOB3 = kOW3 + kHid, kNParam = kOB3 + 1;
static_assert(kNParam == 4673, "parameter layout");

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// ---- pattern ---------------------------------------------------------------
__global__ void spai_count_kernel(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                  int32_t* __restrict__ lcnt, int32_t* __restrict__ ucnt) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t l = 0, u = 0;
  for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
    const int32_t c = indices[k];
    l += c <= i;
    u += c >= i;
  }
  lcnt[i] = l;
  ucnt[i] = u;
}

__global__ void spai_fill_kernel(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                 const int32_t* __restrict__ lptr, const int32_t* __restrict__ uptr,
                                 int32_t* __restrict__ lcol, int32_t* __restrict__ lpos, int32_t* __restrict__ ucol) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t l = lptr[i], u = uptr[i];
  for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
    const int32_t c = indices[k];
    if (c <= i) { lcol[l] = c; lpos[l] = k; ++l; }
    if (c >= i) { ucol[u] = c; ++u; }
  }
}

__global__ void spai_umap_kernel(int64_t n, const int32_t* __restrict__ uptr, const int32_t* __restrict__ ucol,
                                 const int32_t* __restrict__ lptr, const int32_t* __restrict__ lcol,
                                 int32_t* __restrict__ umap, int* __restrict__ missing) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  for (int32_t u = uptr[j]; u < uptr[j + 1]; ++u) {
    const int32_t i = ucol[u];  // entry (j, i), i >= j: the lower entry (i, j)
    int32_t lo = lptr[i], hi = lptr[i + 1] - 1, found = -1;
    while (lo <= hi) {
      const int32_t mid = (lo + hi) >> 1;
      const int32_t c = lcol[mid];
      if (c == (int32_t)j) { found = mid; break; }
      if (c < (int32_t)j) lo = mid + 1; else hi = mid - 1;
    }
    umap[u] = found;
    if (found < 0) atomicExch(missing, 1);
  }
}

// ---- features --------------------------------------------------------------
__global__ void spai_mass_kernel(int64_t n, const int32_t* __restrict__ indptr, const double* __restrict__ m_vals,
                                 int m_is_diag, double* __restrict__ mass) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (m_is_diag) {
    mass[i] = m_vals[i];
  } else {
    double s = 0.0;
    for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) s += m_vals[k];
    mass[i] = s;
  }
}

__device__ __forceinline__ int seg_of_row(const int32_t* __restrict__ seg_row, int nseg, int64_t i) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg_row[mid] <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <typename T>
__global__ void spai_features_kernel(int64_t n, int nseg, const int32_t* __restrict__ seg_row, const T* __restrict__ v,
                                     const double* __restrict__ a_vals, const double* __restrict__ mass,
                                     const int32_t* __restrict__ lptr, const int32_t* __restrict__ lcol,
                                     const int32_t* __restrict__ lpos, const double* __restrict__ t_seg,
                                     const double* __restrict__ sigma_seg, const double* __restrict__ h_seg,
                                     float* __restrict__ feat) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = seg_of_row(seg_row, nseg, i);
  const double h = h_seg[s], h2 = h * h;
  const float f4 = (float)log(t_seg[s] / h2), f5 = (float)sigma_seg[s];
  const double mi = mass[i] / h2;
  const double xi = (double)v[3 * i], yi = (double)v[3 * i + 1], zi = (double)v[3 * i + 2];
  for (int32_t e = lptr[i]; e < lptr[i + 1]; ++e) {
    const int32_t j = lcol[e];
    const double dx = xi - (double)v[3 * (int64_t)j], dy = yi - (double)v[3 * (int64_t)j + 1],
                 dz = zi - (double)v[3 * (int64_t)j + 2];
    float* f = feat + (int64_t)e * kNF;
    f[0] = (float)(-a_vals[lpos[e]]);
    f[1] = (float)(sqrt(dx * dx + dy * dy + dz * dz) / h);
    f[2] = (float)mi;
    f[3] = (float)(mass[j] / h2);
    f[4] = f4;
    f[5] = f5;
  }
}

// ---- network ---------------------------------------------------------------
struct SpaiWeights {
  float W1[kHid * kNF], b1[kHid], W2[kHid * kHid], b2[kHid], W3[kHid], b3;
};

__device__ __forceinline__ void load_weights(const __nv_bfloat16* __restrict__ wb, SpaiWeights& s) {
  float* dst = s.W1;  // the struct is the parameter layout, contiguous
  for (int p = threadIdx.x; p < kNParam; p += blockDim.x) dst[p] = __bfloat162float(wb[p]);
}

// Hidden layer 1 of one edge.
__device__ __forceinline__ void layer1(const SpaiWeights& s, const float (&f)[kNF], float (&h1)[kHid]) {
#pragma unroll 4
  for (int o = 0; o < kHid; ++o) {
    float a = s.b1[o];
#pragma unroll
    for (int k = 0; k < kNF; ++k) a = fmaf(s.W1[o * kNF + k], f[k], a);
    h1[o] = tanhf(a);
  }
}

// Pre-activation of hidden unit o of layer 2.
__device__ __forceinline__ float layer2_unit(const SpaiWeights& s, const float (&h1)[kHid], int o) {
  const float4* w = reinterpret_cast<const float4*>(s.W2 + o * kHid);
  float a0 = s.b2[o], a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
  for (int k = 0; k < kHid / 4; ++k) {
    const float4 wv = w[k];
    a0 = fmaf(wv.x, h1[4 * k], a0);
    a1 = fmaf(wv.y, h1[4 * k + 1], a1);
    a2 = fmaf(wv.z, h1[4 * k + 2], a2);
    a3 = fmaf(wv.w, h1[4 * k + 3], a3);
  }
  return (a0 + a1) + (a2 + a3);
}

// ---- network on the tensor pipe ---------------------------------------------
// Forward pass with warp-level BF16 matrix instructions
// (mma.sync.m16n8k16, FP32 accumulate): a warp takes 16 edges at a time.
// Layer 1 (6 -> 64) runs on the FP32 pipe, each lane computing exactly the
// hidden units its A fragments hold (rows lane/4 and lane/4 + 8, units
// 16t + 2(lane%4) + {0,1} and + 8 of every 16-unit step t), so no shuffles
// are needed.  Layer 2 (64 x 64, 90 % of the work) is 32 tiles of 16 x 8 x 16
// per 16 edges; its input is split into three BF16 terms (hi + mid + lo,
// about 24 bits) so that the product with the BF16 weights keeps the FP32
// path's accuracy.  Layer 3 (64 -> 1) is folded into the epilogue of each
// 8-unit output tile, and the four lanes of a row sum their parts.
constexpr int kMmaWarps = 4;
constexpr int kW2Ld = kHid + 8;  // padded row of the staged W2 (BF16): conflict-free B-fragment loads

struct SpaiMmaSmem {
  __nv_bfloat16 W2[kHid * kW2Ld];
  float W1[kHid * kNF], b1[kHid], b2[kHid], W3[kHid], b3;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const uint32_t l = __bfloat16_as_ushort(__float2bfloat16_rn(lo));
  const uint32_t h = __bfloat16_as_ushort(__float2bfloat16_rn(hi));
  return l | (h << 16);
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(32 * kMmaWarps) spai_forward_mma_kernel(int64_t ne, const float* __restrict__ feat,
                                                                          const __nv_bfloat16* __restrict__ wb,
                                                                          float* __restrict__ out) {
  __shared__ __align__(16) SpaiMmaSmem s;
  for (int p = threadIdx.x; p < kHid * kHid; p += blockDim.x) s.W2[(p / kHid) * kW2Ld + p % kHid] = wb[kOW2 + p];
  for (int p = threadIdx.x; p < kHid * kNF; p += blockDim.x) s.W1[p] = __bfloat162float(wb[kOW1 + p]);
  for (int p = threadIdx.x; p < kHid; p += blockDim.x) {
    s.b1[p] = __bfloat162float(wb[kOB1 + p]);
    s.b2[p] = __bfloat162float(wb[kOB2 + p]);
    s.W3[p] = __bfloat162float(wb[kOW3 + p]);
  }
  if (threadIdx.x == 0) s.b3 = __bfloat162float(wb[kOB3]);
  __syncthreads();
  const int lane = threadIdx.x & 31, grp = lane >> 2, tig = lane & 3;
  const int64_t warp0 = (int64_t)blockIdx.x * kMmaWarps + (threadIdx.x >> 5);
  const int64_t nwarp = (int64_t)gridDim.x * kMmaWarps;
  const uint32_t* W2w = reinterpret_cast<const uint32_t*>(s.W2);  // two BF16 per word
  for (int64_t tile = warp0; tile * 16 < ne; tile += nwarp) {
    const int64_t e0 = tile * 16 + grp, e1 = e0 + 8;
    float f0[kNF], f1[kNF];
#pragma unroll
    for (int k = 0; k < kNF; ++k) {
      f0[k] = e0 < ne ? feat[e0 * kNF + k] : 0.f;
      f1[k] = e1 < ne ? feat[e1 * kNF + k] : 0.f;
    }
    // layer 1 for this lane's fragment units; A fragments of layer 2 in
    // three BF16 terms
    uint32_t ahi[4][4], amid[4][4], alo[4][4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
#pragma unroll
      for (int half = 0; half < 2; ++half) {  // units 16t + 8 half + 2 tig + {0, 1}
        const int u = 16 * t + 8 * half + 2 * tig;
        float h[2][2];  // [row 0/8][unit u/u+1]
#pragma unroll
        for (int du = 0; du < 2; ++du) {
          float a0 = s.b1[u + du], a1 = s.b1[u + du];
#pragma unroll
          for (int k = 0; k < kNF; ++k) {
            a0 = fmaf(s.W1[(u + du) * kNF + k], f0[k], a0);
            a1 = fmaf(s.W1[(u + du) * kNF + k], f1[k], a1);
          }
          h[0][du] = tanhf(a0);
          h[1][du] = tanhf(a1);
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const int reg = 2 * half + r;  // a0: (row, k), a1: (row + 8, k), a2: (row, k + 8), a3: (row + 8, k + 8)
          float x0 = h[r][0], x1 = h[r][1];
          const float hi0 = __bfloat162float(__float2bfloat16_rn(x0)), hi1 = __bfloat162float(__float2bfloat16_rn(x1));
          ahi[t][reg] = pack_bf16x2(x0, x1);
          x0 -= hi0;
          x1 -= hi1;
          const float mi0 = __bfloat162float(__float2bfloat16_rn(x0)), mi1 = __bfloat162float(__float2bfloat16_rn(x1));
          amid[t][reg] = pack_bf16x2(x0, x1);
          alo[t][reg] = pack_bf16x2(x0 - mi0, x1 - mi1);
        }
      }
    }
    float part0 = 0.f, part1 = 0.f;  // layer-3 partial sums of rows grp and grp + 8
#pragma unroll 2
    for (int j = 0; j < kHid / 8; ++j) {  // output units 8j .. 8j + 7
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      const int n = 8 * j + grp;  // B column = W2 row
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const uint32_t b0 = W2w[(n * kW2Ld + 16 * t + 2 * tig) >> 1];
        const uint32_t b1 = W2w[(n * kW2Ld + 16 * t + 8 + 2 * tig) >> 1];
        mma_bf16_16816(acc, alo[t], b0, b1);
        mma_bf16_16816(acc, amid[t], b0, b1);
        mma_bf16_16816(acc, ahi[t], b0, b1);
      }
      const int o = 8 * j + 2 * tig;
      part0 = fmaf(s.W3[o], tanhf(acc[0] + s.b2[o]), part0);
      part0 = fmaf(s.W3[o + 1], tanhf(acc[1] + s.b2[o + 1]), part0);
      part1 = fmaf(s.W3[o], tanhf(acc[2] + s.b2[o]), part1);
      part1 = fmaf(s.W3[o + 1], tanhf(acc[3] + s.b2[o + 1]), part1);
    }
    part0 += __shfl_xor_sync(0xffffffffu, part0, 1);
    part0 += __shfl_xor_sync(0xffffffffu, part0, 2);
    part1 += __shfl_xor_sync(0xffffffffu, part1, 1);
    part1 += __shfl_xor_sync(0xffffffffu, part1, 2);
    if (tig == 0) {
      if (e0 < ne) out[e0] = s.b3 + part0;
      if (e1 < ne) out[e1] = s.b3 + part1;
    }
  }
}

// ---- factor, loss and dL/dw ------------------------------------------------
__device__ __forceinline__ double k_at(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                       const double* __restrict__ kv, int32_t row, int32_t col) {
  int32_t lo = indptr[row], hi = indptr[row + 1] - 1;
  while (lo <= hi) {
    const int32_t mid = (lo + hi) >> 1;
    const int32_t c = indices[mid];
    if (c == col) return kv[mid];
    if (c < col) lo = mid + 1; else hi = mid - 1;
  }
  return 0.0;
}

__global__ void spai_factor_kernel(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                   const double* __restrict__ kv, const int32_t* __restrict__ lptr,
                                   const int32_t* __restrict__ lcol, const int32_t* __restrict__ lpos,
                                   const float* __restrict__ w, float* __restrict__ g, double* __restrict__ logq,
                                   float* __restrict__ dldw) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t e0 = lptr[i], ed = lptr[i + 1] - 1;  // ed: the diagonal entry
  const double kii = kv[lpos[ed]];
  double q = kii;
  for (int32_t e = e0; e < ed; ++e) {
    const double we = w[e];
    q -= 2.0 * we * kv[lpos[e]];
    for (int32_t f = e0; f < ed; ++f) q += we * (double)w[f] * k_at(indptr, indices, kv, lcol[e], lcol[f]);
  }
  const bool ok = q > 0.0 && isfinite(q);
  if (!ok) q = kii;  // the Jacobi row
  const double gd = 1.0 / sqrt(q);
  g[ed] = (float)gd;
  if (logq) logq[i] = log(q);
  if (dldw) dldw[ed] = 0.f;
  for (int32_t e = e0; e < ed; ++e) {
    g[e] = ok ? (float)(-(double)w[e] * gd) : 0.f;
    if (dldw) {
      double dq = -2.0 * kv[lpos[e]];
      for (int32_t f = e0; f < ed; ++f) dq += 2.0 * (double)w[f] * k_at(indptr, indices, kv, lcol[e], lcol[f]);
      dldw[e] = ok ? (float)(dq / q) : 0.f;
    }
  }
}

__global__ void spai_gather_kernel(int64_t m, const int32_t* __restrict__ umap, const float* __restrict__ gl,
                                   float* __restrict__ gu) {
  const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (u < m) gu[u] = gl[umap[u]];
}

// ---- backward --------------------------------------------------------------
// One CTA of kBwdThreads threads walks tiles of kBwdThreads edges: every
// thread recomputes its edge's activations and back-propagates dL/dw into
// shared-memory tiles (h1, dz1, dz2, d3 * h2); then the CTA accumulates the
// parameter gradient of the tile (each thread owns a fixed set of parameters,
// summed over the tile's edges in order) and finally writes its partial.
constexpr int kBwdThreads = 128;
constexpr int kParamsPerThread = (kNParam + kBwdThreads - 1) / kBwdThreads;

struct BwdTile {  // rows padded by one word: no bank conflicts on per-thread rows
  float h1[kBwdThreads][kHid + 1];
  float dz1[kBwdThreads][kHid + 1];
  float dz2[kBwdThreads][kHid + 1];
  float g3[kBwdThreads][kHid + 1];
  float f[kBwdThreads][kNF];
  float d3[kBwdThreads];
};

__global__ void __launch_bounds__(kBwdThreads) spai_backward_kernel(int64_t ne, const float* __restrict__ feat,
                                                                    const __nv_bfloat16* __restrict__ wb,
                                                                    const float* __restrict__ dw,
                                                                    float* __restrict__ partial) {
  extern __shared__ __align__(16) unsigned char smem[];
  SpaiWeights& s = *reinterpret_cast<SpaiWeights*>(smem);
  BwdTile& t = *reinterpret_cast<BwdTile*>(smem + ((sizeof(SpaiWeights) + 15) & ~size_t(15)));
  load_weights(wb, s);
  float acc[kParamsPerThread];
#pragma unroll
  for (int r = 0; r < kParamsPerThread; ++r) acc[r] = 0.f;
  const int tid = threadIdx.x;
  for (int64_t base = (int64_t)blockIdx.x * kBwdThreads; base < ne; base += (int64_t)gridDim.x * kBwdThreads) {
    __syncthreads();  // weights loaded / previous tile consumed
    const int64_t e = base + tid;
    float f[kNF], h1[kHid];
    float d3 = 0.f;
    if (e < ne) {
#pragma unroll
      for (int k = 0; k < kNF; ++k) f[k] = feat[e * kNF + k];
      d3 = dw[e];
    } else {
#pragma unroll
      for (int k = 0; k < kNF; ++k) f[k] = 0.f;
    }
    layer1(s, f, h1);
    float dh1[kHid];
#pragma unroll
    for (int k = 0; k < kHid; ++k) dh1[k] = 0.f;
#pragma unroll 1
    for (int o = 0; o < kHid; ++o) {
      const float h2 = tanhf(layer2_unit(s, h1, o));
      const float dz2 = d3 * s.W3[o] * (1.f - h2 * h2);
      t.dz2[tid][o] = dz2;
      t.g3[tid][o] = d3 * h2;
      const float4* w = reinterpret_cast<const float4*>(s.W2 + o * kHid);
#pragma unroll
      for (int k = 0; k < kHid / 4; ++k) {
        const float4 wv = w[k];
        dh1[4 * k] = fmaf(dz2, wv.x, dh1[4 * k]);
        dh1[4 * k + 1] = fmaf(dz2, wv.y, dh1[4 * k + 1]);
        dh1[4 * k + 2] = fmaf(dz2, wv.z, dh1[4 * k + 2]);
        dh1[4 * k + 3] = fmaf(dz2, wv.w, dh1[4 * k + 3]);
      }
    }
#pragma unroll
    for (int k = 0; k < kHid; ++k) {
      t.h1[tid][k] = h1[k];
      t.dz1[tid][k] = dh1[k] * (1.f - h1[k] * h1[k]);
    }
#pragma unroll
    for (int k = 0; k < kNF; ++k) t.f[tid][k] = f[k];
    t.d3[tid] = d3;
    __syncthreads();
    const int ntile = (ne - base < kBwdThreads) ? (int)(ne - base) : kBwdThreads;
#pragma unroll
    for (int r = 0; r < kParamsPerThread; ++r) {
      const int p = tid + r * kBwdThreads;
      if (p >= kNParam) break;
      float a = 0.f;
      if (p < kOB1) {  // W1[o][k] += dz1[o] f[k]
        const int o = p / kNF, k = p % kNF;
        for (int x = 0; x < ntile; ++x) a = fmaf(t.dz1[x][o], t.f[x][k], a);
      } else if (p < kOW2) {
        const int o = p - kOB1;
        for (int x = 0; x < ntile; ++x) a += t.dz1[x][o];
      } else if (p < kOB2) {  // W2[o][k] += dz2[o] h1[k]
        const int o = (p - kOW2) / kHid, k = (p - kOW2) % kHid;
        for (int x = 0; x < ntile; ++x) a = fmaf(t.dz2[x][o], t.h1[x][k], a);
      } else if (p < kOW3) {
        const int o = p - kOB2;
        for (int x = 0; x < ntile; ++x) a += t.dz2[x][o];
      } else if (p < kOB3) {
        const int o = p - kOW3;
        for (int x = 0; x < ntile; ++x) a += t.g3[x][o];
      } else {
        for (int x = 0; x < ntile; ++x) a += t.d3[x];
      }
      acc[r] += a;
    }
  }
#pragma unroll
  for (int r = 0; r < kParamsPerThread; ++r) {
    const int p = tid + r * kBwdThreads;
    if (p < kNParam) partial[(int64_t)blockIdx.x * kNParam + p] = acc[r];
  }
}

__global__ void spai_grad_reduce_kernel(int nblk, const float* __restrict__ partial, float scale,
                                        float* __restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kNParam) return;
  float a = 0.f;
  for (int b = 0; b < nblk; ++b) a += partial[(int64_t)b * kNParam + p];
  grad[p] = a * scale;
}

__global__ void spai_adam_kernel(int np, float* __restrict__ theta, const float* __restrict__ grad,
                                 float* __restrict__ m, float* __restrict__ v, __nv_bfloat16* __restrict__ wb,
                                 float lr, float b1, float b2, float eps, float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const float g = grad[p];
  const float mp = b1 * m[p] + (1.f - b1) * g;
  const float vp = b2 * v[p] + (1.f - b2) * g * g;
  m[p] = mp;
  v[p] = vp;
  const float th = theta[p] - lr * (mp / c1) / (sqrtf(vp / c2) + eps);
  theta[p] = th;
  wb[p] = __float2bfloat16_rn(th);
}

__global__ void spai_to_bf16_kernel(int np, const float* __restrict__ theta, __nv_bfloat16* __restrict__ wb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np) wb[p] = __float2bfloat16_rn(theta[p]);
}

static size_t bwd_smem() { return ((sizeof(SpaiWeights) + 15) & ~size_t(15)) + sizeof(BwdTile); }

}  // namespace lapy

using namespace lapy;

extern "C" int lapy_spai_param_count(void) { return kNParam; }

extern "C" size_t lapy_spai_pattern_workspace_bytes(int64_t n) {
  return a256(4 * (size_t)(n + 1)) * 2 + a256(4 * (size_t)scan_scratch_elems(n + 1)) + 512;
}

extern "C" int lapy_spai_pattern(int64_t n, const int32_t* indptr, const int32_t* indices, int64_t nnz,
                                 int32_t* lptr, int32_t* lcol, int32_t* lpos, int32_t* uptr, int32_t* ucol,
                                 int32_t* umap, void* work, size_t ws_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n <= 0 || !indptr || !indices || nnz < n || !lptr || !lcol || !lpos || !uptr || !ucol || !umap || !work)
    return LAPY_ERR_INVALID;
  if ((nnz + n) % 2 != 0) {
    lapy_set_last_message("spai_pattern: the pattern is not symmetric with a full diagonal");
    return LAPY_ERR_PATTERN;
  }
  if (ws_bytes < lapy_spai_pattern_workspace_bytes(n)) return LAPY_ERR_WORKSPACE;
  char* w = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  int32_t* lcnt = (int32_t*)w; w += a256(4 * (size_t)(n + 1));
  int32_t* ucnt = (int32_t*)w; w += a256(4 * (size_t)(n + 1));
  int32_t* scratch = (int32_t*)w; w += a256(4 * (size_t)scan_scratch_elems(n + 1));
  int* missing = (int*)w;
  const unsigned nb = lapy_ceil_div(n, 256);
  spai_count_kernel<<<nb, 256, 0, stream>>>(n, indptr, indices, lcnt, ucnt);
  LAPY_TRY(lapy_check_launch("spai_count_kernel"));
  LAPY_TRY(exclusive_scan_i32(lcnt, lptr, n, scratch, stream));
  LAPY_TRY(exclusive_scan_i32(ucnt, uptr, n, scratch, stream));
  int32_t tot[2] = {0, 0};
  LAPY_CUDA_TRY(cudaMemcpyAsync(&tot[0], lptr + n, 4, cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaMemcpyAsync(&tot[1], uptr + n, 4, cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if ((int64_t)tot[0] != (nnz + n) / 2 || tot[1] != tot[0]) {
    lapy_set_last_message("spai_pattern: the pattern is not symmetric with a full diagonal");
    return LAPY_ERR_PATTERN;
  }
  spai_fill_kernel<<<nb, 256, 0, stream>>>(n, indptr, indices, lptr, uptr, lcol, lpos, ucol);
  LAPY_TRY(lapy_check_launch("spai_fill_kernel"));
  LAPY_CUDA_TRY(cudaMemsetAsync(missing, 0, sizeof(int), stream));
  spai_umap_kernel<<<nb, 256, 0, stream>>>(n, uptr, ucol, lptr, lcol, umap, missing);
  LAPY_TRY(lapy_check_launch("spai_umap_kernel"));
  int miss = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&miss, missing, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (miss) {
    lapy_set_last_message("spai_pattern: the pattern is not symmetric");
    return LAPY_ERR_PATTERN;
  }
  return LAPY_OK;
}

extern "C" int lapy_spai_features(int64_t n, int nseg, const int32_t* seg_row, const void* v, int coords_f32,
                                  const int32_t* indptr, const double* a_vals, const double* m_vals, int m_is_diag,
                                  const int32_t* lptr, const int32_t* lcol, const int32_t* lpos, const double* t_seg,
                                  const double* sigma_seg, const double* h_seg, double* mass_work, float* feat,
                                  void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n <= 0 || nseg <= 0 || !seg_row || !v || !indptr || !a_vals || !m_vals || !lptr || !lcol || !lpos || !t_seg ||
      !sigma_seg || !h_seg || !mass_work || !feat)
    return LAPY_ERR_INVALID;
  const unsigned nb = lapy_ceil_div(n, 256);
  spai_mass_kernel<<<nb, 256, 0, stream>>>(n, indptr, m_vals, m_is_diag, mass_work);
  LAPY_TRY(lapy_check_launch("spai_mass_kernel"));
  if (coords_f32)
    spai_features_kernel<float><<<nb, 256, 0, stream>>>(n, nseg, seg_row, (const float*)v, a_vals, mass_work, lptr,
                                                       lcol, lpos, t_seg, sigma_seg, h_seg, feat);
  else
    spai_features_kernel<double><<<nb, 256, 0, stream>>>(n, nseg, seg_row, (const double*)v, a_vals, mass_work, lptr,
                                                        lcol, lpos, t_seg, sigma_seg, h_seg, feat);
  return lapy_check_launch("spai_features_kernel");
}

extern "C" int lapy_spai_forward(int64_t ne, const float* feat, const void* weights_bf16, float* w_out,
                                 void* stream_) {
  if (ne <= 0 || !feat || !weights_bf16 || !w_out) return LAPY_ERR_INVALID;
  const unsigned grid = std::min<unsigned>(lapy_ceil_div(ne, 16 * kMmaWarps), 16u * lapy_num_sms());
  spai_forward_mma_kernel<<<grid, 32 * kMmaWarps, 0, (cudaStream_t)stream_>>>(
      ne, feat, (const __nv_bfloat16*)weights_bf16, w_out);
  return lapy_check_launch("spai_forward_mma_kernel");
}

extern "C" int lapy_spai_factor(int64_t n, const int32_t* indptr, const int32_t* indices, const double* k_vals,
                                const int32_t* lptr, const int32_t* lcol, const int32_t* lpos, const float* w,
                                float* g_lower, double* logq, float* dldw, void* stream_) {
  if (n <= 0 || !indptr || !indices || !k_vals || !lptr || !lcol || !lpos || !w || !g_lower) return LAPY_ERR_INVALID;
  spai_factor_kernel<<<lapy_ceil_div(n, 128), 128, 0, (cudaStream_t)stream_>>>(n, indptr, indices, k_vals, lptr,
                                                                             lcol, lpos, w, g_lower, logq, dldw);
  return lapy_check_launch("spai_factor_kernel");
}

extern "C" int lapy_spai_transpose_values(int64_t m, const int32_t* umap, const float* g_lower, float* g_upper,
                                          void* stream_) {
  if (m <= 0 || !umap || !g_lower || !g_upper) return LAPY_ERR_INVALID;
  spai_gather_kernel<<<lapy_ceil_div(m, 256), 256, 0, (cudaStream_t)stream_>>>(m, umap, g_lower, g_upper);
  return lapy_check_launch("spai_gather_kernel");
}

static int bwd_blocks(int64_t ne) {
  return std::max(1, std::min<int>((int)std::min<int64_t>(lapy_ceil_div(ne, kBwdThreads), 1 << 20),
                                   2 * lapy_num_sms()));
}

extern "C" size_t lapy_spai_backward_workspace_bytes(int64_t ne) {
  return a256(4 * (size_t)kNParam * bwd_blocks(std::max<int64_t>(ne, 1))) + 256;
}

extern "C" int lapy_spai_backward(int64_t ne, const float* feat, const void* weights_bf16, const float* dldw,
                                  float scale, float* grad, void* work, size_t ws_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (ne <= 0 || !feat || !weights_bf16 || !dldw || !grad || !work) return LAPY_ERR_INVALID;
  const int nblk = bwd_blocks(ne);
  if (ws_bytes < a256(4 * (size_t)kNParam * nblk) + 256) return LAPY_ERR_WORKSPACE;
  float* partial = (float*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  const size_t smem = bwd_smem();
  LAPY_CUDA_TRY(cudaFuncSetAttribute(spai_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  spai_backward_kernel<<<nblk, kBwdThreads, smem, stream>>>(ne, feat, (const __nv_bfloat16*)weights_bf16, dldw,
                                                            partial);
  LAPY_TRY(lapy_check_launch("spai_backward_kernel"));
  spai_grad_reduce_kernel<<<lapy_ceil_div(kNParam, 256), 256, 0, stream>>>(nblk, partial, scale, grad);
  return lapy_check_launch("spai_grad_reduce_kernel");
}

extern "C" int lapy_spai_adam(int nparam, float* theta, const float* grad, float* m, float* v, void* weights_bf16,
                              float lr, float beta1, float beta2, float eps, int step, void* stream_) {
  if (nparam <= 0 || !theta || !grad || !m || !v || !weights_bf16 || step <= 0) return LAPY_ERR_INVALID;
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  spai_adam_kernel<<<lapy_ceil_div(nparam, 256), 256, 0, (cudaStream_t)stream_>>>(
      nparam, theta, grad, m, v, (__nv_bfloat16*)weights_bf16, lr, beta1, beta2, eps, c1, c2);
  return lapy_check_launch("spai_adam_kernel");
}

extern "C" int lapy_spai_weights_to_bf16(int nparam, const float* theta, void* weights_bf16, void* stream_) {
  if (nparam <= 0 || !theta || !weights_bf16) return LAPY_ERR_INVALID;
  spai_to_bf16_kernel<<<lapy_ceil_div(nparam, 256), 256, 0, (cudaStream_t)stream_>>>(nparam, theta,
                                                                                   (__nv_bfloat16*)weights_bf16);
  return lapy_check_launch("spai_to_bf16_kernel");
}
