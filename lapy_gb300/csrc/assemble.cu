// FEM assembly for triangle and tetrahedral meshes: deterministic CSR build
// (segmented sort-and-reduce) and per-element cotangent stiffness / mass.
//
// This translation unit is compiled with --fmad=false so that the element
// arithmetic rounds every product separately, as NumPy does in
// lapy/solver.py:_fem_tria / _fem_tria_aniso / _fem_tetra.
#include "common.cuh"
#include "scan.cuh"

namespace lapy {

// Local (i, j) slot tables in the reference's COO order.
// Triangles: solver.py:174-175  (t1,t2,t2,t3,t3,t1,t1,t2,t3) x (t2,t1,t3,t2,t1,t3,t1,t2,t3)
// Tetrahedra: solver.py:492-497.
__constant__ int8_t kTriaI[9] = {0, 1, 1, 2, 2, 0, 0, 1, 2};
__constant__ int8_t kTriaJ[9] = {1, 0, 2, 1, 0, 2, 0, 1, 2};
__constant__ int8_t kTetI[16] = {0, 1, 1, 2, 2, 0, 0, 3, 1, 3, 2, 3, 0, 1, 2, 3};
__constant__ int8_t kTetJ[16] = {1, 0, 2, 1, 0, 2, 3, 0, 3, 1, 3, 2, 0, 1, 2, 3};

__device__ __forceinline__ void local_ij(int npe, int l, int& i, int& j) {
  if (npe == 3) {
    i = kTriaI[l];
    j = kTriaJ[l];
  } else {
    i = kTetI[l];
    j = kTetJ[l];
  }
}

// ---------------------------------------------------------------------------
// Symbolic phase
// ---------------------------------------------------------------------------
struct SymbolicWs {
  int32_t* row_count;   // n      COO entries per row, later fill cursor
  int32_t* bucket_ptr;  // n + 1  exclusive scan of row_count
  int32_t* row_nnz;     // n      distinct columns per row
  uint64_t* keys;       // m*L    (col << 32 | pos), bucketed by row
  uint64_t* sorted;     // m*L    keys sorted inside each row bucket
  int32_t* scan_scratch;
};

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

static size_t symbolic_layout(int64_t n, int64_t m, int npe, char* base, SymbolicWs* ws) {
  const int64_t L = (int64_t)npe * npe;
  const int64_t coo = m * L;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  char* p0 = take(sizeof(int32_t) * (size_t)n);
  char* p1 = take(sizeof(int32_t) * (size_t)(n + 1));
  char* p2 = take(sizeof(int32_t) * (size_t)n);
  char* p3 = take(sizeof(uint64_t) * (size_t)coo);
  char* p4 = take(sizeof(uint64_t) * (size_t)coo);
  char* p5 = take(sizeof(int32_t) * (size_t)scan_scratch_elems(n + 1));
  if (ws) {
    ws->row_count = (int32_t*)p0;
    ws->bucket_ptr = (int32_t*)p1;
    ws->row_nnz = (int32_t*)p2;
    ws->keys = (uint64_t*)p3;
    ws->sorted = (uint64_t*)p4;
    ws->scan_scratch = (int32_t*)p5;
  }
  return off;
}

__global__ void coo_count_kernel(const int32_t* __restrict__ elems, int64_t m, int npe,
                                 int32_t* __restrict__ row_count, int64_t n, int* bad) {
  const int64_t L = (int64_t)npe * npe;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * L) return;
  const int64_t e = idx / L;
  const int l = (int)(idx - e * L);
  int li, lj;
  local_ij(npe, l, li, lj);
  const int32_t r = elems[e * npe + li];
  const int32_t c = elems[e * npe + lj];
  if (r < 0 || r >= n || c < 0 || c >= n) {
    atomicExch(bad, 1);
    return;
  }
  atomicAdd(&row_count[r], 1);
}

__global__ void coo_bucket_kernel(const int32_t* __restrict__ elems, int64_t m, int npe,
                                  const int32_t* __restrict__ bucket_ptr,
                                  int32_t* __restrict__ cursor, uint64_t* __restrict__ keys,
                                  int64_t n) {
  const int64_t L = (int64_t)npe * npe;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * L) return;
  const int64_t e = idx / L;
  const int l = (int)(idx - e * L);
  int li, lj;
  local_ij(npe, l, li, lj);
  const int32_t r = elems[e * npe + li];
  const int32_t c = elems[e * npe + lj];
  if (r < 0 || r >= n || c < 0 || c >= n) return;
  const int32_t slot = bucket_ptr[r] + atomicAdd(&cursor[r], 1);
  keys[slot] = ((uint64_t)(uint32_t)c << 32) | (uint64_t)(uint32_t)idx;
}

// Warp per row: rank sort of the row's bucket (keys are unique, so the rank
// of a key is the number of smaller keys), then count distinct columns.
__global__ void row_sort_kernel(int64_t n, const int32_t* __restrict__ bucket_ptr,
                                const uint64_t* __restrict__ keys,
                                uint64_t* __restrict__ sorted, int32_t* __restrict__ row_nnz) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= n) return;
  const int32_t b0 = bucket_ptr[row], b1 = bucket_ptr[row + 1];
  const int k = b1 - b0;
  for (int a = lane; a < k; a += 32) {
    const uint64_t ka = keys[b0 + a];
    int rank = 0;
    for (int b = 0; b < k; ++b) rank += (keys[b0 + b] < ka) ? 1 : 0;
    sorted[b0 + rank] = ka;
  }
  __syncwarp();
  // distinct columns: entries whose column differs from the previous entry
  int cnt = 0;
  for (int a = lane; a < k; a += 32) {
    const uint32_t ca = (uint32_t)(sorted[b0 + a] >> 32);
    const bool first = (a == 0) || ((uint32_t)(sorted[b0 + a - 1] >> 32) != ca);
    cnt += first ? 1 : 0;
  }
  cnt = warp_sum(cnt);
  if (lane == 0) row_nnz[row] = cnt;
}

// Warp per row: write column indices, run starts and source positions.
__global__ void row_fill_kernel(int64_t n, const int32_t* __restrict__ bucket_ptr,
                                const uint64_t* __restrict__ sorted,
                                const int32_t* __restrict__ indptr, int32_t* __restrict__ indices,
                                int32_t* __restrict__ seg_ptr, int32_t* __restrict__ seg_src) {
  const int lane = threadIdx.x & 31;
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= n) return;
  const int32_t b0 = bucket_ptr[row], b1 = bucket_ptr[row + 1];
  const int k = b1 - b0;
  int32_t out = indptr[row];
  for (int base = 0; base < k; base += 32) {
    const int a = base + lane;
    bool first = false;
    uint32_t col = 0;
    if (a < k) {
      const uint64_t key = sorted[b0 + a];
      col = (uint32_t)(key >> 32);
      first = (a == 0) || ((uint32_t)(sorted[b0 + a - 1] >> 32) != col);
      seg_src[b0 + a] = (int32_t)(uint32_t)(key & 0xffffffffu);
    }
    const unsigned mask = __ballot_sync(0xffffffffu, first);
    if (first) {
      const int rank = __popc(mask & ((1u << lane) - 1u));
      indices[out + rank] = (int32_t)col;
      seg_ptr[out + rank] = b0 + a;
    }
    out += __popc(mask);
  }
}

// ---------------------------------------------------------------------------
// Numeric phase
// ---------------------------------------------------------------------------
struct NumericWs {
  double* vol;       // m      (element measure in the coordinate type, widened)
  double* partials;  // kVolBlocks
  double* clamp;     // max(nseg, 1): max(1e-4 * mean(vol), eps) per mesh
  char* local_a;     // m*L    local stiffness values (output type)
  char* local_m;     // m*L    local mass values (output type)
};
constexpr int kVolBlocks = 1024;
constexpr int kVolThreads = 256;

static size_t numeric_layout(int64_t m, int npe, int nseg, char* base, NumericWs* ws) {
  const int64_t L = (int64_t)npe * npe;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + off : nullptr;
    off += align256(bytes);
    return p;
  };
  char* p0 = take(sizeof(double) * (size_t)m);
  char* p1 = take(sizeof(double) * kVolBlocks);
  char* p2 = take(sizeof(double) * (size_t)std::max(nseg, 2));
  char* p3 = take(sizeof(double) * (size_t)(m * L));
  char* p4 = take(sizeof(double) * (size_t)(m * L));
  if (ws) {
    ws->vol = (double*)p0;
    ws->partials = (double*)p1;
    ws->clamp = (double*)p2;
    ws->local_a = p3;
    ws->local_m = p4;
  }
  return off;
}

template <typename T>
struct V3 {
  T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3<T> load_v(const T* v, int32_t i) {
  return V3<T>{v[3 * (int64_t)i], v[3 * (int64_t)i + 1], v[3 * (int64_t)i + 2]};
}
template <typename T>
__device__ __forceinline__ V3<T> sub(V3<T> a, V3<T> b) {
  return V3<T>{a.x - b.x, a.y - b.y, a.z - b.z};
}
// NumPy order: np.sum(a * b, axis=1) over 3 columns = (a0*b0 + a1*b1) + a2*b2
template <typename T>
__device__ __forceinline__ T dot3(V3<T> a, V3<T> b) {
  T s = a.x * b.x;
  s = s + a.y * b.y;
  s = s + a.z * b.z;
  return s;
}
// np.cross: (a1*b2 - a2*b1, a2*b0 - a0*b2, a0*b1 - a1*b0)
template <typename T>
__device__ __forceinline__ V3<T> cross3(V3<T> a, V3<T> b) {
  return V3<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

template <typename T>
__device__ __forceinline__ T tria_vol(const T* v, const int32_t* t, int64_t e) {
  const V3<T> v1 = load_v(v, t[3 * e]), v2 = load_v(v, t[3 * e + 1]), v3 = load_v(v, t[3 * e + 2]);
  const V3<T> v3mv2 = sub(v3, v2), v1mv3 = sub(v1, v3);
  const V3<T> cr = cross3(v3mv2, v1mv3);
  return T(2) * sqrt(dot3(cr, cr));  // solver.py:155-156  (= 4 * area)
}

template <typename T>
__device__ __forceinline__ T tet_vol(const T* v, const int32_t* t, int64_t e) {
  const V3<T> v1 = load_v(v, t[4 * e]), v2 = load_v(v, t[4 * e + 1]), v3 = load_v(v, t[4 * e + 2]),
              v4 = load_v(v, t[4 * e + 3]);
  const V3<T> e1 = sub(v2, v1), e3 = sub(v1, v3), e4 = sub(v4, v1);
  const V3<T> cr = cross3(e1, e3);
  return abs(dot3(e4, cr));  // solver.py:433-434  (= 6 * volume)
}

// Pass 1: element measures and per-block partial sums (for the global mean).
template <typename T, int NPE>
__global__ void elem_vol_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                double* __restrict__ vol, double* __restrict__ partials) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < m;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T w = (NPE == 3) ? tria_vol<T>(v, t, e) : tet_vol<T>(v, t, e);
    vol[e] = (double)w;
    acc += (double)w;
  }
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// clamp = max(1e-4 * mean(vol), DBL_EPSILON)  (solver.py:158, :272, :436)
template <typename T>
__global__ void vol_clamp_kernel(const double* __restrict__ partials, int nparts, int64_t m,
                                 double* __restrict__ clamp) {
  __shared__ double sh[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partials[i];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    const T mean = (T)(acc / (double)m);
    const T c = T(0.0001) * mean;
    const double eps = 2.220446049250313e-16;
    clamp[0] = ((double)c > eps) ? (double)c : eps;
  }
}

// Per-mesh clamps of a batch: one block per mesh sums the measures of its
// element range [seg_elem[s], seg_elem[s+1]) in a fixed order, so that each
// mesh is clamped with its own mean exactly as a single-mesh assembly does.
template <typename T>
__global__ void seg_vol_clamp_kernel(const double* __restrict__ vol, const int32_t* __restrict__ seg_elem,
                                     double* __restrict__ clamp) {
  __shared__ double sh[32];
  const int s = blockIdx.x;
  const int32_t e0 = seg_elem[s], e1 = seg_elem[s + 1];
  double acc = 0.0;
  for (int32_t e = e0 + (int32_t)threadIdx.x; e < e1; e += blockDim.x) acc += vol[e];
  acc = block_sum(acc, sh);
  if (threadIdx.x == 0) {
    const T mean = (e1 > e0) ? (T)(acc / (double)(e1 - e0)) : T(0);
    const T c = T(0.0001) * mean;
    const double eps = 2.220446049250313e-16;
    clamp[s] = ((double)c > eps) ? (double)c : eps;
  }
}

// Where the clamp of element e comes from: clamp[0] for a single mesh, else
// the clamp of the mesh whose element range holds e.
struct ClampDesc {
  const double* clamp;
  const int32_t* seg_elem;  // nseg + 1 element offsets (batches), or null
  int nseg;
};

template <typename T>
__device__ __forceinline__ T clamp_vol(T vol, const ClampDesc& cd, int64_t e) {
  const T eps = (T)2.220446049250313e-16;
  if (!(vol < eps)) return vol;
  int s = 0;
  if (cd.seg_elem) {  // largest s with seg_elem[s] <= e
    int lo = 0, hi = cd.nseg - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((int64_t)cd.seg_elem[mid] <= e) lo = mid; else hi = mid - 1;
    }
    s = lo;
  }
  return (T)cd.clamp[s];
}

// Pass 2 (triangles): local stiffness (cotangent) and mass values.
template <typename T, typename O>
__global__ void tria_local_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                  const ClampDesc clamp, int lump,
                                  O* __restrict__ la, O* __restrict__ lm) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  const V3<T> v1 = load_v(v, t[3 * e]), v2 = load_v(v, t[3 * e + 1]), v3 = load_v(v, t[3 * e + 2]);
  const V3<T> v2mv1 = sub(v2, v1), v3mv2 = sub(v3, v2), v1mv3 = sub(v1, v3);
  const V3<T> cr = cross3(v3mv2, v1mv3);
  T vol = T(2) * sqrt(dot3(cr, cr));
  vol = clamp_vol(vol, clamp, e);
  // solver.py:163-169
  const T a12 = dot3(v3mv2, v1mv3) / vol;
  const T a23 = dot3(v1mv3, v2mv1) / vol;
  const T a31 = dot3(v2mv1, v3mv2) / vol;
  const T a11 = -a12 - a31;
  const T a22 = -a12 - a23;
  const T a33 = -a31 - a23;
  O* pa = la + 9 * e;
  pa[0] = (O)a12; pa[1] = (O)a12; pa[2] = (O)a23; pa[3] = (O)a23; pa[4] = (O)a31;
  pa[5] = (O)a31; pa[6] = (O)a11; pa[7] = (O)a22; pa[8] = (O)a33;
  O* pm = lm + 9 * e;
  if (!lump) {  // solver.py:182-186
    const O bii = (O)(vol / T(24));
    const O bij = (O)(vol / T(48));
#pragma unroll
    for (int k = 0; k < 6; ++k) pm[k] = bij;
    pm[6] = bii; pm[7] = bii; pm[8] = bii;
  } else {  // solver.py:190  (only the diagonal slots are read)
    const O bii = (O)(vol / T(12));
#pragma unroll
    for (int k = 0; k < 6; ++k) pm[k] = O(0);
    pm[6] = bii; pm[7] = bii; pm[8] = bii;
  }
}

// Pass 2 (anisotropic triangles, solver.py:254-307).  Edge vectors and the
// element measure are in the coordinate type; the curvature frame u1, u2 and
// aniso_mat are float64 as curvature_tria produces them, so the projections
// and quotients run in float64 exactly as NumPy's type promotion does.
template <typename T, typename O>
__global__ void tria_aniso_local_kernel(const T* __restrict__ v, const int32_t* __restrict__ t,
                                        int64_t m, const double* __restrict__ u1,
                                        const double* __restrict__ u2,
                                        const double* __restrict__ an,
                                        const ClampDesc clamp, int lump,
                                        O* __restrict__ la, O* __restrict__ lm) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  const V3<T> v1 = load_v(v, t[3 * e]), v2 = load_v(v, t[3 * e + 1]), v3 = load_v(v, t[3 * e + 2]);
  const V3<T> v2mv1 = sub(v2, v1), v3mv2 = sub(v3, v2), v1mv3 = sub(v1, v3);
  const V3<double> U1{u1[3 * e], u1[3 * e + 1], u1[3 * e + 2]};
  const V3<double> U2{u2[3 * e], u2[3 * e + 1], u2[3 * e + 2]};
  auto widen = [](V3<T> a) { return V3<double>{(double)a.x, (double)a.y, (double)a.z}; };
  const V3<double> d21 = widen(v2mv1), d32 = widen(v3mv2), d13 = widen(v1mv3);
  const double p21[2] = {dot3(U1, d21), dot3(U2, d21)};
  const double p32[2] = {dot3(U1, d32), dot3(U2, d32)};
  const double p13[2] = {dot3(U1, d13), dot3(U2, d13)};
  const V3<T> cr = cross3(v3mv2, v1mv3);
  T vol = T(2) * sqrt(dot3(cr, cr));
  vol = clamp_vol(vol, clamp, e);
  const double a0 = an[2 * e], a1 = an[2 * e + 1];
  const double dv = (double)vol;
  // np.sum(x * aniso_mat * y, axis=1) = (x0*a0)*y0 + (x1*a1)*y1
  const double a12 = ((p32[0] * a0) * p13[0] + (p32[1] * a1) * p13[1]) / dv;
  const double a23 = ((p13[0] * a0) * p21[0] + (p13[1] * a1) * p21[1]) / dv;
  const double a31 = ((p21[0] * a0) * p32[0] + (p21[1] * a1) * p32[1]) / dv;
  const double a11 = -a12 - a31;
  const double a22 = -a12 - a23;
  const double a33 = -a31 - a23;
  O* pa = la + 9 * e;
  pa[0] = (O)a12; pa[1] = (O)a12; pa[2] = (O)a23; pa[3] = (O)a23; pa[4] = (O)a31;
  pa[5] = (O)a31; pa[6] = (O)a11; pa[7] = (O)a22; pa[8] = (O)a33;
  O* pm = lm + 9 * e;
  if (!lump) {
    const O bii = (O)(vol / T(24));
    const O bij = (O)(vol / T(48));
#pragma unroll
    for (int k = 0; k < 6; ++k) pm[k] = bij;
    pm[6] = bii; pm[7] = bii; pm[8] = bii;
  } else {
    const O bii = (O)(vol / T(12));
#pragma unroll
    for (int k = 0; k < 6; ++k) pm[k] = O(0);
    pm[6] = bii; pm[7] = bii; pm[8] = bii;
  }
}

// Pass 2 (tetrahedra, solver.py:426-532).
template <typename T, typename O>
__global__ void tet_local_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                 const ClampDesc clamp, int lump, O* __restrict__ la,
                                 O* __restrict__ lm) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  const V3<T> v1 = load_v(v, t[4 * e]), v2 = load_v(v, t[4 * e + 1]), v3 = load_v(v, t[4 * e + 2]),
              v4 = load_v(v, t[4 * e + 3]);
  const V3<T> e1 = sub(v2, v1), e2 = sub(v3, v2), e3 = sub(v1, v3), e4 = sub(v4, v1),
              e5 = sub(v4, v2), e6 = sub(v4, v3);
  const V3<T> cr = cross3(e1, e3);
  T vol = abs(dot3(e4, cr));
  vol = clamp_vol(vol, clamp, e);
  const T e11 = dot3(e1, e1), e22 = dot3(e2, e2), e33 = dot3(e3, e3), e44 = dot3(e4, e4),
          e55 = dot3(e5, e5), e66 = dot3(e6, e6);
  const T e12 = dot3(e1, e2), e13 = dot3(e1, e3), e14 = dot3(e1, e4), e15 = dot3(e1, e5),
          e23 = dot3(e2, e3), e25 = dot3(e2, e5), e26 = dot3(e2, e6), e34 = dot3(e3, e4),
          e36 = dot3(e3, e6);
  (void)e11; (void)e22; (void)e33; (void)e44; (void)e55;
  // solver.py:460-465
  const T a12 = ((-e36) * e26 + e23 * e66) / vol;
  const T a13 = ((-e15) * e25 + e12 * e55) / vol;
  const T a14 = (e23 * e26 - e36 * e22) / vol;
  const T a23 = ((-e14) * e34 + e13 * e44) / vol;
  const T a24 = (e13 * e34 - e14 * e33) / vol;
  const T a34 = ((-e14) * e13 + e11 * e34) / vol;
  // solver.py:467-470
  const T a11 = (-a12 - a13) - a14;
  const T a22 = (-a12 - a23) - a24;
  const T a33 = (-a13 - a23) - a34;
  const T a44 = (-a14 - a24) - a34;
  const T six = T(6);
  O* pa = la + 16 * e;  // solver.py:472-498 (then / 6.0)
  pa[0] = (O)(a12 / six); pa[1] = (O)(a12 / six); pa[2] = (O)(a23 / six); pa[3] = (O)(a23 / six);
  pa[4] = (O)(a13 / six); pa[5] = (O)(a13 / six); pa[6] = (O)(a14 / six); pa[7] = (O)(a14 / six);
  pa[8] = (O)(a24 / six); pa[9] = (O)(a24 / six); pa[10] = (O)(a34 / six); pa[11] = (O)(a34 / six);
  pa[12] = (O)(a11 / six); pa[13] = (O)(a22 / six); pa[14] = (O)(a33 / six); pa[15] = (O)(a44 / six);
  O* pm = lm + 16 * e;
  if (!lump) {  // solver.py:504-525
    const O bii = (O)(vol / T(60));
    const O bij = (O)(vol / T(120));
#pragma unroll
    for (int k = 0; k < 12; ++k) pm[k] = bij;
    pm[12] = bii; pm[13] = bii; pm[14] = bii; pm[15] = bii;
  } else {  // solver.py:529
    const O bii = (O)(vol / T(24));
#pragma unroll
    for (int k = 0; k < 12; ++k) pm[k] = O(0);
    pm[12] = bii; pm[13] = bii; pm[14] = bii; pm[15] = bii;
  }
}

// Pass 3: per nonzero, sum its run of local values in (element, slot) order.
template <typename O>
__global__ void segmented_reduce_kernel(int64_t nnz, const int32_t* __restrict__ seg_ptr,
                                        const int32_t* __restrict__ seg_src,
                                        const O* __restrict__ la, const O* __restrict__ lm,
                                        O* __restrict__ a, O* __restrict__ mvals) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const int32_t s0 = seg_ptr[k], s1 = seg_ptr[k + 1];
  O sa = la[seg_src[s0]];
  O sm = mvals ? lm[seg_src[s0]] : O(0);
  for (int32_t s = s0 + 1; s < s1; ++s) {
    const int32_t src = seg_src[s];
    sa = sa + la[src];
    if (mvals) sm = sm + lm[src];
  }
  a[k] = sa;
  if (mvals) mvals[k] = sm;
}

// Lumped mass: per row, sum the diagonal run of the local mass values.
template <typename O>
__global__ void lumped_reduce_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                     const int32_t* __restrict__ indices,
                                     const int32_t* __restrict__ seg_ptr,
                                     const int32_t* __restrict__ seg_src,
                                     const O* __restrict__ lm, O* __restrict__ mdiag) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  O s = O(0);
  bool any = false;
  for (int32_t k = indptr[r]; k < indptr[r + 1]; ++k) {
    if (indices[k] == (int32_t)r) {
      for (int32_t q = seg_ptr[k]; q < seg_ptr[k + 1]; ++q) {
        s = any ? s + lm[seg_src[q]] : lm[seg_src[q]];
        any = true;
      }
      break;
    }
  }
  mdiag[r] = s;
}

}  // namespace lapy

using namespace lapy;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" size_t lapy_csr_symbolic_workspace_bytes(int64_t n, int64_t m, int npe) {
  if (n < 0 || m < 0 || (npe != 3 && npe != 4)) return 0;
  return symbolic_layout(n, m, npe, nullptr, nullptr) + 256;
}

extern "C" int lapy_csr_symbolic_count(const int32_t* elems, int64_t m, int npe, int64_t n,
                                       int32_t* indptr, int64_t* nnz_out, void* workspace,
                                       size_t ws_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((npe != 3 && npe != 4) || n <= 0 || m <= 0 || !elems || !indptr || !nnz_out) {
    lapy_set_last_message("csr_symbolic_count: invalid arguments (npe=%d n=%lld m=%lld)", npe,
                          (long long)n, (long long)m);
    return LAPY_ERR_INVALID;
  }
  const int64_t L = (int64_t)npe * npe;
  if (m * L >= (int64_t)INT32_MAX || n >= (int64_t)INT32_MAX) {
    lapy_set_last_message("csr_symbolic_count: %lld local entries exceed int32", (long long)(m * L));
    return LAPY_ERR_INVALID;
  }
  if (ws_bytes < lapy_csr_symbolic_workspace_bytes(n, m, npe)) return LAPY_ERR_WORKSPACE;
  SymbolicWs ws;
  char* base = (char*)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  symbolic_layout(n, m, npe, base, &ws);
  // error flag lives in the scan scratch tail (one int), cleared here
  int* bad = (int*)(ws.row_nnz);  // row_nnz is unused until row_sort; reuse slot 0 as a flag
  LAPY_CUDA_TRY(cudaMemsetAsync(ws.row_count, 0, sizeof(int32_t) * n, stream));
  LAPY_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), stream));
  const int64_t coo = m * L;
  coo_count_kernel<<<lapy_ceil_div(coo, 256), 256, 0, stream>>>(elems, m, npe, ws.row_count, n, bad);
  LAPY_TRY(lapy_check_launch("coo_count_kernel"));
  int hbad = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (hbad) {
    lapy_set_last_message("csr_symbolic_count: element index outside [0, %lld)", (long long)n);
    return LAPY_ERR_INVALID;
  }
  LAPY_TRY(exclusive_scan_i32(ws.row_count, ws.bucket_ptr, n, ws.scan_scratch, stream));
  LAPY_CUDA_TRY(cudaMemsetAsync(ws.row_count, 0, sizeof(int32_t) * n, stream));
  coo_bucket_kernel<<<lapy_ceil_div(coo, 256), 256, 0, stream>>>(elems, m, npe, ws.bucket_ptr,
                                                                 ws.row_count, ws.keys, n);
  LAPY_TRY(lapy_check_launch("coo_bucket_kernel"));
  row_sort_kernel<<<lapy_ceil_div(n * 32, 256), 256, 0, stream>>>(n, ws.bucket_ptr, ws.keys,
                                                                  ws.sorted, ws.row_nnz);
  LAPY_TRY(lapy_check_launch("row_sort_kernel"));
  LAPY_TRY(exclusive_scan_i32(ws.row_nnz, indptr, n, ws.scan_scratch, stream));
  int32_t nnz = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&nnz, indptr + n, sizeof(int32_t), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  *nnz_out = nnz;
  return LAPY_OK;
}

extern "C" int lapy_csr_symbolic_fill(const int32_t* elems, int64_t m, int npe, int64_t n,
                                      const int32_t* indptr, int64_t nnz, int32_t* indices,
                                      int32_t* seg_ptr, int32_t* seg_src, void* workspace,
                                      size_t ws_bytes, void* stream_) {
  (void)elems;
  cudaStream_t stream = (cudaStream_t)stream_;
  if ((npe != 3 && npe != 4) || n <= 0 || m <= 0 || !indptr || !indices || !seg_ptr || !seg_src)
    return LAPY_ERR_INVALID;
  if (ws_bytes < lapy_csr_symbolic_workspace_bytes(n, m, npe)) return LAPY_ERR_WORKSPACE;
  SymbolicWs ws;
  char* base = (char*)(((uintptr_t)workspace + 255) & ~uintptr_t(255));
  symbolic_layout(n, m, npe, base, &ws);
  const int64_t coo = m * (int64_t)npe * npe;
  row_fill_kernel<<<lapy_ceil_div(n * 32, 256), 256, 0, stream>>>(n, ws.bucket_ptr, ws.sorted, indptr,
                                                                  indices, seg_ptr, seg_src);
  LAPY_TRY(lapy_check_launch("row_fill_kernel"));
  const int32_t total = (int32_t)coo;
  LAPY_CUDA_TRY(cudaMemcpyAsync(seg_ptr + nnz, &total, sizeof(int32_t), cudaMemcpyHostToDevice, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}

extern "C" size_t lapy_fem_numeric_workspace_bytes(int64_t m, int npe) {
  if (m < 0 || (npe != 3 && npe != 4)) return 0;
  return numeric_layout(m, npe, 1, nullptr, nullptr) + 256;
}

extern "C" size_t lapy_fem_batch_numeric_workspace_bytes(int64_t m, int npe, int nseg) {
  if (m < 0 || (npe != 3 && npe != 4) || nseg < 1) return 0;
  return numeric_layout(m, npe, nseg, nullptr, nullptr) + 256;
}

namespace {

enum class ElemKind { Tria, TriaAniso, Tet };

template <typename T, typename O>
int fem_numeric_impl(ElemKind kind, const T* v, const int32_t* t, int64_t m, const double* u1,
                     const double* u2, const double* an, int64_t n, const int32_t* indptr,
                     const int32_t* indices, const int32_t* seg_ptr, const int32_t* seg_src,
                     int64_t nnz, int lump, O* a_vals, O* m_vals, const NumericWs& ws,
                     int nseg, const int32_t* seg_elem, cudaStream_t stream) {
  const int npe = (kind == ElemKind::Tet) ? 4 : 3;
  const unsigned vb = (unsigned)std::min<int64_t>(kVolBlocks, std::max<int64_t>(1, lapy_ceil_div(m, kVolThreads)));
  if (npe == 3)
    elem_vol_kernel<T, 3><<<vb, kVolThreads, 0, stream>>>(v, t, m, ws.vol, ws.partials);
  else
    elem_vol_kernel<T, 4><<<vb, kVolThreads, 0, stream>>>(v, t, m, ws.vol, ws.partials);
  LAPY_TRY(lapy_check_launch("elem_vol_kernel"));
  ClampDesc cd{ws.clamp, nullptr, 1};
  if (seg_elem) {
    seg_vol_clamp_kernel<T><<<nseg, 256, 0, stream>>>(ws.vol, seg_elem, ws.clamp);
    LAPY_TRY(lapy_check_launch("seg_vol_clamp_kernel"));
    cd = ClampDesc{ws.clamp, seg_elem, nseg};
  } else {
    vol_clamp_kernel<T><<<1, 256, 0, stream>>>(ws.partials, (int)vb, m, ws.clamp);
    LAPY_TRY(lapy_check_launch("vol_clamp_kernel"));
  }
  O* la = (O*)ws.local_a;
  O* lm = (O*)ws.local_m;
  const unsigned eb = lapy_ceil_div(m, 128);
  if (kind == ElemKind::Tria)
    tria_local_kernel<T, O><<<eb, 128, 0, stream>>>(v, t, m, cd, lump, la, lm);
  else if (kind == ElemKind::TriaAniso)
    tria_aniso_local_kernel<T, O><<<eb, 128, 0, stream>>>(v, t, m, u1, u2, an, cd, lump, la, lm);
  else
    tet_local_kernel<T, O><<<eb, 128, 0, stream>>>(v, t, m, cd, lump, la, lm);
  LAPY_TRY(lapy_check_launch("elem_local_kernel"));
  segmented_reduce_kernel<O><<<lapy_ceil_div(nnz, 256), 256, 0, stream>>>(
      nnz, seg_ptr, seg_src, la, lm, a_vals, lump ? nullptr : m_vals);
  LAPY_TRY(lapy_check_launch("segmented_reduce_kernel"));
  if (lump) {
    lumped_reduce_kernel<O><<<lapy_ceil_div(n, 256), 256, 0, stream>>>(n, indptr, indices, seg_ptr,
                                                                      seg_src, lm, m_vals);
    LAPY_TRY(lapy_check_launch("lumped_reduce_kernel"));
  }
  return LAPY_OK;
}

int fem_numeric_dispatch(ElemKind kind, const void* v, int coords_f32, const int32_t* t, int64_t m,
                         const void* u1, const void* u2, const void* an, int64_t n,
                         const int32_t* indptr, const int32_t* indices, const int32_t* seg_ptr,
                         const int32_t* seg_src, int64_t nnz, int lump, int out_f32, void* a_vals,
                         void* m_vals, void* work, size_t ws_bytes, void* stream_, int nseg = 1,
                         const int32_t* seg_elem = nullptr) {
  cudaStream_t stream = (cudaStream_t)stream_;
  const int npe = (kind == ElemKind::Tet) ? 4 : 3;
  if (!v || !t || m <= 0 || n <= 0 || nnz <= 0 || !indptr || !indices || !seg_ptr || !seg_src ||
      !a_vals || !m_vals || !work) {
    lapy_set_last_message("fem_numeric: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (kind == ElemKind::TriaAniso && (!u1 || !u2 || !an)) {
    lapy_set_last_message("fem_tria_aniso_numeric: u1, u2 and aniso_mat are required");
    return LAPY_ERR_INVALID;
  }
  if (nseg < 1 || (seg_elem == nullptr && nseg != 1)) {
    lapy_set_last_message("fem_numeric: nseg must be >= 1, with seg_elem for nseg > 1");
    return LAPY_ERR_INVALID;
  }
  if (ws_bytes < lapy_fem_batch_numeric_workspace_bytes(m, npe, nseg)) return LAPY_ERR_WORKSPACE;
  NumericWs ws;
  char* base = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  numeric_layout(m, npe, nseg, base, &ws);
  const double* U1 = (const double*)u1;
  const double* U2 = (const double*)u2;
  const double* AN = (const double*)an;
  if (coords_f32) {
    if (out_f32)
      return fem_numeric_impl<float, float>(kind, (const float*)v, t, m, U1, U2, AN, n, indptr,
                                            indices, seg_ptr, seg_src, nnz, lump, (float*)a_vals,
                                            (float*)m_vals, ws, nseg, seg_elem, stream);
    return fem_numeric_impl<float, double>(kind, (const float*)v, t, m, U1, U2, AN, n, indptr,
                                           indices, seg_ptr, seg_src, nnz, lump, (double*)a_vals,
                                           (double*)m_vals, ws, nseg, seg_elem, stream);
  }
  if (out_f32)
    return fem_numeric_impl<double, float>(kind, (const double*)v, t, m, U1, U2, AN, n, indptr,
                                           indices, seg_ptr, seg_src, nnz, lump, (float*)a_vals,
                                           (float*)m_vals, ws, nseg, seg_elem, stream);
  return fem_numeric_impl<double, double>(kind, (const double*)v, t, m, U1, U2, AN, n, indptr,
                                          indices, seg_ptr, seg_src, nnz, lump, (double*)a_vals,
                                          (double*)m_vals, ws, nseg, seg_elem, stream);
}

}  // namespace

extern "C" int lapy_fem_tria_numeric(const void* v, int coords_f32, const int32_t* t, int64_t m,
                                     int64_t n, const int32_t* indptr, const int32_t* indices,
                                     const int32_t* seg_ptr, const int32_t* seg_src, int64_t nnz,
                                     int lump, int out_f32, void* a_vals, void* m_vals, void* work,
                                     size_t ws_bytes, void* stream) {
  return fem_numeric_dispatch(ElemKind::Tria, v, coords_f32, t, m, nullptr, nullptr, nullptr, n,
                              indptr, indices, seg_ptr, seg_src, nnz, lump, out_f32, a_vals, m_vals,
                              work, ws_bytes, stream);
}

extern "C" int lapy_fem_tria_aniso_numeric(const void* v, int coords_f32, const int32_t* t,
                                           int64_t m, const double* u1, const double* u2,
                                           const double* aniso_mat, int64_t n,
                                           const int32_t* indptr, const int32_t* indices,
                                           const int32_t* seg_ptr, const int32_t* seg_src,
                                           int64_t nnz, int lump, int out_f32, void* a_vals,
                                           void* m_vals, void* work, size_t ws_bytes, void* stream) {
  return fem_numeric_dispatch(ElemKind::TriaAniso, v, coords_f32, t, m, u1, u2, aniso_mat, n,
                              indptr, indices, seg_ptr, seg_src, nnz, lump, out_f32, a_vals, m_vals,
                              work, ws_bytes, stream);
}

extern "C" int lapy_fem_tet_numeric(const void* v, int coords_f32, const int32_t* t, int64_t m,
                                    int64_t n, const int32_t* indptr, const int32_t* indices,
                                    const int32_t* seg_ptr, const int32_t* seg_src, int64_t nnz,
                                    int lump, int out_f32, void* a_vals, void* m_vals, void* work,
                                    size_t ws_bytes, void* stream) {
  return fem_numeric_dispatch(ElemKind::Tet, v, coords_f32, t, m, nullptr, nullptr, nullptr, n,
                              indptr, indices, seg_ptr, seg_src, nnz, lump, out_f32, a_vals, m_vals,
                              work, ws_bytes, stream);
}

extern "C" int lapy_fem_batch_numeric(int npe, const void* v, int coords_f32, const int32_t* t, int64_t m,
                                      int nseg, const int32_t* seg_elem, int64_t n, const int32_t* indptr,
                                      const int32_t* indices, const int32_t* seg_ptr, const int32_t* seg_src,
                                      int64_t nnz, int lump, int out_f32, void* a_vals, void* m_vals, void* work,
                                      size_t ws_bytes, void* stream) {
  if ((npe != 3 && npe != 4) || nseg < 1 || !seg_elem) {
    lapy_set_last_message("fem_batch_numeric: npe must be 3 or 4, nseg >= 1 and seg_elem given");
    return LAPY_ERR_INVALID;
  }
  return fem_numeric_dispatch(npe == 4 ? ElemKind::Tet : ElemKind::Tria, v, coords_f32, t, m, nullptr, nullptr,
                              nullptr, n, indptr, indices, seg_ptr, seg_src, nnz, lump, out_f32, a_vals, m_vals,
                              work, ws_bytes, stream, nseg, seg_elem);
}
