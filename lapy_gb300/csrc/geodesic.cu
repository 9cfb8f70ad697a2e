// Per-element gradient, row normalisation and integrated divergence for the
// heat-method geodesics (lapy/diffgeo.py:116-165), plus the Dirichlet row /
// column masking used by the Poisson solve (lapy/solver.py:847-865).
//
// Compiled with --fmad=false: products and sums round separately, in NumPy's
// order, in the coordinate type; function values are float64 and the mixed
// expressions promote to float64 exactly as NumPy does.
#include <cmath>
#include "common.cuh"

namespace lapy {

template <typename T>
struct P3 {
  T x, y, z;
};
template <typename T>
__device__ __forceinline__ P3<T> ld3(const T* v, int64_t i) {
  return P3<T>{v[3 * i], v[3 * i + 1], v[3 * i + 2]};
}
template <typename T>
__device__ __forceinline__ P3<T> operator-(P3<T> a, P3<T> b) {
  return P3<T>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
__device__ __forceinline__ P3<T> neg(P3<T> a) {
  return P3<T>{-a.x, -a.y, -a.z};
}
template <typename A, typename B>
__device__ __forceinline__ auto cross(P3<A> a, P3<B> b) -> P3<decltype(A() * B())> {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename A, typename B>
__device__ __forceinline__ auto dot(P3<A> a, P3<B> b) -> decltype(A() * B()) {
  auto s = a.x * b.x;
  s = s + a.y * b.y;
  s = s + a.z * b.z;
  return s;
}
template <typename T>
__device__ __forceinline__ P3<double> widen(P3<T> a) {
  return P3<double>{(double)a.x, (double)a.y, (double)a.z};
}

// diffgeo.py:261-298 (tria_compute_gradient), one thread per (element, function)
template <typename T>
__global__ void tria_gradient_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                     const double* __restrict__ f, int nf, double* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * nf) return;
  const int64_t e = idx / nf;
  const int q = (int)(idx - e * nf);
  const int32_t i0 = t[3 * e], i1 = t[3 * e + 1], i2 = t[3 * e + 2];
  const P3<T> v0 = ld3(v, i0), v1 = ld3(v, i1), v2 = ld3(v, i2);
  const P3<T> e2 = v1 - v0, e0 = v2 - v1, e1 = v0 - v2;
  P3<T> n = cross(e2, neg(e1));
  T ln = sqrt(dot(n, n));
  if (ln < (T)2.220446049250313e-16) ln = T(1);
  const T lni = T(1) / ln;
  n = P3<T>{n.x * lni, n.y * lni, n.z * lni};
  const double f0 = f[(int64_t)i0 * nf + q], f1 = f[(int64_t)i1 * nf + q], f2 = f[(int64_t)i2 * nf + q];
  const P3<double> w0 = widen(e0), w1 = widen(e1), w2 = widen(e2);
  // (f0*e0 + f1*e1) + f2*e2
  const P3<double> c{(f0 * w0.x + f1 * w1.x) + f2 * w2.x, (f0 * w0.y + f1 * w1.y) + f2 * w2.y,
                     (f0 * w0.z + f1 * w1.z) + f2 * w2.z};
  const P3<double> cr = cross(widen(n), c);
  const double li = (double)lni;
  double* o = out + idx * 3;
  o[0] = li * cr.x;
  o[1] = li * cr.y;
  o[2] = li * cr.z;
}

// diffgeo.py:880-920 (tet_compute_gradient)
template <typename T>
__global__ void tet_gradient_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                    const double* __restrict__ f, int nf, double* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * nf) return;
  const int64_t e = idx / nf;
  const int q = (int)(idx - e * nf);
  const int32_t i0 = t[4 * e], i1 = t[4 * e + 1], i2 = t[4 * e + 2], i3 = t[4 * e + 3];
  const P3<T> v0 = ld3(v, i0), v1 = ld3(v, i1), v2 = ld3(v, i2), v3 = ld3(v, i3);
  const P3<T> e0 = v1 - v0, e2 = v0 - v2, e3 = v3 - v0, e4 = v3 - v1, e5 = v3 - v2;
  const P3<T> cr = cross(e0, e2);
  T vol = abs(dot(e3, cr));
  if (vol < (T)2.220446049250313e-16) vol = T(1);
  const T voli = T(1) / vol;
  const P3<T> cr25 = cross(e2, e5), cr34 = cross(e3, e4), cr2e0 = cross(neg(e2), e0);
  const double f0 = f[(int64_t)i0 * nf + q];
  const double d1 = f[(int64_t)i1 * nf + q] - f0, d2 = f[(int64_t)i2 * nf + q] - f0,
               d3 = f[(int64_t)i3 * nf + q] - f0;
  const P3<double> a = widen(cr25), b = widen(cr34), c = widen(cr2e0);
  const double vi = (double)voli;
  double* o = out + idx * 3;
  o[0] = vi * ((d1 * a.x + d2 * b.x) + d3 * c.x);
  o[1] = vi * ((d1 * a.y + d2 * b.y) + d3 * c.y);
  o[2] = vi * ((d1 * a.z + d2 * b.z) + d3 * c.z);
}

// g / ||g|| per 3-vector, with nan_to_num's result for zero vectors (0).  The
// vector is scaled by its largest component first, so that squaring cannot
// underflow (diffgeo.py:153 squares the raw components, which underflows to
// 0/0 for heat values below ~1e-154; this form gives the unit vector there).
__global__ void normalize_rows3_kernel(int64_t rows, double* __restrict__ g) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double* p = g + 3 * r;
  const double x = p[0], y = p[1], z = p[2];
  const double s = fmax(fabs(x), fmax(fabs(y), fabs(z)));
  if (!(s > 0.0) || !isfinite(s)) {
    // zero vector: 0/0 -> nan -> 0; non-finite input: the quotient is nan or 0 -> 0
    p[0] = 0.0;
    p[1] = 0.0;
    p[2] = 0.0;
    return;
  }
  const double a = x / s, b = y / s, c = z / s;
  const double nrm = sqrt((a * a + b * b) + c * c);
  p[0] = a / nrm;
  p[1] = b / nrm;
  p[2] = c / nrm;
}

// Per-element divergence contributions x_l (diffgeo.py:340-363, :957-981).
template <typename T>
__global__ void tria_div_local_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                      const double* __restrict__ tf, int nf, double* __restrict__ xl) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * nf) return;
  const int64_t e = idx / nf;
  const int q = (int)(idx - e * nf);
  const P3<T> v0 = ld3(v, t[3 * e]), v1 = ld3(v, t[3 * e + 1]), v2 = ld3(v, t[3 * e + 2]);
  const P3<T> e2 = v1 - v0, e0 = v2 - v1, e1 = v0 - v2;
  const P3<T> n = cross(e2, neg(e1));
  T ln = sqrt(dot(n, n));
  if (ln < (T)2.220446049250313e-16) ln = T(1);
  const T cot0 = dot(e2, neg(e1)) / ln, cot1 = dot(e0, neg(e2)) / ln, cot2 = dot(e1, neg(e0)) / ln;
  const P3<T> c0{cot0 * e0.x, cot0 * e0.y, cot0 * e0.z};
  const P3<T> c1{cot1 * e1.x, cot1 * e1.y, cot1 * e1.z};
  const P3<T> c2{cot2 * e2.x, cot2 * e2.y, cot2 * e2.z};
  const double* g = tf + idx * 3;
  const P3<double> G{g[0], g[1], g[2]};
  const double x0 = dot(widen(c2 - c1), G), x1 = dot(widen(c0 - c2), G), x2 = dot(widen(c1 - c0), G);
  xl[(e * 3 + 0) * nf + q] = x0;
  xl[(e * 3 + 1) * nf + q] = x1;
  xl[(e * 3 + 2) * nf + q] = x2;
}

template <typename T>
__global__ void tet_div_local_kernel(const T* __restrict__ v, const int32_t* __restrict__ t, int64_t m,
                                     const double* __restrict__ tf, int nf, double* __restrict__ xl) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= m * nf) return;
  const int64_t e = idx / nf;
  const int q = (int)(idx - e * nf);
  const P3<T> v0 = ld3(v, t[4 * e]), v1 = ld3(v, t[4 * e + 1]), v2 = ld3(v, t[4 * e + 2]),
              v3 = ld3(v, t[4 * e + 3]);
  const P3<T> e0 = v1 - v0, e1 = v2 - v1, e2 = v2 - v0, e3 = v3 - v0, e4 = v3 - v1;
  const P3<T> n0 = cross(e1, e4), n1 = cross(e3, e2), n2 = cross(e0, e3), n3 = cross(e2, e0);
  const double* g = tf + idx * 3;
  const P3<double> G{g[0], g[1], g[2]};
  xl[(e * 4 + 0) * nf + q] = dot(widen(n0), G);
  xl[(e * 4 + 1) * nf + q] = dot(widen(n1), G);
  xl[(e * 4 + 2) * nf + q] = dot(widen(n2), G);
  xl[(e * 4 + 3) * nf + q] = dot(widen(n3), G);
}

// Per vertex: sum the contributions of its incident elements, in element
// order, read from the diagonal run of the assembly map; scale by `scale`.
__global__ void vertex_gather_kernel(int64_t n, int npe, const int32_t* __restrict__ diag_pos,
                                     const int32_t* __restrict__ seg_ptr, const int32_t* __restrict__ seg_src,
                                     const double* __restrict__ xl, int nf, double scale,
                                     double* __restrict__ out) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * nf) return;
  const int64_t i = idx / nf;
  const int q = (int)(idx - i * nf);
  const int L = npe * npe;
  const int d0 = L - npe;  // first diagonal slot
  double s = 0.0;
  const int32_t k = diag_pos[i];
  if (k >= 0) {
    for (int32_t r = seg_ptr[k]; r < seg_ptr[k + 1]; ++r) {
      const int32_t src = seg_src[r];
      const int32_t e = src / L;
      const int slot = src - e * L;
      if (slot < d0) continue;
      s += xl[((int64_t)e * npe + (slot - d0)) * nf + q];
    }
  }
  out[idx] = scale * s;
}

__global__ void dirichlet_mask_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                      const int32_t* __restrict__ indices, const double* __restrict__ vals,
                                      const uint8_t* __restrict__ dmask, double* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const bool dr = dmask[r] != 0;
  for (int32_t k = indptr[r]; k < indptr[r + 1]; ++k) {
    const int32_t c = indices[k];
    if (dr || dmask[c]) out[k] = (c == (int32_t)r && dr) ? 1.0 : 0.0;
    else out[k] = vals[k];
  }
}

}  // namespace lapy

using namespace lapy;

extern "C" int lapy_csr_dirichlet_mask(int64_t n, const int32_t* indptr, const int32_t* indices,
                                       const double* vals, const uint8_t* dmask, double* out, void* stream) {
  if (n <= 0 || !indptr || !indices || !vals || !dmask || !out) return LAPY_ERR_INVALID;
  dirichlet_mask_kernel<<<lapy_ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(n, indptr, indices, vals, dmask, out);
  return lapy_check_launch("dirichlet_mask_kernel");
}

extern "C" int lapy_tria_gradient(const void* v, int coords_f32, const int32_t* t, int64_t m, const double* f,
                                  int nf, double* out, void* stream) {
  if (!v || !t || m <= 0 || !f || nf <= 0 || !out) return LAPY_ERR_INVALID;
  const unsigned g = lapy_ceil_div(m * nf, 256);
  if (coords_f32)
    tria_gradient_kernel<float><<<g, 256, 0, (cudaStream_t)stream>>>((const float*)v, t, m, f, nf, out);
  else
    tria_gradient_kernel<double><<<g, 256, 0, (cudaStream_t)stream>>>((const double*)v, t, m, f, nf, out);
  return lapy_check_launch("tria_gradient_kernel");
}

extern "C" int lapy_tet_gradient(const void* v, int coords_f32, const int32_t* t, int64_t m, const double* f,
                                 int nf, double* out, void* stream) {
  if (!v || !t || m <= 0 || !f || nf <= 0 || !out) return LAPY_ERR_INVALID;
  const unsigned g = lapy_ceil_div(m * nf, 256);
  if (coords_f32)
    tet_gradient_kernel<float><<<g, 256, 0, (cudaStream_t)stream>>>((const float*)v, t, m, f, nf, out);
  else
    tet_gradient_kernel<double><<<g, 256, 0, (cudaStream_t)stream>>>((const double*)v, t, m, f, nf, out);
  return lapy_check_launch("tet_gradient_kernel");
}

extern "C" int lapy_normalize_rows3(int64_t rows, int reserved, double* g, void* stream) {
  (void)reserved;
  if (rows <= 0 || !g) return LAPY_ERR_INVALID;
  normalize_rows3_kernel<<<lapy_ceil_div(rows, 256), 256, 0, (cudaStream_t)stream>>>(rows, g);
  return lapy_check_launch("normalize_rows3_kernel");
}

static int divergence_impl(int npe, const void* v, int coords_f32, const int32_t* t, int64_t m, int64_t n,
                           const int32_t* diag_pos, const int32_t* seg_ptr, const int32_t* seg_src,
                           const double* tfunc, int nf, double* out, double* work, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!v || !t || m <= 0 || n <= 0 || !diag_pos || !seg_ptr || !seg_src || !tfunc || nf <= 0 || !out || !work)
    return LAPY_ERR_INVALID;
  const unsigned g = lapy_ceil_div(m * nf, 256);
  if (npe == 3) {
    if (coords_f32) tria_div_local_kernel<float><<<g, 256, 0, stream>>>((const float*)v, t, m, tfunc, nf, work);
    else tria_div_local_kernel<double><<<g, 256, 0, stream>>>((const double*)v, t, m, tfunc, nf, work);
  } else {
    if (coords_f32) tet_div_local_kernel<float><<<g, 256, 0, stream>>>((const float*)v, t, m, tfunc, nf, work);
    else tet_div_local_kernel<double><<<g, 256, 0, stream>>>((const double*)v, t, m, tfunc, nf, work);
  }
  LAPY_TRY(lapy_check_launch("div_local_kernel"));
  // diffgeo.py:366 (0.5 * sum) for triangles, :982-987 (-1/6 * sum) for tetrahedra
  const double scale = (npe == 3) ? 0.5 : -(1.0 / 6.0);
  vertex_gather_kernel<<<lapy_ceil_div(n * nf, 256), 256, 0, stream>>>(n, npe, diag_pos, seg_ptr, seg_src, work,
                                                                       nf, scale, out);
  return lapy_check_launch("vertex_gather_kernel");
}

extern "C" int lapy_tria_divergence(const void* v, int coords_f32, const int32_t* t, int64_t m, int64_t n,
                                    const int32_t* diag_pos, const int32_t* seg_ptr, const int32_t* seg_src,
                                    const double* tfunc, int nf, double* out, double* work, void* stream) {
  return divergence_impl(3, v, coords_f32, t, m, n, diag_pos, seg_ptr, seg_src, tfunc, nf, out, work, stream);
}

extern "C" int lapy_tet_divergence(const void* v, int coords_f32, const int32_t* t, int64_t m, int64_t n,
                                   const int32_t* diag_pos, const int32_t* seg_ptr, const int32_t* seg_src,
                                   const double* tfunc, int nf, double* out, double* work, void* stream) {
  return divergence_impl(4, v, coords_f32, t, m, n, diag_pos, seg_ptr, seg_src, tfunc, nf, out, work, stream);
}
