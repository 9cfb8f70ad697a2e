// Curvature frame of a triangle mesh on the device: the pre-step of the
// anisotropic Laplace-Beltrami assembly (lapy/tria_mesh.py:1078-1279, with
// tria_normals :750-773, vertex_normals :775-817, vertex_areas :715-733,
// smooth_laplace :1747-1792 and map_vfunc_to_tfunc :1668-1694).
//
// Decomposition (one thread per triangle, vertex or matrix entry):
//   1. half-edge owners: for each triangle corner, the CSR position of the
//      directed edge (a, b) records its triangle; a position claimed twice
//      means the mesh is not oriented;
//   2. triangle normals and areas;
//   3. per vertex: incident triangles (the owners of the row's half-edges,
//      sorted by index), vertex area and area-weighted normal, and the
//      lengths of its interior edges;
//   4. the mean interior edge length (fixed-order reduction);
//   5. per vertex: the dihedral-angle tensor sum over its interior edges,
//      divided by their count;
//   6. Laplace smoothing: repeated products with the 1-ring averaging matrix
//      on the mesh's own CSR pattern;
//   7. per vertex: the 3 x 3 symmetric eigenproblem, directions ordered by
//      alignment with the vertex normal, the principal pair and its signs;
//   8. per triangle: the vertex frame pooled, projected into the triangle's
//      plane and completed by the normal.
// Sums run in the order NumPy's accumulations take (np.add.at in index
// order, row sums in column order) and the file is compiled without fused
// multiply-add.  The 3 x 3 eigenproblem follows the LAPACK driver that
// numpy.linalg.eigh calls (dsyevd: Householder reduction to tridiagonal form,
// implicit QL/QR iteration with Givens rotations and Wilkinson shifts, the
// reflector applied to the rotations, eigenvalues sorted ascending), restated
// from that published algorithm, so that each eigenvector comes out with the
// same sign: the reference averages vertex directions over triangles, where
// the signs matter.
#include <algorithm>
#include <cmath>
#include "common.cuh"
#include "scan.cuh"

namespace lapy {

static size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 ld3(const double* p, int64_t i) { return D3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
__device__ __forceinline__ void st3(double* p, int64_t i, D3 a) {
  p[3 * i] = a.x;
  p[3 * i + 1] = a.y;
  p[3 * i + 2] = a.z;
}
__device__ __forceinline__ D3 sub3(D3 a, D3 b) { return D3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 add3(D3 a, D3 b) { return D3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 neg3(D3 a) { return D3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ D3 scale3(D3 a, double s) { return D3{a.x * s, a.y * s, a.z * s}; }
// np.cross component order
__device__ __forceinline__ D3 cross3d(D3 a, D3 b) {
  return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// np.sum(a * b, axis=1) over three columns
__device__ __forceinline__ double dot3d(D3 a, D3 b) {
  double s = a.x * b.x;
  s = s + a.y * b.y;
  return s + a.z * b.z;
}

constexpr double kEps = 2.220446049250313e-16;  // sys.float_info.epsilon
// Largest vertex valence (neighbours) handled; larger ones are reported.
constexpr int kCurvMaxValence = 32;

// Position of column c in CSR row r (sorted columns), or -1.
__device__ __forceinline__ int32_t csr_find(const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                           int32_t r, int32_t c) {
  int32_t lo = indptr[r], hi = indptr[r + 1] - 1;
  while (lo <= hi) {
    const int32_t mid = (lo + hi) >> 1;
    const int32_t x = indices[mid];
    if (x == c) return mid;
    if (x < c) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

// ---- 3 x 3 symmetric eigenproblem ------------------------------------------
namespace eig3 {
constexpr double EPS = 1.1102230246251565e-16;  // unit roundoff
constexpr double SAFMIN = 2.2250738585072014e-308;
constexpr double EPS2 = EPS * EPS;

__device__ __forceinline__ double fsign(double a, double b) { return copysign(fabs(a), b); }

// sqrt(x^2 + y^2) without unnecessary overflow
__device__ double hypot2(double x, double y) {
  const double xa = fabs(x), ya = fabs(y);
  const double w = fmax(xa, ya), z = fmin(xa, ya);
  if (z == 0.0 || w > 1.79e308) return w;
  const double q = z / w;
  return w * sqrt(1.0 + q * q);
}

// Plane rotation [c s; -s c] [f; g] = [r; 0] with c >= 0 and r carrying the
// sign of f (the convention of current LAPACK releases).
__device__ void rotg(double f, double g, double& c, double& s, double& r) {
  const double rtmin = 1.4916681462400413e-154;  // sqrt(SAFMIN)
  const double rtmax = 9.480751908109176e+153;   // sqrt(SAFMAX / 2)
  const double f1 = fabs(f), g1 = fabs(g);
  if (g == 0.0) {
    c = 1.0;
    s = 0.0;
    r = f;
  } else if (f == 0.0) {
    c = 0.0;
    s = fsign(1.0, g);
    r = g1;
  } else if (f1 > rtmin && f1 < rtmax && g1 > rtmin && g1 < rtmax) {
    const double d = sqrt(f * f + g * g);
    c = f1 / d;
    r = fsign(d, f);
    s = g / r;
  } else {
    const double u = fmin(1.0 / SAFMIN, fmax(SAFMIN, fmax(f1, g1)));
    const double fs = f / u, gs = g / u;
    const double d = sqrt(fs * fs + gs * gs);
    c = fabs(fs) / d;
    r = fsign(d, f);
    s = gs / r;
    r = r * u;
  }
}

// Eigen-decomposition of the 2 x 2 block [a b; b c]: rt1 (larger in
// magnitude), rt2, and the rotation (cs, sn) whose first column is rt1's
// eigenvector.
__device__ void sym2(double a, double b, double c, double& rt1, double& rt2, double& cs1, double& sn1) {
  const double sm = a + c, df = a - c, adf = fabs(df), tb = b + b, ab = fabs(tb);
  double acmx, acmn;
  if (fabs(a) > fabs(c)) {
    acmx = a;
    acmn = c;
  } else {
    acmx = c;
    acmn = a;
  }
  double rt;
  if (adf > ab) {
    const double q = ab / adf;
    rt = adf * sqrt(1.0 + q * q);
  } else if (adf < ab) {
    const double q = adf / ab;
    rt = ab * sqrt(1.0 + q * q);
  } else {
    rt = ab * sqrt(2.0);
  }
  int sgn1;
  if (sm < 0.0) {
    rt1 = 0.5 * (sm - rt);
    sgn1 = -1;
    rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
  } else if (sm > 0.0) {
    rt1 = 0.5 * (sm + rt);
    sgn1 = 1;
    rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
  } else {
    rt1 = 0.5 * rt;
    rt2 = -0.5 * rt;
    sgn1 = 1;
  }
  int sgn2;
  double csv;
  if (df >= 0.0) {
    csv = df + rt;
    sgn2 = 1;
  } else {
    csv = df - rt;
    sgn2 = -1;
  }
  if (fabs(csv) > ab) {
    const double ct = -tb / csv;
    sn1 = 1.0 / sqrt(1.0 + ct * ct);
    cs1 = ct * sn1;
  } else if (ab == 0.0) {
    cs1 = 1.0;
    sn1 = 0.0;
  } else {
    const double tn = -csv / tb;
    cs1 = 1.0 / sqrt(1.0 + tn * tn);
    sn1 = tn * cs1;
  }
  if (sgn1 == sgn2) {
    const double tn = cs1;
    cs1 = -sn1;
    sn1 = tn;
  }
}

// Z := Z * P' for the rotations (c[k], s[k]) acting on columns j0+k, j0+k+1,
// applied in increasing (forward) or decreasing k.
__device__ void rot_cols(double (&Z)[3][3], int j0, int nrot, const double* c, const double* s, bool forward) {
  for (int t = 0; t < nrot; ++t) {
    const int k = forward ? t : nrot - 1 - t;
    const double ct = c[k], st = s[k];
    if (ct != 1.0 || st != 0.0) {
      const int j = j0 + k;
      for (int i = 0; i < 3; ++i) {
        const double temp = Z[i][j + 1];
        Z[i][j + 1] = ct * temp - st * Z[i][j];
        Z[i][j] = st * temp + ct * Z[i][j];
      }
    }
  }
}

// Eigenvalues (ascending, in d) and eigenvectors (columns of Z) of the
// symmetric tridiagonal matrix diag(d) + offdiag(e), Z starting from I:
// implicit QL or QR sweeps (by which end is larger) with Wilkinson shifts,
// 2 x 2 blocks solved directly.  Indices are 1-based as in the algorithm's
// published form.
__device__ void tridiag_eig(double (&d)[4], double (&e)[3], double (&Z)[3][3]) {
  const int n = 3, nmaxit = n * 30;
  int jtot = 0, l1 = 1;
  double cw[2], sw[2];
  while (l1 <= n) {
    if (l1 > 1) e[l1 - 1] = 0.0;
    int m = n;
    for (int mm = l1; mm <= n - 1; ++mm) {
      const double tst = fabs(e[mm]);
      if (tst == 0.0) {
        m = mm;
        break;
      }
      if (tst <= (sqrt(fabs(d[mm])) * sqrt(fabs(d[mm + 1]))) * EPS) {
        e[mm] = 0.0;
        m = mm;
        break;
      }
    }
    int l = l1;
    const int lsv = l;
    int lend = m;
    const int lendsv = lend;
    l1 = m + 1;
    if (lend == l) continue;
    double anorm = 0.0;
    for (int i = l; i <= lend; ++i) anorm = fmax(anorm, fabs(d[i]));
    for (int i = l; i < lend; ++i) anorm = fmax(anorm, fabs(e[i]));
    if (anorm == 0.0) continue;
    if (fabs(d[lend]) < fabs(d[l])) {
      lend = lsv;
      l = lendsv;
    }
    if (lend > l) {  // QL
      while (true) {
        int mq = lend;
        for (int mm = l; mm <= lend - 1; ++mm) {
          const double tst = fabs(e[mm]) * fabs(e[mm]);
          if (tst <= (EPS2 * fabs(d[mm])) * fabs(d[mm + 1]) + SAFMIN) {
            mq = mm;
            break;
          }
        }
        if (mq < lend) e[mq] = 0.0;
        double p = d[l];
        if (mq == l) {
          d[l] = p;
          ++l;
          if (l <= lend) continue;
          break;
        }
        if (mq == l + 1) {
          double rt1, rt2, c, s;
          sym2(d[l], e[l], d[l + 1], rt1, rt2, c, s);
          cw[0] = c;
          sw[0] = s;
          rot_cols(Z, l - 1, 1, cw, sw, false);
          d[l] = rt1;
          d[l + 1] = rt2;
          e[l] = 0.0;
          l += 2;
          if (l <= lend) continue;
          break;
        }
        if (jtot == nmaxit) break;
        ++jtot;
        double g = (d[l + 1] - p) / (2.0 * e[l]);
        double r = hypot2(g, 1.0);
        g = d[mq] - p + (e[l] / (g + fsign(r, g)));
        double s = 1.0, c = 1.0;
        p = 0.0;
        for (int i = mq - 1; i >= l; --i) {
          const double f = s * e[i], b = c * e[i];
          rotg(g, f, c, s, r);
          if (i != mq - 1) e[i + 1] = r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          cw[i - l] = c;
          sw[i - l] = -s;
        }
        rot_cols(Z, l - 1, mq - l, cw, sw, false);
        d[l] = d[l] - p;
        e[l] = g;
      }
    } else {  // QR
      while (true) {
        int mq = lend;
        for (int mm = l; mm >= lend + 1; --mm) {
          const double tst = fabs(e[mm - 1]) * fabs(e[mm - 1]);
          if (tst <= (EPS2 * fabs(d[mm])) * fabs(d[mm - 1]) + SAFMIN) {
            mq = mm;
            break;
          }
        }
        if (mq > lend) e[mq - 1] = 0.0;
        double p = d[l];
        if (mq == l) {
          d[l] = p;
          --l;
          if (l >= lend) continue;
          break;
        }
        if (mq == l - 1) {
          double rt1, rt2, c, s;
          sym2(d[l - 1], e[l - 1], d[l], rt1, rt2, c, s);
          cw[0] = c;
          sw[0] = s;
          rot_cols(Z, mq - 1, 1, cw, sw, true);
          d[l - 1] = rt1;
          d[l] = rt2;
          e[l - 1] = 0.0;
          l -= 2;
          if (l >= lend) continue;
          break;
        }
        if (jtot == nmaxit) break;
        ++jtot;
        double g = (d[l - 1] - p) / (2.0 * e[l - 1]);
        double r = hypot2(g, 1.0);
        g = d[mq] - p + (e[l - 1] / (g + fsign(r, g)));
        double s = 1.0, c = 1.0;
        p = 0.0;
        for (int i = mq; i <= l - 1; ++i) {
          const double f = s * e[i], b = c * e[i];
          rotg(g, f, c, s, r);
          if (i != mq) e[i - 1] = r;
          g = d[i] - p;
          r = (d[i + 1] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i] = g + p;
          g = c * r - b;
          cw[i - mq] = c;
          sw[i - mq] = s;
        }
        rot_cols(Z, mq - 1, l - mq, cw, sw, true);
        d[l] = d[l] - p;
        e[l - 1] = g;
      }
    }
    if (jtot >= nmaxit) break;
  }
  // ascending order, selection sort (column swaps)
  for (int ii = 2; ii <= n; ++ii) {
    const int i = ii - 1;
    int k = i;
    double p = d[i];
    for (int j = ii; j <= n; ++j)
      if (d[j] < p) {
        k = j;
        p = d[j];
      }
    if (k != i) {
      d[k] = d[i];
      d[i] = p;
      for (int r = 0; r < 3; ++r) {
        const double tmp = Z[r][i - 1];
        Z[r][i - 1] = Z[r][k - 1];
        Z[r][k - 1] = tmp;
      }
    }
  }
}

// Symmetric A (lower triangle used) = V diag(w) V', w ascending.
__device__ void sym3(const double (&A)[3][3], double (&w)[3], double (&V)[3][3]) {
  double a11 = A[1][1], a21 = A[2][1], a22 = A[2][2];
  // reflector H = I - tau v v', v = (1, x), taking (A[1][0], A[2][0]) to (beta, 0)
  double alpha = A[1][0], x = A[2][0], tau = 0.0;
  if (fabs(x) != 0.0) {
    const double beta = -fsign(hypot2(alpha, fabs(x)), alpha);
    tau = (beta - alpha) / beta;
    x = x * (1.0 / (alpha - beta));
    alpha = beta;
  }
  const double v0 = 1.0, v1 = x;
  if (tau != 0.0) {
    // y = tau * A22 * v (lower-triangle product), y -= (tau/2 (y'v)) v,
    // A22 -= v y' + y v'
    double y0 = 0.0, y1 = 0.0;
    {
      double t1 = tau * v0, t2 = 0.0;
      y0 = y0 + t1 * a11;
      y1 = y1 + t1 * a21;
      t2 = t2 + a21 * v1;
      y0 = y0 + tau * t2;
      t1 = tau * v1;
      y1 = y1 + t1 * a22;
      y1 = y1 + tau * 0.0;
    }
    const double al = -0.5 * tau * (y0 * v0 + y1 * v1);
    y0 = y0 + al * v0;
    y1 = y1 + al * v1;
    {
      double t1 = -1.0 * y0, t2 = -1.0 * v0;
      a11 = a11 + v0 * t1 + y0 * t2;
      a21 = a21 + v1 * t1 + y1 * t2;
      t1 = -1.0 * y1;
      t2 = -1.0 * v1;
      a22 = a22 + v1 * t1 + y1 * t2;
    }
  }
  double d[4] = {0.0, A[0][0], a11, a22};  // 1-based
  double e[3] = {0.0, alpha, a21};
  double Z[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  tridiag_eig(d, e, Z);
  if (tau != 0.0) {
    for (int j = 0; j < 3; ++j) {
      const double wj = Z[1][j] * v0 + Z[2][j] * v1;
      const double t = -tau * wj;
      Z[1][j] = Z[1][j] + v0 * t;
      Z[2][j] = Z[2][j] + v1 * t;
    }
  }
  for (int i = 0; i < 3; ++i) {
    w[i] = d[i + 1];
    for (int j = 0; j < 3; ++j) V[i][j] = Z[i][j];
  }
}
}  // namespace eig3

// ---- kernels ------------------------------------------------------------------
// 1. half-edge owners (and the orientation check)
__global__ void curv_owner_kernel(int64_t m, const int32_t* __restrict__ t, const int32_t* __restrict__ indptr,
                                  const int32_t* __restrict__ indices, int32_t* __restrict__ owner,
                                  int* __restrict__ bad) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m) return;
  for (int c = 0; c < 3; ++c) {
    const int32_t a = t[3 * f + c], b = t[3 * f + (c + 1) % 3];
    const int32_t pos = csr_find(indptr, indices, a, b);
    if (pos < 0) {
      atomicOr(bad, 2);
      continue;
    }
    if (atomicCAS(&owner[pos], -1, (int32_t)f) != -1) atomicOr(bad, 1);
  }
}

// 2. triangle normals (v1 - v0) x (v2 - v0), unit (lengths < eps left as is)
//    and areas 0.5 |(v1 - v0) x (v2 - v0)|
__global__ void curv_tri_kernel(int64_t m, const double* __restrict__ v, const int32_t* __restrict__ t,
                                double* __restrict__ tn, double* __restrict__ area) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m) return;
  const D3 p0 = ld3(v, t[3 * f]), p1 = ld3(v, t[3 * f + 1]), p2 = ld3(v, t[3 * f + 2]);
  const D3 n = cross3d(sub3(p1, p0), sub3(p2, p0));
  double ln = sqrt(dot3d(n, n));
  area[f] = 0.5 * ln;
  if (ln < kEps) ln = 1.0;
  st3(tn, f, D3{n.x / ln, n.y / ln, n.z / ln});
}

// incident triangles of vertex i (owners of its half-edges), ascending
__device__ __forceinline__ int incident(int64_t i, const int32_t* __restrict__ indptr,
                                        const int32_t* __restrict__ indices, const int32_t* __restrict__ owner,
                                        int32_t (&tri)[kCurvMaxValence]) {
  int nt = 0;
  for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
    if (indices[k] == (int32_t)i) continue;
    const int32_t f = owner[k];
    if (f < 0 || nt >= kCurvMaxValence) continue;
    int j = nt++;
    while (j > 0 && tri[j - 1] > f) {
      tri[j] = tri[j - 1];
      --j;
    }
    tri[j] = f;
  }
  return nt;
}

// interior edge (a, b), a < b: the triangles holding a->b and b->a, or -1
__device__ __forceinline__ bool interior_edge(int32_t a, int32_t b, int32_t kab, const int32_t* __restrict__ indptr,
                                              const int32_t* __restrict__ indices, const int32_t* __restrict__ owner,
                                              int32_t& ta, int32_t& tb) {
  ta = owner[kab];
  const int32_t kba = csr_find(indptr, indices, b, a);
  tb = kba >= 0 ? owner[kba] : -1;
  return ta >= 0 && tb >= 0;
}

// 3. per vertex: area (incident triangle areas in index order, / 3), normal
//    (corner cross products in np.add.at order: corner 0 over the triangles,
//    then corner 1, then corner 2), and the lengths of the interior edges
//    (i, j), j > i, at their CSR positions (lengths below eps count as 1;
//    -1 marks the other positions)
__global__ void curv_vertex1_kernel(int64_t n, const double* __restrict__ v, const int32_t* __restrict__ t,
                                    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                    const int32_t* __restrict__ owner, const double* __restrict__ area,
                                    double* __restrict__ varea, double* __restrict__ vn, double* __restrict__ el,
                                    int* __restrict__ bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t tri[kCurvMaxValence];
  const int nt = incident(i, indptr, indices, owner, tri);
  if (indptr[i + 1] - indptr[i] - 1 > kCurvMaxValence) atomicOr(bad, 4);
  double a = 0.0;
  for (int q = 0; q < nt; ++q) a = a + area[tri[q]];
  varea[i] = a / 3.0;
  D3 nsum{0.0, 0.0, 0.0};
  for (int c = 0; c < 3; ++c) {
    for (int q = 0; q < nt; ++q) {
      const int32_t f = tri[q];
      if (t[3 * f + c] != (int32_t)i) continue;
      const D3 p0 = ld3(v, t[3 * f]), p1 = ld3(v, t[3 * f + 1]), p2 = ld3(v, t[3 * f + 2]);
      const D3 d10 = sub3(p1, p0), d21 = sub3(p2, p1), d02 = sub3(p0, p2);
      const D3 cr = c == 0 ? cross3d(d10, neg3(d02)) : c == 1 ? cross3d(d21, neg3(d10)) : cross3d(d02, neg3(d21));
      nsum = add3(nsum, cr);
    }
  }
  double ln = sqrt(dot3d(nsum, nsum));
  if (ln < kEps) ln = 1.0;
  st3(vn, i, D3{nsum.x / ln, nsum.y / ln, nsum.z / ln});
  const D3 pi = ld3(v, i);
  for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
    const int32_t j = indices[k];
    double len = -1.0;
    int32_t ta, tb;
    if (j > (int32_t)i && interior_edge((int32_t)i, j, k, indptr, indices, owner, ta, tb)) {
      const D3 ev = sub3(ld3(v, j), pi);
      len = sqrt(dot3d(ev, ev));
      if (len < kEps) len = 1.0;
    }
    el[k] = len;
  }
}

// 4. sum and count of the interior edge lengths (one block, fixed order)
__global__ void curv_mean_kernel(int64_t nnz, const double* __restrict__ el, double* __restrict__ out) {
  __shared__ double sh[32];
  __shared__ double shc[32];
  double s = 0.0, c = 0.0;
  for (int64_t k = threadIdx.x; k < nnz; k += blockDim.x) {
    if (el[k] >= 0.0) {
      s += el[k];
      c += 1.0;
    }
  }
  s = block_sum(s, sh);
  c = block_sum(c, shc);
  if (threadIdx.x == 0) {
    out[0] = s;
    out[1] = c;
  }
}

// dihedral tensor of the interior edge (a, b), a < b (tria_mesh.py:1112-1160):
// signed angle between the normals of the triangles holding a->b and b->a,
// times the edge length over the mean, times e e' of the unit edge vector
// (upper triangle: xx, xy, xz, yy, yz, zz)
__device__ __forceinline__ void edge_tensor(const double* __restrict__ v, const double* __restrict__ tn, int32_t a,
                                            int32_t b, int32_t ta, int32_t tb, double mean_el, double (&ee)[6]) {
  const D3 na = ld3(tn, ta), nb = ld3(tn, tb);
  double ang = acos(fmin(fmax(dot3d(na, nb), -1.0), 1.0));
  D3 ev = sub3(ld3(v, b), ld3(v, a));
  double len = sqrt(dot3d(ev, ev));
  const double sg = dot3d(cross3d(na, nb), ev);
  ang = ang * -(sg > 0.0 ? 1.0 : sg < 0.0 ? -1.0 : 0.0);
  if (len < kEps) len = 1.0;
  ev = D3{ev.x / len, ev.y / len, ev.z / len};
  const double w = ang * (len / mean_el);
  ee[0] = (ev.x * ev.x) * w;
  ee[1] = (ev.x * ev.y) * w;
  ee[2] = (ev.x * ev.z) * w;
  ee[3] = (ev.y * ev.y) * w;
  ee[4] = (ev.y * ev.z) * w;
  ee[5] = (ev.z * ev.z) * w;
}

// 5. per vertex: sum of the tensors of its interior edges in np.add.at order
//    (edges (i, j), j > i, then edges (k, i), k < i, each by ascending other
//    end), divided by their count
__global__ void curv_vertex2_kernel(int64_t n, const double* __restrict__ v, const int32_t* __restrict__ indptr,
                                    const int32_t* __restrict__ indices, const int32_t* __restrict__ owner,
                                    const double* __restrict__ tn, const double* __restrict__ elsum,
                                    double* __restrict__ vv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double mean_el = elsum[1] > 0.0 ? elsum[0] / elsum[1] : 1.0;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  double deg = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
      const int32_t j = indices[k];
      int32_t a, b, kab;
      if (pass == 0) {
        if (j <= (int32_t)i) continue;
        a = (int32_t)i;
        b = j;
        kab = k;
      } else {
        if (j >= (int32_t)i) continue;
        a = j;
        b = (int32_t)i;
        kab = csr_find(indptr, indices, a, b);
        if (kab < 0) continue;
      }
      int32_t ta, tb;
      if (!interior_edge(a, b, kab, indptr, indices, owner, ta, tb)) continue;
      double ee[6];
      edge_tensor(v, tn, a, b, ta, tb, mean_el, ee);
      for (int c = 0; c < 6; ++c) acc[c] = acc[c] + ee[c];
      deg = deg + 1.0;
    }
  }
  if (deg == 0.0) deg = 1.0;
  for (int c = 0; c < 6; ++c) vv[6 * i + c] = acc[c] / deg;
}

// 6. one smoothing step out = S in (6 columns): S row i = the 1-ring of i,
//    entry area_i * (1 / (sum over the ring of area_i))
__global__ void curv_smooth_kernel(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                   const double* __restrict__ varea, const double* __restrict__ in,
                                   double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ai = varea[i];
  double rs = 0.0;
  for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k)
    if (indices[k] != (int32_t)i) rs = rs + ai;
  if (rs == 0.0) rs = 1.0;
  const double sij = ai * (1.0 / rs);
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int32_t k = indptr[i]; k < indptr[i + 1]; ++k) {
    const int32_t j = indices[k];
    if (j == (int32_t)i) continue;
    for (int c = 0; c < 6; ++c) acc[c] = acc[c] + sij * in[6 * (int64_t)j + c];
  }
  // (1 - lambda) f + lambda S f with lambda = 1
  for (int c = 0; c < 6; ++c) out[6 * i + c] = 0.0 * in[6 * i + c] + 1.0 * acc[c];
}

// 7. per vertex frame (tria_mesh.py:1165-1219); out: planar blocks
//    u_min (n x 3), u_max (n x 3), c_min, c_max, c_mean, c_gauss (n each),
//    normals (n x 3)
__global__ void curv_frame_kernel(int64_t n, const double* __restrict__ vv, const double* __restrict__ vn,
                                  double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* q = vv + 6 * i;
  const double A[3][3] = {{q[0], q[1], q[2]}, {q[1], q[3], q[4]}, {q[2], q[4], q[5]}};
  double w[3], V[3][3];
  eig3::sym3(A, w, V);
  const D3 nv = ld3(vn, i);
  // order by |v_c . n| descending (ties: the earlier column first)
  double al[3];
  for (int c = 0; c < 3; ++c) al[c] = -fabs(V[0][c] * nv.x + V[1][c] * nv.y + V[2][c] * nv.z);
  int o[3] = {0, 1, 2};
  for (int a = 1; a < 3; ++a) {
    const int x = o[a];
    int b = a;
    while (b > 0 && al[o[b - 1]] > al[x]) {
      o[b] = o[b - 1];
      --b;
    }
    o[b] = x;
  }
  D3 umin{V[0][o[2]], V[1][o[2]], V[2][o[2]]};
  D3 umax{V[0][o[1]], V[1][o[1]], V[2][o[1]]};
  D3 nrm{V[0][o[0]], V[1][o[0]], V[2][o[0]]};
  double cmin = w[o[1]], cmax = w[o[2]];
  const double cmean = (cmin + cmax) / 2.0;
  const double cgauss = cmin * cmax;
  if (cmin > cmax) {
    const double tc = cmin;
    cmin = cmax;
    cmax = tc;
    const D3 tu = umin;
    umin = umax;
    umax = tu;
  }
  const double sd = dot3d(nrm, nv);
  const double sg = sd > 0.0 ? 1.0 : sd < 0.0 ? -1.0 : 0.0;
  nrm = scale3(nrm, sg);
  if (dot3d(cross3d(umin, umax), nrm) < 0.0) umax = neg3(umax);
  st3(out, i, umin);
  st3(out + 3 * n, i, umax);
  out[6 * n + i] = cmin;
  out[7 * n + i] = cmax;
  out[8 * n + i] = cmean;
  out[9 * n + i] = cgauss;
  st3(out + 10 * n, i, nrm);
}

// 8. per triangle frame (tria_mesh.py:1221-1279); out: planar blocks
//    u1 (m x 3: u_min pooled and projected), u2 (m x 3: n x u1), c_min,
//    c_max (m each, pooled)
__global__ void curv_pool_kernel(int64_t n, int64_t m, const int32_t* __restrict__ t, const double* __restrict__ vf,
                                 const double* __restrict__ tn, double* __restrict__ out) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m) return;
  const int64_t a = t[3 * f], b = t[3 * f + 1], c = t[3 * f + 2];
  // np.sum(vfunc[t] / 3, axis=1): (x_a / 3 + x_b / 3) + x_c / 3
  auto pool = [&](const double* x, int64_t stride, int k) {
    return (x[stride * a + k] / 3.0 + x[stride * b + k] / 3.0) + x[stride * c + k] / 3.0;
  };
  const D3 tu{pool(vf, 3, 0), pool(vf, 3, 1), pool(vf, 3, 2)};
  const double tcmin = pool(vf + 6 * n, 1, 0), tcmax = pool(vf + 7 * n, 1, 0);
  const D3 nn = ld3(tn, f);
  const double dp = dot3d(nn, tu);
  D3 u1 = sub3(tu, D3{nn.x * dp, nn.y * dp, nn.z * dp});
  const double ln = fmax(sqrt(dot3d(u1, u1)), 1e-8);
  u1 = D3{u1.x / ln, u1.y / ln, u1.z / ln};
  const D3 u2 = cross3d(nn, u1);
  st3(out, f, u1);
  st3(out + 3 * m, f, u2);
  out[6 * m + f] = tcmin;
  out[7 * m + f] = tcmax;
}

}  // namespace lapy

using namespace lapy;

extern "C" size_t lapy_tria_curvature_workspace_bytes(int64_t n, int64_t m, int64_t nnz) {
  if (n <= 0 || m <= 0 || nnz <= 0) return 0;
  return a256(4 * (size_t)nnz) + a256(8 * 3 * (size_t)m) + a256(8 * (size_t)m) + a256(8 * (size_t)n) +
         a256(8 * 3 * (size_t)n) + a256(8 * (size_t)nnz) + a256(64) + 2 * a256(8 * 6 * (size_t)n) +
         a256(8 * 13 * (size_t)n) + a256(64) + 512;
}

extern "C" int lapy_tria_curvature(const double* v, int64_t n, const int32_t* t, int64_t m, const int32_t* indptr,
                                   const int32_t* indices, int64_t nnz, int smoothit, double* vtx_out,
                                   double* tri_out, void* work, size_t ws_bytes, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!v || n <= 0 || !t || m <= 0 || !indptr || !indices || nnz <= 0 || smoothit < 0 || !work) {
    lapy_set_last_message("tria_curvature: invalid arguments");
    return LAPY_ERR_INVALID;
  }
  if (ws_bytes < lapy_tria_curvature_workspace_bytes(n, m, nnz)) return LAPY_ERR_WORKSPACE;
  char* w = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  int32_t* owner = (int32_t*)w; w += a256(4 * (size_t)nnz);
  double* tn = (double*)w; w += a256(8 * 3 * (size_t)m);
  double* area = (double*)w; w += a256(8 * (size_t)m);
  double* varea = (double*)w; w += a256(8 * (size_t)n);
  double* vn = (double*)w; w += a256(8 * 3 * (size_t)n);
  double* el = (double*)w; w += a256(8 * (size_t)nnz);
  double* elsum = (double*)w; w += a256(64);
  double* vv0 = (double*)w; w += a256(8 * 6 * (size_t)n);
  double* vv1 = (double*)w; w += a256(8 * 6 * (size_t)n);
  double* vframe = (double*)w; w += a256(8 * 13 * (size_t)n);
  int* bad = (int*)w;
  const unsigned nb = lapy_ceil_div(n, 128), mb = lapy_ceil_div(m, 128);
  LAPY_CUDA_TRY(cudaMemsetAsync(owner, 0xff, 4 * (size_t)nnz, stream));  // -1
  LAPY_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), stream));
  curv_owner_kernel<<<mb, 128, 0, stream>>>(m, t, indptr, indices, owner, bad);
  LAPY_TRY(lapy_check_launch("curv_owner_kernel"));
  int hbad = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (hbad & 2) {
    lapy_set_last_message("tria_curvature: an element edge is missing from the CSR pattern");
    return LAPY_ERR_PATTERN;
  }
  if (hbad & 1) {
    lapy_set_last_message("Error: Can only compute edge information for oriented meshes!");
    return LAPY_ERR_INVALID;
  }
  curv_tri_kernel<<<mb, 128, 0, stream>>>(m, v, t, tn, area);
  LAPY_TRY(lapy_check_launch("curv_tri_kernel"));
  curv_vertex1_kernel<<<nb, 128, 0, stream>>>(n, v, t, indptr, indices, owner, area, varea, vn, el, bad);
  LAPY_TRY(lapy_check_launch("curv_vertex1_kernel"));
  curv_mean_kernel<<<1, 1024, 0, stream>>>(nnz, el, elsum);
  LAPY_TRY(lapy_check_launch("curv_mean_kernel"));
  curv_vertex2_kernel<<<nb, 128, 0, stream>>>(n, v, indptr, indices, owner, tn, elsum, vv0);
  LAPY_TRY(lapy_check_launch("curv_vertex2_kernel"));
  double* cur = vv0;
  double* nxt = vv1;
  for (int it = 0; it < smoothit; ++it) {
    curv_smooth_kernel<<<nb, 128, 0, stream>>>(n, indptr, indices, varea, cur, nxt);
    LAPY_TRY(lapy_check_launch("curv_smooth_kernel"));
    std::swap(cur, nxt);
  }
  double* vf = vtx_out ? vtx_out : vframe;
  curv_frame_kernel<<<nb, 128, 0, stream>>>(n, cur, vn, vf);
  LAPY_TRY(lapy_check_launch("curv_frame_kernel"));
  if (tri_out) {
    curv_pool_kernel<<<mb, 128, 0, stream>>>(n, m, t, vf, tn, tri_out);
    LAPY_TRY(lapy_check_launch("curv_pool_kernel"));
  }
  LAPY_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (hbad & 4) {
    lapy_set_last_message("tria_curvature: a vertex has more than %d neighbours", kCurvMaxValence);
    return LAPY_ERR_INVALID;
  }
  return LAPY_OK;
}
