// Batched symmetric eigensolver for the small projected matrices of the
// Lanczos iteration, FP64 throughout, one CTA per matrix:
//   1. Householder reduction to tridiagonal form (Golub & Van Loan, Alg. 8.3.1),
//   2. bisection on Sturm sequence counts for the wanted eigenvalues
//      (Barth, Martin & Wilkinson 1967),
//   3. inverse iteration on the tridiagonal with partial pivoting, with
//      modified Gram-Schmidt inside clusters of (near-)equal eigenvalues
//      (Peters & Wilkinson 1971),
//   4. back-transformation by the stored Householder reflectors.
#include <cfloat>
#include <cmath>
#include "dense.cuh"

namespace lapy {

constexpr int kEigThreads = 256;

size_t sym_eig_work_doubles(int lda, int want) {
  return (size_t)lda * 6 + (size_t)want * 2 + (size_t)want * 6 * lda + 64;
}

__device__ __forceinline__ int sturm_count(const double* d, const double* e2, int n, double x,
                                           double pivmin) {
  int cnt = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++cnt;
  for (int i = 1; i < n; ++i) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// Tridiagonal (d, e) minus theta*I: LU with partial pivoting, then solve in place on y.
__device__ void tri_solve_shifted(const double* d, const double* e, int n, double theta, double* U0,
                                  double* U1, double* U2, double* L, double* P, double* y,
                                  double tiny) {
  double x0 = d[0] - theta, x1 = (n > 1) ? e[0] : 0.0, x2 = 0.0;
  for (int k = 0; k < n - 1; ++k) {
    const double y0 = e[k], y1 = d[k + 1] - theta, y2 = (k + 2 < n) ? e[k + 1] : 0.0;
    double p0, p1, p2, o0, o1, o2;
    if (fabs(x0) >= fabs(y0)) {
      p0 = x0; p1 = x1; p2 = x2; o0 = y0; o1 = y1; o2 = y2; P[k] = 0.0;
    } else {
      p0 = y0; p1 = y1; p2 = y2; o0 = x0; o1 = x1; o2 = x2; P[k] = 1.0;
    }
    if (fabs(p0) < tiny) p0 = (p0 < 0 ? -tiny : tiny);
    const double l = o0 / p0;
    L[k] = l;
    U0[k] = p0; U1[k] = p1; U2[k] = p2;
    x0 = o1 - l * p1;
    x1 = o2 - l * p2;
    x2 = 0.0;
  }
  if (fabs(x0) < tiny) x0 = (x0 < 0 ? -tiny : tiny);
  U0[n - 1] = x0; U1[n - 1] = 0.0; U2[n - 1] = 0.0;
  // forward: row swaps and eliminations on the right-hand side
  for (int k = 0; k < n - 1; ++k) {
    if (P[k] != 0.0) { const double t = y[k]; y[k] = y[k + 1]; y[k + 1] = t; }
    y[k + 1] -= L[k] * y[k];
  }
  // backward
  y[n - 1] /= U0[n - 1];
  if (n > 1) y[n - 2] = (y[n - 2] - U1[n - 2] * y[n - 1]) / U0[n - 2];
  for (int k = n - 3; k >= 0; --k) y[k] = (y[k] - U1[k] * y[k + 1] - U2[k] * y[k + 2]) / U0[k];
}

__global__ void __launch_bounds__(kEigThreads) sym_eig_kernel(double* Aall, int lda,
                                                              const int32_t* nsize, int want,
                                                              double* theta_all, double* S_all,
                                                              double* work_all, size_t wstride,
                                                              const int32_t* active) {
  __shared__ double sh[32];
  __shared__ double s_tau, s_beta, s_K;
  __shared__ int s_skip;
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  const int n = nsize[b];
  const int t = threadIdx.x;
  double* A = Aall + (int64_t)b * lda * lda;
  double* W = work_all + (int64_t)b * wstride;
  double* d = W;
  double* e = W + lda;
  double* tau = W + 2 * lda;
  double* pv = W + 3 * lda;
  double* e2 = W + 4 * lda;
  double* vv = W + 5 * lda;
  double* th = W + 6 * lda;             // want
  int* clus = (int*)(W + 6 * lda + want);  // want ints (cluster leader flag)
  double* vecw = W + 6 * lda + 2 * want;   // want * 6 * lda
  double* theta = theta_all + (int64_t)b * want;
  double* S = S_all + (int64_t)b * lda * want;
  const int nw = min(want, n);

  // ---- 1. Householder tridiagonalisation (lower), A[i*lda + j]
  for (int k = 0; k < n - 2; ++k) {
    // column k below the subdiagonal
    double s2 = 0.0;
    for (int i = k + 2 + t; i < n; i += kEigThreads) {
      const double x = A[(int64_t)i * lda + k];
      s2 += x * x;
    }
    s2 = block_sum(s2, sh);
    if (t == 0) {
      const double alpha = A[(int64_t)(k + 1) * lda + k];
      if (s2 == 0.0) {
        s_skip = 1;
        s_tau = 0.0;
        e[k] = alpha;
      } else {
        s_skip = 0;
        const double beta = -copysign(sqrt(alpha * alpha + s2), alpha);
        s_tau = (beta - alpha) / beta;
        s_beta = 1.0 / (alpha - beta);
        e[k] = beta;
      }
      tau[k] = s_tau;
      d[k] = A[(int64_t)k * lda + k];
    }
    __syncthreads();
    if (s_skip) continue;
    // v: v[k+1] = 1, v[i] = A[i][k] * s_beta (stored back into column k)
    const int m0 = k + 1;
    for (int i = m0 + t; i < n; i += kEigThreads) {
      double vi;
      if (i == m0) vi = 1.0;
      else {
        vi = A[(int64_t)i * lda + k] * s_beta;
        A[(int64_t)i * lda + k] = vi;
      }
      vv[i] = vi;
    }
    __syncthreads();
    // p = tau * A22 v  (A22 symmetric; thread i reads column i -> coalesced)
    double pdot = 0.0;
    for (int i = m0 + t; i < n; i += kEigThreads) {
      double acc = 0.0;
      for (int j = m0; j < n; ++j) acc += A[(int64_t)j * lda + i] * vv[j];
      acc *= s_tau;
      pv[i] = acc;
      pdot += acc * vv[i];
    }
    pdot = block_sum(pdot, sh);
    if (t == 0) s_K = -0.5 * s_tau * pdot;
    __syncthreads();
    for (int i = m0 + t; i < n; i += kEigThreads) pv[i] += s_K * vv[i];  // w
    __syncthreads();
    // A22 -= v w' + w v'
    for (int i = m0 + t; i < n; i += kEigThreads) {
      const double vi = vv[i], wi = pv[i];
      for (int j = m0; j < n; ++j) A[(int64_t)j * lda + i] -= vv[j] * wi + pv[j] * vi;
    }
    __syncthreads();
  }
  if (t == 0) {
    if (n >= 2) {
      d[n - 2] = A[(int64_t)(n - 2) * lda + (n - 2)];
      e[n - 2] = A[(int64_t)(n - 1) * lda + (n - 2)];
      tau[n - 2] = 0.0;
    }
    d[n - 1] = A[(int64_t)(n - 1) * lda + (n - 1)];
    if (n >= 1) e[n - 1] = 0.0;
  }
  __syncthreads();
  for (int i = t; i < n; i += kEigThreads) e2[i] = e[i] * e[i];
  __syncthreads();

  // ---- 2. bisection for the nw largest eigenvalues
  double gl = 0.0, gu = 0.0, emax2 = 0.0;
  {
    double lo = DBL_MAX, hi = -DBL_MAX, em = 0.0;
    for (int i = t; i < n; i += kEigThreads) {
      const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i < n - 1 ? fabs(e[i]) : 0.0);
      lo = fmin(lo, d[i] - r);
      hi = fmax(hi, d[i] + r);
      if (i < n - 1) em = fmax(em, e2[i]);
    }
    // block min/max via shared scratch
    __syncthreads();
    if (t < 32) sh[t] = DBL_MAX;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    if ((t & 31) == 0) sh[t >> 5] = lo;
    __syncthreads();
    if (t == 0) {
      double m = DBL_MAX;
      for (int w = 0; w < kEigThreads / 32; ++w) m = fmin(m, sh[w]);
      s_tau = m;
    }
    __syncthreads();
    gl = s_tau;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    if ((t & 31) == 0) sh[t >> 5] = hi;
    __syncthreads();
    if (t == 0) {
      double m = -DBL_MAX;
      for (int w = 0; w < kEigThreads / 32; ++w) m = fmax(m, sh[w]);
      s_tau = m;
    }
    __syncthreads();
    gu = s_tau;
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) em = fmax(em, __shfl_xor_sync(0xffffffffu, em, o));
    if ((t & 31) == 0) sh[t >> 5] = em;
    __syncthreads();
    if (t == 0) {
      double m = 0.0;
      for (int w = 0; w < kEigThreads / 32; ++w) m = fmax(m, sh[w]);
      s_tau = m;
    }
    __syncthreads();
    emax2 = s_tau;
    __syncthreads();
  }
  const double tnorm = fmax(fabs(gl), fabs(gu));
  const double pivmin = DBL_MIN * fmax(1.0, emax2) * 4.0;
  gl -= 4.0 * DBL_EPSILON * tnorm + 2 * pivmin;
  gu += 4.0 * DBL_EPSILON * tnorm + 2 * pivmin;
  for (int j = t; j < nw; j += kEigThreads) {
    const int idx = n - 1 - j;  // index from the bottom
    double lo = gl, hi = gu;
    for (int itb = 0; itb < 200; ++itb) {
      const double mid = 0.5 * (lo + hi);
      if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin || mid == lo || mid == hi) break;
      if (sturm_count(d, e2, n, mid, pivmin) <= idx) lo = mid; else hi = mid;
    }
    th[j] = 0.5 * (lo + hi);
  }
  __syncthreads();

  // ---- 3. inverse iteration; clusters of close eigenvalues share one thread
  const double ctol = 1e-7 * fmax(tnorm, DBL_MIN);
  for (int j = t; j < nw; j += kEigThreads) clus[j] = (j == 0) || (th[j - 1] - th[j] > ctol);
  __syncthreads();
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  for (int j = t; j < nw; j += kEigThreads) {
    if (!clus[j]) continue;
    int jend = j + 1;
    while (jend < nw && !clus[jend]) ++jend;
    for (int q = j; q < jend; ++q) {
      double* U0 = vecw + (int64_t)q * 6 * lda;
      double* U1 = U0 + lda;
      double* U2 = U1 + lda;
      double* Lm = U2 + lda;
      double* Pv = Lm + lda;
      double* y = Pv + lda;
      // shift: separate members of an exact cluster slightly (as LAPACK dstein)
      double sh_theta = th[q];
      if (q > j) sh_theta = th[j] - (double)(q - j) * 10.0 * DBL_EPSILON * fmax(fabs(th[j]), tnorm);
      // deterministic start vector
      for (int i = 0; i < n; ++i) {
        unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)(q * 40503u + 0x9e3779b9u);
        h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
        y[i] = ((double)(h & 0xffffff) / 16777216.0) - 0.5;
      }
      for (int itr = 0; itr < 4; ++itr) {
        tri_solve_shifted(d, e, n, sh_theta, U0, U1, U2, Lm, Pv, y, tiny);
        // MGS against previous members of the cluster
        for (int r = j; r < q; ++r) {
          const double* yr = vecw + (int64_t)r * 6 * lda + 5 * lda;
          double dp = 0.0;
          for (int i = 0; i < n; ++i) dp += yr[i] * y[i];
          for (int i = 0; i < n; ++i) y[i] -= dp * yr[i];
        }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += y[i] * y[i];
        nrm = sqrt(nrm);
        const double inv = nrm > 0 ? 1.0 / nrm : 0.0;
        for (int i = 0; i < n; ++i) y[i] *= inv;
      }
    }
  }
  __syncthreads();

  // ---- 4. back-transformation z = H_0 ... H_{n-3} y  (warp per vector)
  const int lane = t & 31, warp = t >> 5;
  for (int q = warp; q < nw; q += kEigThreads / 32) {
    double* y = vecw + (int64_t)q * 6 * lda + 5 * lda;
    for (int k = n - 3; k >= 0; --k) {
      const double tk = tau[k];
      if (tk == 0.0) continue;
      double dp = 0.0;
      for (int i = k + 1 + lane; i < n; i += 32) dp += (i == k + 1 ? 1.0 : A[(int64_t)i * lda + k]) * y[i];
      dp = warp_sum(dp);
      for (int i = k + 1 + lane; i < n; i += 32) y[i] -= tk * dp * (i == k + 1 ? 1.0 : A[(int64_t)i * lda + k]);
      __syncwarp();
    }
    for (int i = lane; i < lda; i += 32) S[(int64_t)i * want + q] = (i < n) ? y[i] : 0.0;
    if (lane == 0) theta[q] = th[q];
  }
  // columns beyond n (if want > n) are zero
  for (int q = nw + warp; q < want; q += kEigThreads / 32) {
    for (int i = lane; i < lda; i += 32) S[(int64_t)i * want + q] = 0.0;
    if (lane == 0) theta[q] = 0.0;
  }
}

int sym_eig_top(int nmat, double* A, int lda, const int32_t* nsize, int want, double* theta,
                double* S, double* work, const int32_t* active, cudaStream_t stream) {
  if (nmat <= 0) return LAPY_OK;
  sym_eig_kernel<<<nmat, kEigThreads, 0, stream>>>(A, lda, nsize, want, theta, S, work,
                                                  sym_eig_work_doubles(lda, want), active);
  return lapy_check_launch("sym_eig_kernel");
}

}  // namespace lapy
