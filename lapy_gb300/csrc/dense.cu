// Batched symmetric eigensolver for the small projected matrices of the
// Lanczos iteration, FP64 throughout, one CTA per matrix:
//   1. Householder reduction to tridiagonal form (Golub & Van Loan, Alg. 8.3.1),
//   2. multisection on Sturm sequence counts for the wanted eigenvalues
//      (Barth, Martin & Wilkinson 1967), several lanes per eigenvalue, with a
//      division-free count,
//   3. inverse iteration on the tridiagonal with partial pivoting (Peters &
//      Wilkinson 1971), all eigenvalues at once with the LU factors reused
//      across sweeps, and modified Gram-Schmidt inside clusters of
//      (near-)equal eigenvalues after every sweep,
//   4. back-transformation by the stored Householder reflectors.
// FP64 throughput is low on this GPU, so the sequential parts (counts,
// triangular solves) are arranged to issue as few FP64 instructions as
// possible and to keep every warp of the CTA busy.
#include <cfloat>
#include <cmath>
#include "dense.cuh"
#include "dfloat.cuh"

namespace lapy {

constexpr int kEigThreads = 256;

size_t sym_eig_work_doubles(int lda, int want) {
  return (size_t)lda * 4 + (size_t)want * 2 + (size_t)want * 5 * lda + 64;
}

__device__ __forceinline__ int exponent_field(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}

// Number of eigenvalues of the tridiagonal (d, e2 = e^2) below x, from the
// signs of its leading principal minors p_i = (d_i - x) p_{i-1} -
// e2_{i-1} p_{i-2} (the Sturm sequence; Wilkinson, The Algebraic Eigenvalue
// Problem, 1965, ch. 5): a sign change from p_{i-1} to p_i is a negative
// pivot of T - xI = LDL'.  The recurrence needs no division (the FP64 pipe is
// the bottleneck here).  The pair of latest minors is rescaled by a power of
// two whenever its larger exponent leaves [2^-400, 2^400], and a minor that
// comes out exactly zero is replaced, with its predecessor, by the pair
// (s, -2^-600 s), s = sign of the predecessor: a negative pivot of magnitude
// 2^-600, as the ratio form replaces a zero pivot by -pivmin.
__device__ __forceinline__ int sturm_count(const double* d, const double* e2, int n, double x) {
  double a = 1.0, b = d[0] - x;
  if (b == 0.0) b = -0x1p-600;
  int cnt = signbit(b) ? 1 : 0;
  for (int i = 1; i < n; ++i) {
    double c = fma(d[i] - x, b, -e2[i - 1] * a);
    if ((__double_as_longlong(c) << 1) == 0) {
      a = copysign(1.0, b);
      c = -0x1p-600 * a;
    } else {
      a = b;
    }
    cnt += (signbit(c) != signbit(a)) ? 1 : 0;
    b = c;
    const int em = max(exponent_field(a), exponent_field(b));
    if (em > 1023 + 400 || em < 1023 - 400) {
      const double s = __hiloint2double((2046 - em) << 20, 0);  // 2^(1023 - em)
      a *= s;
      b *= s;
    }
  }
  return cnt;
}

// LU with partial pivoting of the tridiagonal (d, e) minus theta*I (Peters &
// Wilkinson 1971).  Factors are stored with stride ld (one column per
// eigenvalue): the reciprocal pivots U0i, the two superdiagonals U1, U2 of U,
// the multipliers L and the row-swap flags P.  Pivots below `tiny` in
// magnitude are replaced by +-tiny.
__device__ void tri_factor(const double* d, const double* e, int n, double theta, double* U0i,
                           double* U1, double* U2, double* L, double* P, int ld, double tiny) {
  double x0 = d[0] - theta, x1 = (n > 1) ? e[0] : 0.0, x2 = 0.0;
  for (int k = 0; k < n - 1; ++k) {
    const double y0 = e[k], y1 = d[k + 1] - theta, y2 = (k + 2 < n) ? e[k + 1] : 0.0;
    const bool sw = fabs(x0) < fabs(y0);
    double p0 = sw ? y0 : x0;
    const double p1 = sw ? y1 : x1, p2 = sw ? y2 : x2;
    const double o0 = sw ? x0 : y0, o1 = sw ? x1 : y1, o2 = sw ? x2 : y2;
    if (fabs(p0) < tiny) p0 = (p0 < 0 ? -tiny : tiny);
    const double r = 1.0 / p0;
    const double l = o0 * r;
    const int64_t o = (int64_t)k * ld;
    P[o] = sw ? 1.0 : 0.0;
    L[o] = l;
    U0i[o] = r;
    U1[o] = p1;
    U2[o] = p2;
    x0 = o1 - l * p1;
    x1 = o2 - l * p2;
    x2 = 0.0;
  }
  if (fabs(x0) < tiny) x0 = (x0 < 0 ? -tiny : tiny);
  const int64_t o = (int64_t)(n - 1) * ld;
  U0i[o] = 1.0 / x0;
  U1[o] = 0.0;
  U2[o] = 0.0;
}

// Solve with the factors of tri_factor in place on y (stride ld).
__device__ void tri_solve(const double* U0i, const double* U1, const double* U2, const double* L,
                          const double* P, int n, int ld, double* y) {
  double yk = y[0];
  for (int k = 0; k < n - 1; ++k) {
    const int64_t o = (int64_t)k * ld;
    double yn = y[o + ld];
    if (P[o] != 0.0) { const double t = yk; yk = yn; yn = t; }
    y[o] = yk;
    yk = yn - L[o] * yk;
  }
  const int64_t ol = (int64_t)(n - 1) * ld;
  double z1 = yk * U0i[ol], z2 = 0.0;  // z_{k+1}, z_{k+2}
  y[ol] = z1;
  for (int k = n - 2; k >= 0; --k) {
    const int64_t o = (int64_t)k * ld;
    const double z = (y[o] - U1[o] * z1 - U2[o] * z2) * U0i[o];
    y[o] = z;
    z2 = z1;
    z1 = z;
  }
}

__global__ void __launch_bounds__(kEigThreads, 4) sym_eig_kernel(double* Aall, int lda,
                                                              const int32_t* nsize, int want,
                                                              double* theta_all, double* S_all,
                                                              double* work_all, size_t wstride,
                                                              const int32_t* active) {
  extern __shared__ double svec[];  // v and w of the current reflector, FP64 and double-float (4 lda)
  __shared__ double sh[32];
  __shared__ double s_tau, s_beta, s_K;
  __shared__ int s_skip;
  const int b = blockIdx.x;
  if (active && !active[b]) return;
  const int n = nsize[b];
  const int t = threadIdx.x;
  const int lane_e = t & 31, warp_e = t >> 5, nwarp_e = kEigThreads / 32;
  double* A = Aall + (int64_t)b * lda * lda;
  double* W = work_all + (int64_t)b * wstride;
  double* d = W;
  double* e = W + lda;
  double* tau = W + 2 * lda;
  double* e2 = W + 3 * lda;
  double* th = W + 4 * lda;                // want
  int* clus = (int*)(W + 4 * lda + want);  // 2 want ints: leader flags, cluster starts
  double* vecw = W + 4 * lda + 2 * want;   // 5 want lda: LU factors per eigenvalue
  double* theta = theta_all + (int64_t)b * want;
  double* S = S_all + (int64_t)b * lda * want;
  const int nw = min(want, n);

  // ---- 1. Householder tridiagonalisation (lower), A[i*lda + j].  The
  // trailing block A22 is held in double-float (the 8 bytes of an entry as
  // an FP32 pair): its product with the reflector and its rank-2 update, the
  // O(n^3) part, run on the FP32 pipe, 64x the FP64 rate here; scalars,
  // reflectors (written back as FP64 into row and column k) and the
  // tridiagonal stay FP64.
  float2* Af = reinterpret_cast<float2*>(A);
  for (int64_t q = t; q < (int64_t)n * n; q += kEigThreads) {
    const int64_t r = q / n, c = q - r * n;
    Af[r * lda + c] = df_split(A[r * lda + c]);
  }
  __syncthreads();
  for (int k = 0; k < n - 2; ++k) {
    // column k below the subdiagonal
    double s2 = 0.0;
    for (int i = k + 2 + t; i < n; i += kEigThreads) {
      const double x = df_to_double(Af[(int64_t)i * lda + k]);
      s2 += x * x;
    }
    s2 = block_sum(s2, sh);
    if (t == 0) {
      const double alpha = df_to_double(Af[(int64_t)(k + 1) * lda + k]);
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
      d[k] = df_to_double(Af[(int64_t)k * lda + k]);
    }
    __syncthreads();
    if (s_skip) continue;
    // v: v[k+1] = 1, v[i] = A[i][k] * s_beta, stored (FP64) in column k and,
    // for a contiguous copy read by the back-transformation, in row k (row
    // and column k are not touched by the later steps)
    const int m0 = k + 1;
    double* vs = svec;
    double* ws = svec + lda;
    float2* vsf = reinterpret_cast<float2*>(svec + 2 * lda);
    float2* wsf = reinterpret_cast<float2*>(svec + 3 * lda);
    for (int i = m0 + t; i < n; i += kEigThreads) {
      double vi;
      if (i == m0) vi = 1.0;
      else {
        vi = df_to_double(Af[(int64_t)i * lda + k]) * s_beta;
        A[(int64_t)i * lda + k] = vi;
      }
      A[(int64_t)k * lda + i] = vi;
      vs[i] = vi;
      vsf[i] = df_split(vi);
    }
    __syncthreads();
    // p = tau * A22 v: warp per row (A22 is kept symmetric, so row i is
    // column i), lanes along the row, two rows in flight per warp; the row
    // sums in double-float, reduced over the warp with the two-sum
    double pdot = 0.0;
    for (int i = m0 + warp_e; i < n; i += 2 * nwarp_e) {
      const int i2 = i + nwarp_e;
      const float2* Ai = Af + (int64_t)i * lda;
      const float2* Ai2 = Af + (int64_t)(i2 < n ? i2 : i) * lda;
      float h1 = 0.f, l1 = 0.f, h2 = 0.f, l2 = 0.f;
      for (int j = m0 + lane_e; j < n; j += 32) {
        const float2 vj = vsf[j];
        df_fma(Ai[j], vj, h1, l1);
        df_fma(Ai2[j], vj, h2, l2);
      }
      {
        float h = __fadd_rn(h1, l1), l = __fsub_rn(l1, __fsub_rn(h, h1));
        float g = __fadd_rn(h2, l2), m = __fsub_rn(l2, __fsub_rn(g, h2));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float bh = __shfl_xor_sync(0xffffffffu, h, o), bl = __shfl_xor_sync(0xffffffffu, l, o);
          const float ch = __shfl_xor_sync(0xffffffffu, g, o), cl = __shfl_xor_sync(0xffffffffu, m, o);
          df_add(h, l, bh, bl);
          df_add(g, m, ch, cl);
        }
        h1 = h; l1 = l; h2 = g; l2 = m;
      }
      const double a1 = ((double)h1 + (double)l1) * s_tau;
      const double a2 = ((double)h2 + (double)l2) * s_tau;
      if (lane_e == 0) {
        ws[i] = a1;
        pdot += a1 * vs[i];
        if (i2 < n) {
          ws[i2] = a2;
          pdot += a2 * vs[i2];
        }
      }
    }
    pdot = block_sum(pdot, sh);
    if (t == 0) s_K = -0.5 * s_tau * pdot;
    __syncthreads();
    for (int i = m0 + t; i < n; i += kEigThreads) {  // w
      const double wi = ws[i] + s_K * vs[i];
      ws[i] = wi;
      wsf[i] = df_split(wi);
    }
    __syncthreads();
    // A22 -= v w' + w v' in double-float: warp per row, lanes along the row
    for (int i = m0 + warp_e; i < n; i += nwarp_e) {
      float2* Ai = Af + (int64_t)i * lda;
      const float2 vi = vsf[i], wi = wsf[i];
      for (int j = m0 + lane_e; j < n; j += 32) {
        float uh = 0.f, ul = 0.f;
        df_fma(vsf[j], wi, uh, ul);
        df_fma(wsf[j], vi, uh, ul);
        float2 a = Ai[j];
        df_add(a.x, a.y, -uh, -ul);
        Ai[j] = a;
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    if (n >= 2) {
      d[n - 2] = df_to_double(Af[(int64_t)(n - 2) * lda + (n - 2)]);
      e[n - 2] = df_to_double(Af[(int64_t)(n - 1) * lda + (n - 2)]);
      tau[n - 2] = 0.0;
    }
    d[n - 1] = df_to_double(Af[(int64_t)(n - 1) * lda + (n - 1)]);
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
  // multisection: a group of G lanes per eigenvalue probes G interior points
  // of its interval and keeps the sub-interval where the count passes the
  // eigenvalue's index
  {
    int G = 1;
    while (G < 32 && 2 * G * nw <= kEigThreads) G *= 2;
    const int ngroup = kEigThreads / G, sub = t % G, gl0 = (t & 31) - sub;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gl0);
    const double frac = 1.0 / (double)(G + 1);
    for (int j = t / G; j < nw; j += ngroup) {
      const int idx = n - 1 - j;  // index from the bottom
      double lo = gl, hi = gu;
      for (int itb = 0; itb < 200; ++itb) {
        const double w = hi - lo;
        if (w <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin) break;
        const double x = lo + (double)(sub + 1) * (w * frac);
        const bool le = sturm_count(d, e2, n, x) <= idx;
        const unsigned m = (__ballot_sync(gmask, le) & gmask) >> gl0;
        // the probe just above the highest one at or below the eigenvalue
        const int kk = (m == 0u) ? 0 : 32 - __clz(m);
        const double nlo = (kk == 0) ? lo : lo + (double)kk * (w * frac);
        const double nhi = (kk == G) ? hi : lo + (double)(kk + 1) * (w * frac);
        if (nlo == lo && nhi == hi) break;
        lo = nlo;
        hi = nhi;
      }
      if (sub == 0) th[j] = 0.5 * (lo + hi);
    }
  }
  __syncthreads();

  // ---- 3. inverse iteration for all wanted eigenvalues at once (thread q
  // owns eigenvalue q); the vectors live in S (row-major, stride want) and
  // after each sweep the members of every cluster of close eigenvalues are
  // orthonormalised by modified Gram-Schmidt, one warp per cluster
  const int lane = t & 31, warp = t >> 5;
  const double ctol = 1e-7 * fmax(tnorm, DBL_MIN);
  const double tiny = DBL_EPSILON * fmax(tnorm, DBL_MIN);
  int* lead = clus + want;  // first member of every cluster
  for (int j = t; j < nw; j += kEigThreads) clus[j] = (j == 0) || (th[j - 1] - th[j] > ctol);
  __syncthreads();
  if (t == 0) {
    int c = 0;
    for (int j = 0; j < nw; ++j)
      if (clus[j]) lead[c++] = j;
    s_skip = c;  // number of clusters
  }
  double* Y = S;
  double* U0i = vecw;
  double* U1 = U0i + (int64_t)lda * want;
  double* U2 = U1 + (int64_t)lda * want;
  double* Lm = U2 + (int64_t)lda * want;
  double* Pv = Lm + (int64_t)lda * want;
  for (int q = t; q < nw; q += kEigThreads) {
    int j = q;
    while (j > 0 && !clus[j]) --j;
    // members of a cluster get shifts a few ulps apart (as LAPACK dstein)
    const double shift = th[q] - (double)(q - j) * 10.0 * DBL_EPSILON * fmax(fabs(th[j]), tnorm);
    tri_factor(d, e, n, shift, U0i + q, U1 + q, U2 + q, Lm + q, Pv + q, want, tiny);
    for (int i = 0; i < n; ++i) {  // deterministic start vector
      unsigned h = (unsigned)(i * 2654435761u) ^ (unsigned)(q * 40503u + 0x9e3779b9u);
      h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
      Y[(int64_t)i * want + q] = ((double)(h & 0xffffff) / 16777216.0) - 0.5;
    }
  }
  __syncthreads();
  const int ncl = s_skip;
  for (int itr = 0; itr < 4; ++itr) {
    for (int q = t; q < nw; q += kEigThreads) tri_solve(U0i + q, U1 + q, U2 + q, Lm + q, Pv + q, n, want, Y + q);
    __syncthreads();
    for (int c = warp; c < ncl; c += kEigThreads / 32) {
      const int j0 = lead[c], j1 = (c + 1 < ncl) ? lead[c + 1] : nw;
      for (int m = j0; m < j1; ++m) {
        for (int r = j0; r < m; ++r) {
          double dp = 0.0;
          for (int i = lane; i < n; i += 32) dp += Y[(int64_t)i * want + r] * Y[(int64_t)i * want + m];
          dp = warp_sum(dp);
          for (int i = lane; i < n; i += 32) Y[(int64_t)i * want + m] -= dp * Y[(int64_t)i * want + r];
        }
        double nrm = 0.0;
        for (int i = lane; i < n; i += 32) nrm += Y[(int64_t)i * want + m] * Y[(int64_t)i * want + m];
        nrm = warp_sum(nrm);
        const double inv = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
        for (int i = lane; i < n; i += 32) Y[(int64_t)i * want + m] *= inv;
      }
    }
    __syncthreads();
  }

  // ---- 4. back-transformation Y <- H_0 ... H_{n-3} Y, one reflector at a
  // time for all vectors (the reflector is read from its copy in row k):
  // column dots by (row part, vector) threads, then the rank-1 update.  Y is
  // held in double-float meanwhile (its O(n^2 nw) products run on the FP32
  // pipe); each reflector is split once into shared memory.
  constexpr int kBtCols = 64, kBtRows = kEigThreads / kBtCols;
  const int tx = t % kBtCols, ty = t / kBtCols;
  float2* part = reinterpret_cast<float2*>(svec);                 // kBtRows x want partial dots
  double* dps = svec + (int64_t)kBtRows * want;                   // want scaled dots
  float2* dpsf = reinterpret_cast<float2*>(dps + want);           // the same, double-float
  float2* vkf = reinterpret_cast<float2*>(dps + 2 * (int64_t)want);  // the reflector, double-float (lda)
  float2* Yf = reinterpret_cast<float2*>(Y);
  for (int i = ty; i < n; i += kBtRows)
    for (int q = tx; q < nw; q += kBtCols) Yf[(int64_t)i * want + q] = df_split(Y[(int64_t)i * want + q]);
  __syncthreads();
  for (int k = n - 3; k >= 0; --k) {
    const double tk = tau[k];
    if (tk == 0.0) continue;  // uniform: tau is in global memory, read by all
    const double* vk = A + (int64_t)k * lda;  // vk[k+1] = 1
    for (int i = k + 1 + t; i < n; i += kEigThreads) vkf[i] = df_split(vk[i]);
    __syncthreads();
    for (int q = tx; q < nw; q += kBtCols) {
      float h = 0.f, l = 0.f;
      for (int i = k + 1 + ty; i < n; i += kBtRows) df_fma(vkf[i], Yf[(int64_t)i * want + q], h, l);
      const float hh = __fadd_rn(h, l);
      part[ty * want + q] = make_float2(hh, __fsub_rn(l, __fsub_rn(hh, h)));
    }
    __syncthreads();
    for (int q = t; q < nw; q += kEigThreads) {
      float h = 0.f, l = 0.f;
      for (int r = 0; r < kBtRows; ++r) df_add(h, l, part[r * want + q].x, part[r * want + q].y);
      const double d = tk * ((double)h + (double)l);
      dps[q] = d;
      dpsf[q] = df_split(d);
    }
    __syncthreads();
    for (int i = k + 1 + ty; i < n; i += kBtRows) {
      const float2 vi = vkf[i];
      for (int q = tx; q < nw; q += kBtCols) {
        float uh = 0.f, ul = 0.f;
        df_fma(dpsf[q], vi, uh, ul);
        float2 y = Yf[(int64_t)i * want + q];
        df_add(y.x, y.y, -uh, -ul);
        Yf[(int64_t)i * want + q] = y;
      }
    }
    __syncthreads();
  }
  for (int i = ty; i < n; i += kBtRows)
    for (int q = tx; q < nw; q += kBtCols) Y[(int64_t)i * want + q] = df_to_double(Yf[(int64_t)i * want + q]);
  __syncthreads();
  // rows beyond n and columns beyond nw (if want > n) are zero
  for (int i = ty; i < lda; i += kBtRows)
    for (int q = tx; q < want; q += kBtCols)
      if (i >= n || q >= nw) Y[(int64_t)i * want + q] = 0.0;
  for (int q = t; q < want; q += kEigThreads) theta[q] = (q < nw) ? th[q] : 0.0;
}

int sym_eig_top(int nmat, double* A, int lda, const int32_t* nsize, int want, double* theta,
                double* S, double* work, const int32_t* active, cudaStream_t stream) {
  if (nmat <= 0) return LAPY_OK;
  // v and w of a reflector in FP64 and double-float (4 lda); partial dots,
  // scaled dots and the double-float reflector of the back-transformation
  // (6 want + lda)
  const size_t smem = sizeof(double) * std::max<size_t>(4 * (size_t)lda, 6 * (size_t)want + (size_t)lda);
  if (smem > 48 * 1024) {
    LAPY_CUDA_TRY(cudaFuncSetAttribute(sym_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  sym_eig_kernel<<<nmat, kEigThreads, smem, stream>>>(A, lda, nsize, want, theta, S, work,
                                                     sym_eig_work_doubles(lda, want), active);
  return lapy_check_launch("sym_eig_kernel");
}

}  // namespace lapy
