// CSR helpers: diagonal positions, pattern maps, mean edge length.
#include "common.cuh"

namespace lapy {

__global__ void diag_index_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                  const int32_t* __restrict__ indices, int32_t* __restrict__ pos) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int32_t lo = indptr[r], hi = indptr[r + 1] - 1, found = -1;
  while (lo <= hi) {  // indices are sorted inside each row
    const int32_t mid = (lo + hi) >> 1;
    const int32_t c = indices[mid];
    if (c == (int32_t)r) { found = mid; break; }
    if (c < (int32_t)r) lo = mid + 1; else hi = mid - 1;
  }
  pos[r] = found;
}

__global__ void pattern_map_kernel(int64_t n, const int32_t* __restrict__ a_ptr,
                                   const int32_t* __restrict__ a_idx,
                                   const int32_t* __restrict__ b_ptr,
                                   const int32_t* __restrict__ b_idx, int32_t* __restrict__ pos,
                                   int* missing) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int32_t k = b_ptr[r]; k < b_ptr[r + 1]; ++k) {
    const int32_t c = b_idx[k];
    int32_t lo = a_ptr[r], hi = a_ptr[r + 1] - 1, found = -1;
    while (lo <= hi) {
      const int32_t mid = (lo + hi) >> 1;
      const int32_t ac = a_idx[mid];
      if (ac == c) { found = mid; break; }
      if (ac < c) lo = mid + 1; else hi = mid - 1;
    }
    pos[k] = found;
    if (found < 0) atomicExch(missing, 1);
  }
}

constexpr int kEdgeBlocks = 1024;

// Sum of edge lengths (strict upper triangle) and edge count, per block.
template <typename T>
__global__ void edge_len_kernel(const T* __restrict__ v, int64_t n, const int32_t* __restrict__ indptr,
                                const int32_t* __restrict__ indices, double* __restrict__ psum,
                                long long* __restrict__ pcnt) {
  __shared__ double sh[32];
  __shared__ long long shc[32];
  double s = 0.0;
  long long c = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const T x0 = v[3 * r], y0 = v[3 * r + 1], z0 = v[3 * r + 2];
    for (int32_t k = indptr[r]; k < indptr[r + 1]; ++k) {
      const int32_t j = indices[k];
      if (j <= r) continue;
      const T dx = x0 - v[3 * (int64_t)j], dy = y0 - v[3 * (int64_t)j + 1],
              dz = z0 - v[3 * (int64_t)j + 2];
      // tria_mesh.py:745-747: sqrt(((v_i - v_j) ** 2).sum(1)) in the coordinate type
      T q = dx * dx;
      q = q + dy * dy;
      q = q + dz * dz;
      s += (double)sqrt(q);
      c += 1;
    }
  }
  s = block_sum(s, sh);
  c = block_sum(c, shc);
  if (threadIdx.x == 0) {
    psum[blockIdx.x] = s;
    pcnt[blockIdx.x] = c;
  }
}

__global__ void edge_len_final_kernel(const double* psum, const long long* pcnt, int nb, double* out) {
  __shared__ double sh[32];
  __shared__ long long shc[32];
  double s = 0.0;
  long long c = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    s += psum[i];
    c += pcnt[i];
  }
  s = block_sum(s, sh);
  c = block_sum(c, shc);
  if (threadIdx.x == 0) out[0] = c ? s / (double)c : 0.0;
}

// One CTA per segment: mean edge length of the segment's strict upper
// triangle, summed in a fixed order (thread-strided rows, then block_sum).
template <typename T>
__global__ void seg_edge_len_kernel(const T* __restrict__ v, const int32_t* __restrict__ seg_row,
                                    const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                                    double m, double* __restrict__ out, double* __restrict__ t_out) {
  __shared__ double sh[32];
  __shared__ long long shc[32];
  const int s = blockIdx.x;
  double acc = 0.0;
  long long c = 0;
  for (int64_t r = seg_row[s] + threadIdx.x; r < seg_row[s + 1]; r += blockDim.x) {
    const T x0 = v[3 * r], y0 = v[3 * r + 1], z0 = v[3 * r + 2];
    for (int32_t k = indptr[r]; k < indptr[r + 1]; ++k) {
      const int32_t j = indices[k];
      if (j <= r) continue;
      const T dx = x0 - v[3 * (int64_t)j], dy = y0 - v[3 * (int64_t)j + 1], dz = z0 - v[3 * (int64_t)j + 2];
      T q = dx * dx;
      q = q + dy * dy;
      q = q + dz * dz;
      acc += (double)sqrt(q);
      c += 1;
    }
  }
  acc = block_sum(acc, sh);
  c = block_sum(c, shc);
  if (threadIdx.x == 0) {
    const double avg = c ? acc / (double)c : 0.0;
    out[s] = avg;
    if (t_out) t_out[s] = __dmul_rn(m, __dmul_rn(avg, avg));  // lapy/heat.py:206
  }
}

// out = alpha[s] x + beta[s] y on the rows of segment s (one CTA per
// segment); y_is_diag: y is an n-vector added at the diagonal positions.
__global__ void seg_axpby_kernel(const int32_t* __restrict__ seg_row, const int32_t* __restrict__ indptr,
                                 const int32_t* __restrict__ diag_pos, const double* __restrict__ alpha,
                                 const double* __restrict__ x, const double* __restrict__ beta,
                                 const double* __restrict__ y, int y_is_diag, double* __restrict__ out) {
  const int s = blockIdx.x;
  const double a = alpha[s], b = beta[s];
  const int32_t k0 = indptr[seg_row[s]], k1 = indptr[seg_row[s + 1]];
  for (int32_t k = k0 + threadIdx.x; k < k1; k += blockDim.x)
    out[k] = y_is_diag ? __dmul_rn(a, x[k]) : __dadd_rn(__dmul_rn(a, x[k]), __dmul_rn(b, y[k]));
  if (y_is_diag) {
    __syncthreads();
    for (int32_t r = seg_row[s] + threadIdx.x; r < seg_row[s + 1]; r += blockDim.x)
      out[diag_pos[r]] = __dadd_rn(out[diag_pos[r]], __dmul_rn(b, y[r]));
  }
}

}  // namespace lapy

using namespace lapy;

extern "C" int lapy_seg_avg_edge_length(const void* v, int coords_f32, int nseg, const int32_t* seg_row,
                                        const int32_t* indptr, const int32_t* indices, double m, double* out,
                                        double* t_out, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!v || nseg <= 0 || !seg_row || !indptr || !indices || !out) return LAPY_ERR_INVALID;
  if (coords_f32)
    seg_edge_len_kernel<float><<<nseg, 256, 0, stream>>>((const float*)v, seg_row, indptr, indices, m, out, t_out);
  else
    seg_edge_len_kernel<double><<<nseg, 256, 0, stream>>>((const double*)v, seg_row, indptr, indices, m, out, t_out);
  return lapy_check_launch("seg_edge_len_kernel");
}

extern "C" int lapy_csr_seg_axpby(int nseg, const int32_t* seg_row, const int32_t* indptr,
                                  const int32_t* diag_pos, const double* alpha, const double* x,
                                  const double* beta, const double* y, int y_is_diag, double* out,
                                  void* stream_) {
  if (nseg <= 0 || !seg_row || !indptr || !alpha || !x || !beta || !y || !out || (y_is_diag && !diag_pos))
    return LAPY_ERR_INVALID;
  seg_axpby_kernel<<<nseg, 256, 0, (cudaStream_t)stream_>>>(seg_row, indptr, diag_pos, alpha, x, beta, y,
                                                             y_is_diag, out);
  return lapy_check_launch("seg_axpby_kernel");
}

extern "C" int lapy_csr_diag_index(int64_t n, const int32_t* indptr, const int32_t* indices,
                                   int32_t* diag_pos, void* stream) {
  if (n <= 0 || !indptr || !indices || !diag_pos) return LAPY_ERR_INVALID;
  diag_index_kernel<<<lapy_ceil_div(n, 256), 256, 0, (cudaStream_t)stream>>>(n, indptr, indices, diag_pos);
  return lapy_check_launch("diag_index_kernel");
}

extern "C" int lapy_csr_pattern_map(int64_t n, const int32_t* a_indptr, const int32_t* a_indices,
                                    const int32_t* b_indptr, const int32_t* b_indices, int64_t b_nnz,
                                    int32_t* pos, void* work, void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (n <= 0 || !a_indptr || !a_indices || !b_indptr || !b_indices || !pos || b_nnz < 0 || !work)
    return LAPY_ERR_INVALID;
  int* flag = (int*)work;
  LAPY_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), stream));
  pattern_map_kernel<<<lapy_ceil_div(n, 256), 256, 0, stream>>>(n, a_indptr, a_indices, b_indptr,
                                                                b_indices, pos, flag);
  LAPY_TRY(lapy_check_launch("pattern_map_kernel"));
  int missing = 0;
  LAPY_CUDA_TRY(cudaMemcpyAsync(&missing, flag, sizeof(int), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  if (missing) {
    lapy_set_last_message("csr_pattern_map: an entry of the second matrix is not in A's pattern");
    return LAPY_ERR_PATTERN;
  }
  return LAPY_OK;
}

extern "C" size_t lapy_avg_edge_length_workspace_bytes(int64_t n) {
  (void)n;
  return kEdgeBlocks * (sizeof(double) + sizeof(long long)) + 512;
}

extern "C" int lapy_avg_edge_length(const void* v, int coords_f32, int64_t n, const int32_t* indptr,
                                    const int32_t* indices, double* out, void* work, size_t ws_bytes,
                                    void* stream_) {
  cudaStream_t stream = (cudaStream_t)stream_;
  if (!v || n <= 0 || !indptr || !indices || !out || !work) return LAPY_ERR_INVALID;
  if (ws_bytes < lapy_avg_edge_length_workspace_bytes(n)) return LAPY_ERR_WORKSPACE;
  char* base = (char*)(((uintptr_t)work + 255) & ~uintptr_t(255));
  double* psum = (double*)base;
  long long* pcnt = (long long*)(base + kEdgeBlocks * sizeof(double));
  double* dout = (double*)(base + kEdgeBlocks * (sizeof(double) + sizeof(long long)));
  const unsigned nb = (unsigned)std::min<int64_t>(kEdgeBlocks, std::max<int64_t>(1, lapy_ceil_div(n, 256)));
  if (coords_f32)
    edge_len_kernel<float><<<nb, 256, 0, stream>>>((const float*)v, n, indptr, indices, psum, pcnt);
  else
    edge_len_kernel<double><<<nb, 256, 0, stream>>>((const double*)v, n, indptr, indices, psum, pcnt);
  LAPY_TRY(lapy_check_launch("edge_len_kernel"));
  edge_len_final_kernel<<<1, 256, 0, stream>>>(psum, pcnt, (int)nb, dout);
  LAPY_TRY(lapy_check_launch("edge_len_final_kernel"));
  LAPY_CUDA_TRY(cudaMemcpyAsync(out, dout, sizeof(double), cudaMemcpyDeviceToHost, stream));
  LAPY_CUDA_TRY(cudaStreamSynchronize(stream));
  return LAPY_OK;
}

// ---- batch construction ------------------------------------------------------
// Element connectivity of concatenated meshes: t_out (m x npe int32) = t_in
// (each mesh's own vertex indices, int32 or int64) + seg_row[s] for the mesh
// s whose element range [seg_elem[s], seg_elem[s+1]) holds the element.
// Indices outside [0, rows of the mesh) set *bad; seg_max[s] receives the
// largest index of mesh s (so the host can check that every vertex is used).
template <typename I>
__global__ void seg_offset_elements_kernel(int64_t m, int npe, int nseg, const int32_t* __restrict__ seg_elem,
                                           const int32_t* __restrict__ seg_row, const I* __restrict__ t_in,
                                           int32_t* __restrict__ t_out, int* __restrict__ seg_max,
                                           int* __restrict__ bad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m) return;
  int lo = 0, hi = nseg - 1;  // largest s with seg_elem[s] <= e
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((int64_t)seg_elem[mid] <= e) lo = mid; else hi = mid - 1;
  }
  const int32_t off = seg_row[lo], rows = seg_row[lo + 1] - off;
  int mx = -1;
  for (int c = 0; c < npe; ++c) {
    const I x = t_in[e * npe + c];
    if (x < 0 || x >= (I)rows) {
      atomicOr(bad, 1);
      t_out[e * npe + c] = off;
    } else {
      t_out[e * npe + c] = off + (int32_t)x;
      mx = max(mx, (int)x);
    }
  }
  atomicMax(&seg_max[lo], mx);
}

// out[seg_row[s] + vid[s]] = 1 for every segment s (out zeroed before).
__global__ void seg_unit_set_kernel(int nseg, const int32_t* __restrict__ seg_row, const int32_t* __restrict__ vid,
                                    double* __restrict__ out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nseg) out[(int64_t)seg_row[s] + vid[s]] = 1.0;
}

extern "C" int lapy_seg_offset_elements(int64_t m, int npe, int nseg, const int32_t* seg_elem,
                                        const int32_t* seg_row, const void* t_in, int idx64, int32_t* t_out,
                                        int32_t* seg_max, void* stream) {
  if (m < 0 || npe <= 0 || nseg <= 0 || !seg_elem || !seg_row || !seg_max || (m > 0 && (!t_in || !t_out)))
    return LAPY_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  // seg_max[nseg] doubles as the out-of-range flag
  LAPY_CUDA_TRY(cudaMemsetAsync(seg_max, 0xff, sizeof(int32_t) * (size_t)nseg, st));
  LAPY_CUDA_TRY(cudaMemsetAsync(seg_max + nseg, 0, sizeof(int32_t), st));
  if (m == 0) return LAPY_OK;
  const unsigned nb = lapy_ceil_div(m, 256);
  if (idx64)
    seg_offset_elements_kernel<int64_t><<<nb, 256, 0, st>>>(m, npe, nseg, seg_elem, seg_row, (const int64_t*)t_in,
                                                            t_out, seg_max, seg_max + nseg);
  else
    seg_offset_elements_kernel<int32_t><<<nb, 256, 0, st>>>(m, npe, nseg, seg_elem, seg_row, (const int32_t*)t_in,
                                                            t_out, seg_max, seg_max + nseg);
  return lapy_check_launch("seg_offset_elements_kernel");
}

extern "C" int lapy_seg_unit_vector(int64_t n, int nseg, const int32_t* seg_row, const int32_t* vid, double* out,
                                    void* stream) {
  if (n <= 0 || nseg <= 0 || !seg_row || !vid || !out) return LAPY_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  LAPY_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)n, st));
  seg_unit_set_kernel<<<lapy_ceil_div(nseg, 256), 256, 0, st>>>(nseg, seg_row, vid, out);
  return lapy_check_launch("seg_unit_set_kernel");
}
