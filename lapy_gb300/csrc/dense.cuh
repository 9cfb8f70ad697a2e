// Batched small dense FP64 linear algebra for the Lanczos Ritz steps.
#pragma once
#include "common.cuh"

namespace lapy {

// Top-`want` eigenpairs (largest eigenvalues first) of `nmat` symmetric n_b x n_b
// matrices.  Matrix b lives at A + b*lda*lda (row-major, leading dimension lda,
// overwritten).  n_b = nsize[b] (device array) <= lda.  Output: theta[b*want + i]
// (descending), S[b*lda*want + r*want + i] eigenvector i, row r (rows >= n_b zero).
// Scratch `work` must hold sym_eig_work_doubles(lda, want) doubles per matrix.
size_t sym_eig_work_doubles(int lda, int want);
int sym_eig_top(int nmat, double* A, int lda, const int32_t* nsize, int want, double* theta,
                double* S, double* work, const int32_t* active, cudaStream_t stream);

}  // namespace lapy
