// Dense generalized Hermitian eigensolver for small harmonic problems (n <= 200).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace tmg {

// D (n x n, column-major, complex) <- the CSC matrix (device arrays); D is zeroed first.
void dense_csc_to_dense(cudaStream_t st, int32_t n, const int64_t* colptr, const int32_t* rowind, const zd* vals,
                        zd* D);

// For each of B problems (problem-major n x n blocks K, M): the nev smallest eigenpairs of
// K x = lambda M x.  work: B * 5 * n * n; lam, res: B * nev; X: B * n * nev (column-major per
// problem, M-orthonormal columns); status[p] = 1 when M is not positive definite.
void dense_geig(cudaStream_t st, int B, int n, int nev, const zd* K, const zd* M, zd* work, double* lam, zd* X,
                double* res, int* status);

}  // namespace tmg
