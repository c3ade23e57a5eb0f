// Device kernels of the shift-invert Lanczos eigensolver (FP64 vectors).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace tmg {

// CSR matrix on the device with values of type T.
template <typename T>
struct DevCsr {
    int32_t nrows = 0;
    int64_t nnz = 0;
    const int64_t* rowptr = nullptr;
    const int32_t* col = nullptr;
    const T* val = nullptr;
};

// y(:,v) = A x(:,v) (or y -= A x), ld = leading dimension of x and y.
template <typename T>
void lz_spmv(cudaStream_t st, const DevCsr<T>& A, const T* x, T* y, int nvec, int64_t ld, bool subtract = false);

// out[k] = sum_i conj(A[k*lda + i]) * y[i], k < K  (partials buffer: >= nblk * K entries)
template <typename T>
void lz_multidot(cudaStream_t st, int64_t n, const T* A, int64_t lda, int K, const T* y, T* partial, T* out);
constexpr int LZ_DOT_BLOCKS = 152;

// Lanczos step pieces (scalars live on the device).
// alpha_j = re(dot); w -= alpha_j v_j + beta_{j-1} v_{j-1}
template <typename T>
void lz_three_term_dot(cudaStream_t st, int64_t n, int j, const T* dot, double* alpha, const double* beta, const T* V,
                       T* w);
template <typename T>
void lz_gemv_sub(cudaStream_t st, int64_t n, int K, const T* V, const T* h, T* w);
template <typename T>
void lz_beta_scale(cudaStream_t st, int64_t n, int j, const T* dot, const T* w, const T* Mw, T* V, T* MV, double* beta,
                   int* flag);
template <typename T>
void lz_scale_cols(cudaStream_t st, int64_t n, const T* dot, T* x, T* Mx);   // x, Mx /= sqrt(re(dot))

// Tridiagonal eigenproblem of (alpha, beta) of size m on one CTA: theta ascending,
// S (m x m column-major), lambda = shift + 1/theta, order (by lambda), nconv.
void lz_tridiag(cudaStream_t st, int m, int nev, double shift, double tol, const double* alpha, const double* beta,
                double* theta, double* S, double* lam, int* order, int* nconv, double* work);

// Implicit restart: QR shift sweeps on (alpha, beta) with the m-nev smallest theta,
// accumulating Q (m x m column-major).  rot: scratch of 2*(m-nev)*(m-1) doubles.
void lz_restart_qr(cudaStream_t st, int m, int nev, const double* theta, double* alpha, double* beta, double* Q,
                   double* rot);

// Y(:, c) = sum_k X(:, k) * C[k + c*ldc], c < ncol (complex/real X, real C)
template <typename T>
void lz_gemm_real(cudaStream_t st, int64_t n, int K, int ncol, const T* X, const double* C, int ldc, T* Y);

// f = beta[nev-1] * Y + beta[m-1] * Q(m-1, nev-1) * v  (scalars read on the device; beta[m-1]
// is the dangling coefficient, untouched by the QR sweeps)
template <typename T>
void lz_combine_f(cudaStream_t st, int64_t n, const T* Y, const T* v, const double* beta, int nev, int m,
                  const double* Q, T* f);

template <typename T>
void lz_copy(cudaStream_t st, int64_t n, const T* src, T* dst);
template <typename T>
void lz_axpy(cudaStream_t st, int64_t n, double a, const T* x, T* y);     // y += a x
template <typename T>
void lz_sub(cudaStream_t st, int64_t n, const T* b, const T* ax, T* r);   // r = b - ax
template <typename T>
void lz_norm2(cudaStream_t st, int64_t n, const T* x, double* partial, double* out);   // out = ||x||^2

}  // namespace tmg
