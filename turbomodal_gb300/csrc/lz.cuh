// Device kernels of the shift-invert Lanczos eigensolver, batched over B problems that
// advance in lockstep (FP64 vectors; per-problem scalars stay on the device).
//
// Every vector argument is a batch base pointer with a per-problem stride; scalar arrays
// (alpha, beta, dots, ...) are laid out problem-major.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace tmg {

// CSR matrix with a shared pattern and per-problem values (val + p * vstride).
template <typename T>
struct DevCsr {
    int32_t nrows = 0;
    int64_t nnz = 0;
    const int64_t* rowptr = nullptr;
    const int32_t* col = nullptr;
    const T* val = nullptr;
    int64_t vstride = 0;
};

constexpr int LZ_DOT_BLOCKS = 152;
constexpr int LZ_MAXM = 512;      // largest Lanczos subspace (tridiagonal size) the kernels handle

// y[p](:, v) = A[p] x[p](:, v)   (or y -= A x); vectors of length A.nrows at x + p*xs + v*ld
template <typename T>
void lz_spmv(cudaStream_t st, int B, const DevCsr<T>& A, const T* x, int64_t xs, T* y, int64_t ys, int nvec, int64_t ld,
             bool subtract = false);

// out[p*K + k] = sum_i conj(A[p*as + k*lda + i]) * y[p*ys + i]; partial: >= B*K*LZ_DOT_BLOCKS
template <typename T>
void lz_multidot(cudaStream_t st, int B, int64_t n, const T* A, int64_t as, int64_t lda, int K, const T* y, int64_t ys,
                 T* partial, T* out);

// alpha[p*ldab + j] = re(dot[p]); w -= alpha_j v_j + beta_{j-1} v_{j-1}
template <typename T>
void lz_three_term(cudaStream_t st, int B, int64_t n, int j, const T* dot, double* alpha, const double* beta, int ldab,
                   const T* V, int64_t vs, T* w, int64_t ws);
// w[p] -= V[p](:, 0:K) h[p*ldh : ...]
template <typename T>
void lz_gemv_sub(cudaStream_t st, int B, int64_t n, int K, const T* V, int64_t vs, const T* h, int ldh, T* w, int64_t ws);
// beta_j = sqrt|re(dot)|, v_{j+1} = w / beta_j, Mv_{j+1} = Mw / beta_j; flag[p] = j+1 on breakdown
template <typename T>
void lz_beta_scale(cudaStream_t st, int B, int64_t n, int j, const T* dot, const T* w, const T* Mw, int64_t ws, T* V,
                   T* MV, int64_t vs, double* beta, int ldab, int* flag);
// v_0, Mv_0 /= sqrt(re(dot)) (first basis vector)
template <typename T>
void lz_scale_first(cudaStream_t st, int B, int64_t n, const T* dot, T* V, T* MV, int64_t vs);

// Tridiagonal eigenproblem of each problem (one CTA per problem): theta ascending,
// S (m x m column-major), lambda = shift + 1/theta, order (by lambda), nconv.  `shifts`
// (device, one per problem) replaces `shift` when given.
void lz_tridiag(cudaStream_t st, int B, int m, int ldab, int nev, double shift, double tol, const double* alpha,
                const double* beta, double* theta, double* S, double* lam, int* order, int* nconv, double* Z,
                const double* shifts = nullptr);

// Implicit restart QR sweeps of each problem; Q: m x m per problem; rot: scratch per problem
void lz_restart_qr(cudaStream_t st, int B, int m, int ldab, int nev, const double* theta, double* alpha, double* beta,
                   double* Q, double* rot, int64_t rot_stride);

// Y[p](:, c) = sum_k X[p](:, k) C[p*cs + k + c*ldc], c < ncol
template <typename T>
void lz_gemm_real(cudaStream_t st, int B, int64_t n, int K, int ncol, const T* X, int64_t xs, const double* C, int64_t cs,
                  int ldc, T* Y, int64_t ys);

// f = beta[nev-1] * Y + beta[m-1] * Q(m-1, nev-1) * v   (per problem)
template <typename T>
void lz_combine_f(cudaStream_t st, int B, int64_t n, const T* Y, int64_t ys, const T* v, int64_t vs, const double* beta,
                  int ldab, int nev, int m, const double* Q, T* f, int64_t fs);

// continuation vector normalisation of the restart (src/hermitian_lanczos.cpp:243-254)
template <typename T>
void lz_restart_norm(cudaStream_t st, int B, int64_t n, int nev, const T* dot, const T* f, const T* Mf, int64_t fs, T* V,
                     T* MV, int64_t vs, double* beta, int ldab);

template <typename T>
void lz_copy(cudaStream_t st, int64_t n, const T* src, T* dst);
// ||x[p]||^2 -> out[p]
template <typename T>
void lz_norm2(cudaStream_t st, int B, int64_t n, const T* x, int64_t xs, double* partial, double* out);

}  // namespace tmg
