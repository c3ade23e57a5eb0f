// Lanczos eigensolver device kernels: sparse matrix-vector products with the shared
// projection matrices, deterministic two-stage reductions, classical Gram-Schmidt
// reorthogonalisation, and the small FP64 tridiagonal problems (eigen-decomposition by
// implicit QL, implicit-restart QR sweeps) on one CTA.
#include <algorithm>

#include "lz.cuh"

namespace tmg {

template <typename T>
__global__ void k_spmv(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                       const T* __restrict__ av, const T* __restrict__ x, T* __restrict__ y, int64_t ld, int sub) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nrows) return;
    const int64_t v = blockIdx.y;
    const T* xv = x + v * ld;
    T s = zero_of<T>();
    for (int64_t p = rp[i]; p < rp[i + 1]; p++) s += av[p] * xv[ci[p]];
    if (sub) y[v * ld + i] -= s;
    else y[v * ld + i] = s;
}

template <typename T>
void lz_spmv(cudaStream_t st, const DevCsr<T>& A, const T* x, T* y, int nvec, int64_t ld, bool subtract) {
    if (A.nrows == 0 || nvec == 0) return;
    TMG_LAUNCH(k_spmv<T>, dim3((unsigned)ceil_div(A.nrows, 128), nvec), 128, 0, st, A.nrows, A.rowptr, A.col, A.val,
               x, y, ld, subtract ? 1 : 0);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__device__ T block_sum(T v, T* sh) {
    using R = typename real_of<T>::type;
    // warp tree then first warp
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        R* p = reinterpret_cast<R*>(&v);
        p[0] += __shfl_down_sync(0xffffffff, p[0], o);
        if constexpr (sizeof(T) == 2 * sizeof(R)) p[1] += __shfl_down_sync(0xffffffff, p[1], o);
    }
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    T r = zero_of<T>();
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) r += sh[q];
    __syncthreads();
    return r;
}

template <typename T>
__global__ void __launch_bounds__(256) k_multidot1(int64_t n, const T* __restrict__ A, int64_t lda, int K,
                                                   const T* __restrict__ y, T* __restrict__ partial) {
    __shared__ T sh[8];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    for (int k = 0; k < K; k++) {
        T s = zero_of<T>();
        for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += conj(A[k * lda + i]) * y[i];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) partial[(int64_t)k * gridDim.x + blockIdx.x] = s;
    }
}

template <typename T>
__global__ void k_multidot2(int K, int nb, const T* __restrict__ partial, T* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    T s = zero_of<T>();
    for (int b = 0; b < nb; b++) s += partial[(int64_t)k * nb + b];
    out[k] = s;
}

template <typename T>
void lz_multidot(cudaStream_t st, int64_t n, const T* A, int64_t lda, int K, const T* y, T* partial, T* out) {
    TMG_LAUNCH(k_multidot1<T>, LZ_DOT_BLOCKS, 256, 0, st, n, A, lda, K, y, partial);
    TMG_LAUNCH(k_multidot2<T>, (unsigned)ceil_div(K, 128), 128, 0, st, K, LZ_DOT_BLOCKS, partial, out);
    TMG_CHECK_LAUNCH();
}

// w -= alpha_j v_j + beta_{j-1} v_{j-1}; alpha_j = re(dot) stored by thread 0
template <typename T>
__global__ void k_three_term(int64_t n, int j, const T* __restrict__ dot, double* __restrict__ alpha,
                             const double* __restrict__ beta, const T* __restrict__ V, T* __restrict__ w) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const double a = re(dot[0]);
    if (i == 0) alpha[j] = a;
    if (i >= n) return;
    T v = w[i] - a * V[(int64_t)j * n + i];
    if (j > 0) v = v - beta[j - 1] * V[(int64_t)(j - 1) * n + i];
    w[i] = v;
}
template <typename T>
void lz_three_term_dot(cudaStream_t st, int64_t n, int j, const T* dot, double* alpha, const double* beta, const T* V,
                       T* w) {
    TMG_LAUNCH(k_three_term<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, j, dot, alpha, beta, V, w);
    TMG_CHECK_LAUNCH();
}

// w -= V(:, 0:K) h
template <typename T>
__global__ void k_gemv_sub(int64_t n, int K, const T* __restrict__ V, const T* __restrict__ h, T* __restrict__ w) {
    __shared__ T hs[256];
    for (int k = threadIdx.x; k < K && k < 256; k += blockDim.x) hs[k] = h[k];
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = zero_of<T>();
    for (int k = 0; k < K; k++) acc += V[(int64_t)k * n + i] * hs[k];
    w[i] -= acc;
}
template <typename T>
void lz_gemv_sub(cudaStream_t st, int64_t n, int K, const T* V, const T* h, T* w) {
    TMG_LAUNCH(k_gemv_sub<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, K, V, h, w);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_beta_scale(int64_t n, int j, const T* __restrict__ dot, const T* __restrict__ w,
                             const T* __restrict__ Mw, T* __restrict__ V, T* __restrict__ MV, double* __restrict__ beta,
                             int* __restrict__ flag) {
    const double b = sqrt(fabs(re(dot[0])));
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i == 0) {
        beta[j] = b;
        if (b < 1e-14 && flag[0] == 0) flag[0] = j + 1;
    }
    if (i >= n) return;
    const double ib = 1.0 / b;
    V[(int64_t)(j + 1) * n + i] = ib * w[i];
    MV[(int64_t)(j + 1) * n + i] = ib * Mw[i];
}
template <typename T>
void lz_beta_scale(cudaStream_t st, int64_t n, int j, const T* dot, const T* w, const T* Mw, T* V, T* MV, double* beta,
                   int* flag) {
    TMG_LAUNCH(k_beta_scale<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, j, dot, w, Mw, V, MV, beta, flag);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_scale_cols(int64_t n, const T* __restrict__ dot, T* __restrict__ x, T* __restrict__ Mx) {
    const double s = sqrt(re(dot[0]));
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = x[i] / s;
    Mx[i] = Mx[i] / s;
}
template <typename T>
void lz_scale_cols(cudaStream_t st, int64_t n, const T* dot, T* x, T* Mx) {
    TMG_LAUNCH(k_scale_cols<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, dot, x, Mx);
    TMG_CHECK_LAUNCH();
}

// ------------------------------------------------------------------------------------
// Tridiagonal eigenproblem (implicit QL with eigenvectors, EISPACK tql2 formulation).
// Thread 0 runs the scalar recurrences and records each sweep's rotations; every thread
// then applies the sweep to its own row of Z.
__global__ void __launch_bounds__(256) k_tridiag(int m, int nev, double shift, double tol,
                                                 const double* __restrict__ alpha, const double* __restrict__ beta,
                                                 double* __restrict__ theta, double* __restrict__ S,
                                                 double* __restrict__ lam, int* __restrict__ order,
                                                 int* __restrict__ nconv, double* __restrict__ Z) {
    __shared__ double d[256], e[256], rc[256], rs[256], lamv[256];
    __shared__ int perm[256], ord[256];
    __shared__ int s_l, s_m, s_go, s_lo, s_hi;
    const int k = threadIdx.x;
    for (int c = 0; c < m; c++)
        if (k < m) Z[(int64_t)c * m + k] = (c == k) ? 1.0 : 0.0;
    if (k < m) { d[k] = alpha[k]; e[k] = (k < m - 1) ? beta[k] : 0.0; }
    __syncthreads();
    const double eps = 2.220446049250313e-16;
    double f = 0.0, tst1 = 0.0;   // meaningful in thread 0 only
    for (int l = 0; l < m; l++) {
        if (k == 0) {
            tst1 = fmax(tst1, fabs(d[l]) + fabs(e[l]));
            int mm = l;
            while (mm < m) {
                if (fabs(e[mm]) <= eps * tst1) break;
                mm++;
            }
            s_m = mm;
            s_go = (mm > l) ? 1 : 0;
        }
        __syncthreads();
        int iter = 0;
        while (s_go) {
            if (k == 0) {
                const int mm = s_m;
                iter++;
                double g = d[l];
                double p = (d[l + 1] - g) / (2.0 * e[l]);
                double r = hypot(p, 1.0);
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < m; i++) d[i] -= h;
                f = f + h;
                p = d[mm];
                double c = 1.0, c2 = c, c3 = c;
                const double el1 = e[l + 1];
                double s = 0.0, s2 = 0.0;
                for (int i = mm - 1; i >= l; i--) {
                    c3 = c2; c2 = c; s2 = s;
                    g = c * e[i];
                    h = c * p;
                    r = hypot(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    rc[i] = c;
                    rs[i] = s;
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
                s_lo = l;
                s_hi = mm - 1;
                s_go = (fabs(e[l]) > eps * tst1 && iter < 200) ? 1 : 0;
            }
            __syncthreads();
            if (k < m) {
                for (int i = s_hi; i >= s_lo; i--) {
                    const double c = rc[i], s = rs[i];
                    const double h = Z[(int64_t)(i + 1) * m + k];
                    const double zi = Z[(int64_t)i * m + k];
                    Z[(int64_t)(i + 1) * m + k] = s * zi + c * h;
                    Z[(int64_t)i * m + k] = c * zi - s * h;
                }
            }
            __syncthreads();
        }
        if (k == 0) { d[l] = d[l] + f; e[l] = 0.0; }
        __syncthreads();
    }
    if (k == 0) {
        for (int i = 0; i < m; i++) perm[i] = i;
        for (int i = 0; i < m - 1; i++) {   // selection sort ascending, as tql2's final pass
            int kk = i;
            double p = d[perm[i]];
            for (int j = i + 1; j < m; j++)
                if (d[perm[j]] < p) { kk = j; p = d[perm[j]]; }
            if (kk != i) { const int t = perm[i]; perm[i] = perm[kk]; perm[kk] = t; }
        }
        for (int i = 0; i < m; i++) {
            const double th = d[perm[i]];
            lamv[i] = fabs(th) > 1e-15 ? shift + 1.0 / th : 1e30;
            ord[i] = i;
        }
        for (int i = 1; i < m; i++) {       // stable insertion sort by lambda
            const int v = ord[i];
            int j = i - 1;
            while (j >= 0 && lamv[ord[j]] > lamv[v]) { ord[j + 1] = ord[j]; j--; }
            ord[j + 1] = v;
        }
    }
    __syncthreads();
    if (k < m) {
        theta[k] = d[perm[k]];
        lam[k] = lamv[k];
        order[k] = ord[k];
        for (int c = 0; c < m; c++) S[(int64_t)c * m + k] = Z[(int64_t)perm[c] * m + k];
    }
    __syncthreads();
    if (k == 0) {
        const double bl = beta[m - 1];
        int nc = 0;
        for (int i = 0; i < min(nev, m); i++) {
            const int ii = ord[i];
            const double res = fabs(bl * S[(int64_t)ii * m + m - 1]);
            if (res < tol * fmax(1.0, fabs(d[perm[ii]]))) nc++;
        }
        nconv[0] = nc;
    }
}

void lz_tridiag(cudaStream_t st, int m, int nev, double shift, double tol, const double* alpha, const double* beta,
                double* theta, double* S, double* lam, int* order, int* nconv, double* work) {
    if (m > 256) throw std::runtime_error("Lanczos subspace above 256 vectors is not supported");
    TMG_LAUNCH(k_tridiag, 1, 256, 0, st, m, nev, shift, tol, alpha, beta, theta, S, lam, order, nconv, work);
    TMG_CHECK_LAUNCH();
}

// src/hermitian_lanczos.cpp:141-218: shifts = the m-nev smallest theta; bulge-chasing
// Givens sweeps on (alpha, beta); rotations accumulated into Q by rows.
__global__ void __launch_bounds__(256) k_restart_qr(int m, int nev, const double* __restrict__ theta,
                                                    double* __restrict__ alpha, double* __restrict__ beta,
                                                    double* __restrict__ Q, double* __restrict__ rot) {
    const int ns = m - nev;
    if (threadIdx.x == 0) {
        for (int s = 0; s < ns; s++) {
            const double mu = theta[s];
            double x = alpha[0] - mu, z = beta[0];
            for (int i = 0; i < m - 1; i++) {
                const double r = hypot(x, z);
                double c, sn;
                if (r < 1e-300) { c = 1.0; sn = 0.0; } else { c = x / r; sn = z / r; }
                if (i > 0) beta[i - 1] = r;
                const double a0 = alpha[i], a1 = alpha[i + 1], b0 = beta[i];
                alpha[i] = c * c * a0 + 2.0 * c * sn * b0 + sn * sn * a1;
                alpha[i + 1] = sn * sn * a0 - 2.0 * c * sn * b0 + c * c * a1;
                beta[i] = c * sn * (a1 - a0) + (c * c - sn * sn) * b0;
                if (i + 2 < m) {
                    const double bulge = sn * beta[i + 1];
                    beta[i + 1] = c * beta[i + 1];
                    x = beta[i];
                    z = bulge;
                }
                rot[2 * ((int64_t)s * (m - 1) + i)] = c;
                rot[2 * ((int64_t)s * (m - 1) + i) + 1] = sn;
            }
        }
    }
    __syncthreads();
    const int row = threadIdx.x;
    if (row >= m) return;
    for (int c = 0; c < m; c++) Q[(int64_t)c * m + row] = (c == row) ? 1.0 : 0.0;
    for (int s = 0; s < ns; s++)
        for (int i = 0; i < m - 1; i++) {
            const double c = rot[2 * ((int64_t)s * (m - 1) + i)], sn = rot[2 * ((int64_t)s * (m - 1) + i) + 1];
            const double q0 = Q[(int64_t)i * m + row], q1 = Q[(int64_t)(i + 1) * m + row];
            Q[(int64_t)i * m + row] = c * q0 + sn * q1;
            Q[(int64_t)(i + 1) * m + row] = -sn * q0 + c * q1;
        }
}

void lz_restart_qr(cudaStream_t st, int m, int nev, const double* theta, double* alpha, double* beta, double* Q,
                   double* rot) {
    TMG_LAUNCH(k_restart_qr, 1, 256, 0, st, m, nev, theta, alpha, beta, Q, rot);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_gemm_real(int64_t n, int K, int ncol, const T* __restrict__ X, const double* __restrict__ C, int ldc,
                            T* __restrict__ Y) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int c0 = 0; c0 < ncol; c0 += 8) {
        T acc[8];
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] = zero_of<T>();
        for (int k = 0; k < K; k++) {
            const T xv = X[(int64_t)k * n + i];
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (c0 + q < ncol) acc[q] += C[(int64_t)(c0 + q) * ldc + k] * xv;
        }
#pragma unroll
        for (int q = 0; q < 8; q++)
            if (c0 + q < ncol) Y[(int64_t)(c0 + q) * n + i] = acc[q];
    }
}
template <typename T>
void lz_gemm_real(cudaStream_t st, int64_t n, int K, int ncol, const T* X, const double* C, int ldc, T* Y) {
    if (n == 0 || ncol == 0) return;
    TMG_LAUNCH(k_gemm_real<T>, (unsigned)ceil_div(n, 128), 128, 0, st, n, K, ncol, X, C, ldc, Y);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_combine_f(int64_t n, const T* __restrict__ Y, const T* __restrict__ v, const double* __restrict__ beta,
                            int nev, int m, const double* __restrict__ Q, T* __restrict__ f) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double bt = beta[nev - 1];
    const double bd = beta[m - 1];
    const double qd = Q[(int64_t)(nev - 1) * m + m - 1];
    f[i] = bt * Y[i] + (bd * qd) * v[i];
}
template <typename T>
void lz_combine_f(cudaStream_t st, int64_t n, const T* Y, const T* v, const double* beta, int nev, int m,
                  const double* Q, T* f) {
    TMG_LAUNCH(k_combine_f<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, Y, v, beta, nev, m, Q, f);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_copy(int64_t n, const T* __restrict__ s, T* __restrict__ d) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) d[i] = s[i];
}
template <typename T>
void lz_copy(cudaStream_t st, int64_t n, const T* src, T* dst) {
    TMG_LAUNCH(k_copy<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, src, dst);
    TMG_CHECK_LAUNCH();
}
template <typename T>
__global__ void k_axpy(int64_t n, double a, const T* __restrict__ x, T* __restrict__ y) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) y[i] += a * x[i];
}
template <typename T>
void lz_axpy(cudaStream_t st, int64_t n, double a, const T* x, T* y) {
    TMG_LAUNCH(k_axpy<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, a, x, y);
    TMG_CHECK_LAUNCH();
}
template <typename T>
__global__ void k_sub(int64_t n, const T* __restrict__ b, const T* __restrict__ ax, T* __restrict__ r) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - ax[i];
}
template <typename T>
void lz_sub(cudaStream_t st, int64_t n, const T* b, const T* ax, T* r) {
    TMG_LAUNCH(k_sub<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, b, ax, r);
    TMG_CHECK_LAUNCH();
}
template <typename T>
__global__ void __launch_bounds__(256) k_norm2a(int64_t n, const T* __restrict__ x, double* __restrict__ partial) {
    __shared__ double sh[8];
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    double s = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += abs2(x[i]);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}
__global__ void k_norm2b(int nb, const double* __restrict__ partial, double* __restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < nb; b++) s += partial[b];
        out[0] = s;
    }
}
template <typename T>
void lz_norm2(cudaStream_t st, int64_t n, const T* x, double* partial, double* out) {
    TMG_LAUNCH(k_norm2a<T>, LZ_DOT_BLOCKS, 256, 0, st, n, x, partial);
    TMG_LAUNCH(k_norm2b, 1, 32, 0, st, LZ_DOT_BLOCKS, partial, out);
    TMG_CHECK_LAUNCH();
}

#define TMG_LZ_INST(T)                                                                                         \
    template void lz_spmv<T>(cudaStream_t, const DevCsr<T>&, const T*, T*, int, int64_t, bool);    \
    template void lz_multidot<T>(cudaStream_t, int64_t, const T*, int64_t, int, const T*, T*, T*);             \
    template void lz_three_term_dot<T>(cudaStream_t, int64_t, int, const T*, double*, const double*, const T*, T*); \
    template void lz_gemv_sub<T>(cudaStream_t, int64_t, int, const T*, const T*, T*);                         \
    template void lz_beta_scale<T>(cudaStream_t, int64_t, int, const T*, const T*, const T*, T*, T*, double*, int*); \
    template void lz_scale_cols<T>(cudaStream_t, int64_t, const T*, T*, T*);                                 \
    template void lz_gemm_real<T>(cudaStream_t, int64_t, int, int, const T*, const double*, int, T*);         \
    template void lz_combine_f<T>(cudaStream_t, int64_t, const T*, const T*, const double*, int, int,          \
                                  const double*, T*);                                                         \
    template void lz_copy<T>(cudaStream_t, int64_t, const T*, T*);                                             \
    template void lz_axpy<T>(cudaStream_t, int64_t, double, const T*, T*);                                     \
    template void lz_sub<T>(cudaStream_t, int64_t, const T*, const T*, T*);                                    \
    template void lz_norm2<T>(cudaStream_t, int64_t, const T*, double*, double*);
TMG_LZ_INST(double)
TMG_LZ_INST(zd)

}  // namespace tmg
