// Lanczos eigensolver device kernels, batched over problems (grid y/z = problem):
// sparse matrix-vector products, deterministic two-stage reductions, classical Gram-Schmidt
// reorthogonalisation, and the small FP64 tridiagonal problems (eigen-decomposition by
// implicit QL, implicit-restart QR sweeps) with one CTA per problem.
#include <algorithm>

#include "lz.cuh"

namespace tmg {

// y = A x (or y -= A x) for CSR A; one warp per row, lanes stride the row's entries so the
// value and column loads are coalesced; grid y = vector, z = problem.
template <typename T>
__device__ __forceinline__ T lz_warp_sum(T v) {
    using R = typename real_of<T>::type;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        R* q = reinterpret_cast<R*>(&v);
        q[0] += __shfl_xor_sync(0xffffffff, q[0], o);
        if constexpr (sizeof(T) == 2 * sizeof(R)) q[1] += __shfl_xor_sync(0xffffffff, q[1], o);
    }
    return v;
}

template <typename T>
__global__ void __launch_bounds__(256) k_spmv(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                                              const T* __restrict__ av, int64_t vstride, const T* __restrict__ x,
                                              int64_t xs, T* __restrict__ y, int64_t ys, int64_t ld, int sub) {
    const int64_t i = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (i >= nrows) return;                      // uniform per warp
    const int64_t v = blockIdx.y, p = blockIdx.z;
    const T* xv = x + p * xs + v * ld;
    const T* a = av + p * vstride;
    T s = zero_of<T>();
    for (int64_t q = rp[i] + lane; q < rp[i + 1]; q += 32) s += a[q] * xv[ci[q]];
    s = lz_warp_sum(s);
    if (lane == 0) {
        T* yv = y + p * ys + v * ld;
        if (sub) yv[i] -= s;
        else yv[i] = s;
    }
}

template <typename T>
void lz_spmv(cudaStream_t st, int B, const DevCsr<T>& A, const T* x, int64_t xs, T* y, int64_t ys, int nvec, int64_t ld,
             bool subtract) {
    if (A.nrows == 0 || nvec == 0 || B == 0) return;
    TMG_LAUNCH(k_spmv<T>, dim3((unsigned)ceil_div(A.nrows, 8), nvec, B), 256, 0, st, A.nrows, A.rowptr, A.col, A.val,
               A.vstride, x, xs, y, ys, ld, subtract ? 1 : 0);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__device__ T block_sum(T v, T* sh) {
    using R = typename real_of<T>::type;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        R* q = reinterpret_cast<R*>(&v);
        q[0] += __shfl_down_sync(0xffffffff, q[0], o);
        if constexpr (sizeof(T) == 2 * sizeof(R)) q[1] += __shfl_down_sync(0xffffffff, q[1], o);
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
__global__ void __launch_bounds__(256) k_multidot1(int64_t n, const T* __restrict__ A, int64_t as, int64_t lda, int K,
                                                   const T* __restrict__ y, int64_t ys, T* __restrict__ partial) {
    __shared__ T sh[8];
    const int64_t p = blockIdx.y;
    A += p * as;
    y += p * ys;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    for (int k = 0; k < K; k++) {
        T s = zero_of<T>();
        for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += conj(A[k * lda + i]) * y[i];
        s = block_sum(s, sh);
        if (threadIdx.x == 0) partial[((int64_t)p * K + k) * gridDim.x + blockIdx.x] = s;
    }
}

template <typename T>
__global__ void k_multidot2(int n_out, int nb, const T* __restrict__ partial, T* __restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_out) return;
    T s = zero_of<T>();
    for (int b = 0; b < nb; b++) s += partial[(int64_t)q * nb + b];
    out[q] = s;
}

template <typename T>
void lz_multidot(cudaStream_t st, int B, int64_t n, const T* A, int64_t as, int64_t lda, int K, const T* y, int64_t ys,
                 T* partial, T* out) {
    TMG_LAUNCH(k_multidot1<T>, dim3(LZ_DOT_BLOCKS, B), 256, 0, st, n, A, as, lda, K, y, ys, partial);
    TMG_LAUNCH(k_multidot2<T>, (unsigned)ceil_div((int64_t)K * B, 128), 128, 0, st, K * B, LZ_DOT_BLOCKS, partial, out);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_three_term(int64_t n, int j, const T* __restrict__ dot, double* __restrict__ alpha,
                             const double* __restrict__ beta, int ldab, const T* __restrict__ V, int64_t vs,
                             T* __restrict__ w, int64_t ws) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    const double a = re(dot[p]);
    if (i == 0) alpha[p * ldab + j] = a;
    if (i >= n) return;
    const T* Vp = V + p * vs;
    T v = w[p * ws + i] - a * Vp[(int64_t)j * n + i];
    if (j > 0) v = v - beta[p * ldab + j - 1] * Vp[(int64_t)(j - 1) * n + i];
    w[p * ws + i] = v;
}
template <typename T>
void lz_three_term(cudaStream_t st, int B, int64_t n, int j, const T* dot, double* alpha, const double* beta, int ldab,
                   const T* V, int64_t vs, T* w, int64_t ws) {
    TMG_LAUNCH(k_three_term<T>, dim3((unsigned)ceil_div(n, 256), B), 256, 0, st, n, j, dot, alpha, beta, ldab, V, vs, w, ws);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_gemv_sub(int64_t n, int K, const T* __restrict__ V, int64_t vs, const T* __restrict__ h, int ldh,
                           T* __restrict__ w, int64_t ws) {
    __shared__ T hs[LZ_MAXM];
    const int64_t p = blockIdx.y;
    for (int k = threadIdx.x; k < K; k += blockDim.x) hs[k] = h[p * ldh + k];
    __syncthreads();
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T* Vp = V + p * vs;
    T acc = zero_of<T>();
    for (int k = 0; k < K; k++) acc += Vp[(int64_t)k * n + i] * hs[k];
    w[p * ws + i] -= acc;
}
template <typename T>
void lz_gemv_sub(cudaStream_t st, int B, int64_t n, int K, const T* V, int64_t vs, const T* h, int ldh, T* w, int64_t ws) {
    if (K > LZ_MAXM) throw std::runtime_error("Lanczos subspace above " + std::to_string(LZ_MAXM) + " vectors is not supported");
    TMG_LAUNCH(k_gemv_sub<T>, dim3((unsigned)ceil_div(n, 256), B), 256, 0, st, n, K, V, vs, h, ldh, w, ws);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_beta_scale(int64_t n, int j, const T* __restrict__ dot, const T* __restrict__ w,
                             const T* __restrict__ Mw, int64_t ws, T* __restrict__ V, T* __restrict__ MV, int64_t vs,
                             double* __restrict__ beta, int ldab, int* __restrict__ flag) {
    const int64_t p = blockIdx.y;
    const double b = sqrt(fabs(re(dot[p])));
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i == 0) {
        beta[p * ldab + j] = b;
        if (!(b >= 1e-14) && flag[p] == 0) flag[p] = j + 1;   // NaN counts as a breakdown
    }
    if (i >= n) return;
    const double ib = 1.0 / b;
    V[p * vs + (int64_t)(j + 1) * n + i] = ib * w[p * ws + i];
    MV[p * vs + (int64_t)(j + 1) * n + i] = ib * Mw[p * ws + i];
}
template <typename T>
void lz_beta_scale(cudaStream_t st, int B, int64_t n, int j, const T* dot, const T* w, const T* Mw, int64_t ws, T* V,
                   T* MV, int64_t vs, double* beta, int ldab, int* flag) {
    TMG_LAUNCH(k_beta_scale<T>, dim3((unsigned)ceil_div(n, 256), B), 256, 0, st, n, j, dot, w, Mw, ws, V, MV, vs, beta,
               ldab, flag);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_scale_first(int64_t n, const T* __restrict__ dot, T* __restrict__ V, T* __restrict__ MV, int64_t vs) {
    const int64_t p = blockIdx.y;
    const double s = sqrt(re(dot[p]));
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    V[p * vs + i] = V[p * vs + i] / s;
    MV[p * vs + i] = MV[p * vs + i] / s;
}
template <typename T>
void lz_scale_first(cudaStream_t st, int B, int64_t n, const T* dot, T* V, T* MV, int64_t vs) {
    TMG_LAUNCH(k_scale_first<T>, dim3((unsigned)ceil_div(n, 256), B), 256, 0, st, n, dot, V, MV, vs);
    TMG_CHECK_LAUNCH();
}

// ------------------------------------------------------------------------------------
// Tridiagonal eigenproblem (implicit QL with eigenvectors, EISPACK tql2 formulation), one
// CTA per problem.  Thread 0 runs the scalar recurrences and records each sweep's
// rotations; every thread then applies the sweep to its own row of Z.
__global__ void __launch_bounds__(256) k_tridiag(int m, int ldab, int nev, double shift0,
                                                 const double* __restrict__ shifts, double tol,
                                                 const double* __restrict__ alpha_b, const double* __restrict__ beta_b,
                                                 double* __restrict__ theta_b, double* __restrict__ S_b,
                                                 double* __restrict__ lam_b, int* __restrict__ order_b,
                                                 int* __restrict__ nconv, double* __restrict__ Z_b) {
    __shared__ double d[LZ_MAXM], e[LZ_MAXM], rc[LZ_MAXM], rs[LZ_MAXM], lamv[LZ_MAXM];
    __shared__ int perm[LZ_MAXM], ord[LZ_MAXM];
    __shared__ int s_m, s_go, s_lo, s_hi;
    const int p = blockIdx.x;
    const double shift = shifts ? shifts[p] : shift0;
    const double* alpha = alpha_b + (int64_t)p * ldab;
    const double* beta = beta_b + (int64_t)p * ldab;
    double* theta = theta_b + (int64_t)p * ldab;
    double* lam = lam_b + (int64_t)p * ldab;
    int* order = order_b + (int64_t)p * ldab;
    double* S = S_b + (int64_t)p * ldab * ldab;
    double* Z = Z_b + (int64_t)p * ldab * ldab;
    const int k = threadIdx.x;   // thread 0 runs the scalar recurrences; rows r = k, k + blockDim, ...
    for (int r = k; r < m; r += blockDim.x) {
        for (int c = 0; c < m; c++) Z[(int64_t)c * m + r] = (c == r) ? 1.0 : 0.0;
        d[r] = alpha[r];
        e[r] = (r < m - 1) ? beta[r] : 0.0;
    }
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
            if (mm >= m) mm = m - 1;   // NaN in alpha / beta: no split found, stay inside d[], e[]
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
                double pp = (d[l + 1] - g) / (2.0 * e[l]);
                double r = hypot(pp, 1.0);
                if (pp < 0) r = -r;
                d[l] = e[l] / (pp + r);
                d[l + 1] = e[l] * (pp + r);
                const double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < m; i++) d[i] -= h;
                f = f + h;
                pp = d[mm];
                double c = 1.0, c2 = c, c3 = c;
                const double el1 = e[l + 1];
                double s = 0.0, s2 = 0.0;
                for (int i = mm - 1; i >= l; i--) {
                    c3 = c2; c2 = c; s2 = s;
                    g = c * e[i];
                    h = c * pp;
                    r = hypot(pp, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = pp / r;
                    pp = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    rc[i] = c;
                    rs[i] = s;
                }
                pp = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * pp;
                d[l] = c * pp;
                s_lo = l;
                s_hi = mm - 1;
                s_go = (fabs(e[l]) > eps * tst1 && iter < 200) ? 1 : 0;
            }
            __syncthreads();
            for (int r = k; r < m; r += blockDim.x) {
                for (int i = s_hi; i >= s_lo; i--) {
                    const double c = rc[i], s = rs[i];
                    const double h = Z[(int64_t)(i + 1) * m + r];
                    const double zi = Z[(int64_t)i * m + r];
                    Z[(int64_t)(i + 1) * m + r] = s * zi + c * h;
                    Z[(int64_t)i * m + r] = c * zi - s * h;
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
            double pp = d[perm[i]];
            for (int j = i + 1; j < m; j++)
                if (d[perm[j]] < pp) { kk = j; pp = d[perm[j]]; }
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
    for (int r = k; r < m; r += blockDim.x) {
        theta[r] = d[perm[r]];
        lam[r] = lamv[r];
        order[r] = ord[r];
        for (int c = 0; c < m; c++) S[(int64_t)c * m + r] = Z[(int64_t)perm[c] * m + r];
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
        nconv[p] = nc;
    }
}

void lz_tridiag(cudaStream_t st, int B, int m, int ldab, int nev, double shift, double tol, const double* alpha,
                const double* beta, double* theta, double* S, double* lam, int* order, int* nconv, double* Z,
                const double* shifts) {
    if (m > LZ_MAXM) throw std::runtime_error("Lanczos subspace above " + std::to_string(LZ_MAXM) + " vectors is not supported");
    TMG_LAUNCH(k_tridiag, B, 256, 0, st, m, ldab, nev, shift, shifts, tol, alpha, beta, theta, S, lam, order, nconv, Z);
    TMG_CHECK_LAUNCH();
}

// src/hermitian_lanczos.cpp:141-218: shifts = the m-nev smallest theta; bulge-chasing
// Givens sweeps on (alpha, beta); rotations accumulated into Q by rows.
__global__ void __launch_bounds__(256) k_restart_qr(int m, int ldab, int nev, const double* __restrict__ theta_b,
                                                    double* __restrict__ alpha_b, double* __restrict__ beta_b,
                                                    double* __restrict__ Q_b, double* __restrict__ rot_b,
                                                    int64_t rot_stride) {
    const int p = blockIdx.x;
    const double* theta = theta_b + (int64_t)p * ldab;
    double* alpha = alpha_b + (int64_t)p * ldab;
    double* beta = beta_b + (int64_t)p * ldab;
    double* Q = Q_b + (int64_t)p * ldab * ldab;
    double* rot = rot_b + (int64_t)p * rot_stride;
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
    for (int row = threadIdx.x; row < m; row += blockDim.x) {
        for (int c = 0; c < m; c++) Q[(int64_t)c * m + row] = (c == row) ? 1.0 : 0.0;
        for (int s = 0; s < ns; s++)
            for (int i = 0; i < m - 1; i++) {
                const double c = rot[2 * ((int64_t)s * (m - 1) + i)], sn = rot[2 * ((int64_t)s * (m - 1) + i) + 1];
                const double q0 = Q[(int64_t)i * m + row], q1 = Q[(int64_t)(i + 1) * m + row];
                Q[(int64_t)i * m + row] = c * q0 + sn * q1;
                Q[(int64_t)(i + 1) * m + row] = -sn * q0 + c * q1;
            }
    }
}

void lz_restart_qr(cudaStream_t st, int B, int m, int ldab, int nev, const double* theta, double* alpha, double* beta,
                   double* Q, double* rot, int64_t rot_stride) {
    if (m > LZ_MAXM) throw std::runtime_error("Lanczos subspace above " + std::to_string(LZ_MAXM) + " vectors is not supported");
    TMG_LAUNCH(k_restart_qr, B, 256, 0, st, m, ldab, nev, theta, alpha, beta, Q, rot, rot_stride);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_gemm_real(int64_t n, int K, int ncol, const T* __restrict__ X, int64_t xs, const double* __restrict__ C,
                            int64_t cs, int ldc, T* __restrict__ Y, int64_t ys) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n) return;
    X += p * xs;
    C += p * cs;
    Y += p * ys;
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
void lz_gemm_real(cudaStream_t st, int B, int64_t n, int K, int ncol, const T* X, int64_t xs, const double* C, int64_t cs,
                  int ldc, T* Y, int64_t ys) {
    if (n == 0 || ncol == 0 || B == 0) return;
    TMG_LAUNCH(k_gemm_real<T>, dim3((unsigned)ceil_div(n, 128), B), 128, 0, st, n, K, ncol, X, xs, C, cs, ldc, Y, ys);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_combine_f(int64_t n, const T* __restrict__ Y, int64_t ys, const T* __restrict__ v, int64_t vs,
                            const double* __restrict__ beta, int ldab, int nev, int m, const double* __restrict__ Q,
                            T* __restrict__ f, int64_t fs) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n) return;
    const double bt = beta[p * ldab + nev - 1];
    const double bd = beta[p * ldab + m - 1];
    const double qd = Q[p * (int64_t)ldab * ldab + (int64_t)(nev - 1) * m + m - 1];
    f[p * fs + i] = bt * Y[p * ys + i] + (bd * qd) * v[p * vs + i];
}
template <typename T>
void lz_combine_f(cudaStream_t st, int B, int64_t n, const T* Y, int64_t ys, const T* v, int64_t vs, const double* beta,
                  int ldab, int nev, int m, const double* Q, T* f, int64_t fs) {
    TMG_LAUNCH(k_combine_f<T>, dim3((unsigned)ceil_div(n, 256), B), 256, 0, st, n, Y, ys, v, vs, beta, ldab, nev, m, Q, f,
               fs);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_restart_norm(int64_t n, int nev, const T* __restrict__ dot, const T* __restrict__ f,
                               const T* __restrict__ Mf, int64_t fs, T* __restrict__ V, T* __restrict__ MV, int64_t vs,
                               double* __restrict__ beta, int ldab) {
    const int64_t p = blockIdx.y;
    const double b = sqrt(fabs(re(dot[p])));
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b > 1e-14) {
        if (i == 0) beta[p * ldab + nev - 1] = b;
        if (i < n) {
            V[p * vs + (int64_t)nev * n + i] = f[p * fs + i] / b;
            MV[p * vs + (int64_t)nev * n + i] = Mf[p * fs + i] / b;
        }
    } else if (i == 0) {
        beta[p * ldab + nev - 1] = 0.0;
    }
}
template <typename T>
void lz_restart_norm(cudaStream_t st, int B, int64_t n, int nev, const T* dot, const T* f, const T* Mf, int64_t fs, T* V,
                     T* MV, int64_t vs, double* beta, int ldab) {
    TMG_LAUNCH(k_restart_norm<T>, dim3((unsigned)ceil_div(n, 256), B), 256, 0, st, n, nev, dot, f, Mf, fs, V, MV, vs, beta,
               ldab);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void k_copy(int64_t n, const T* __restrict__ s, T* __restrict__ d) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) d[i] = s[i];
}
template <typename T>
void lz_copy(cudaStream_t st, int64_t n, const T* src, T* dst) {
    if (n <= 0) return;
    TMG_LAUNCH(k_copy<T>, (unsigned)ceil_div(n, 256), 256, 0, st, n, src, dst);
    TMG_CHECK_LAUNCH();
}

template <typename T>
__global__ void __launch_bounds__(256) k_norm2a(int64_t n, const T* __restrict__ x, int64_t xs, double* __restrict__ partial) {
    __shared__ double sh[8];
    const int64_t p = blockIdx.y;
    x += p * xs;
    const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const int64_t lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    double s = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) s += abs2(x[i]);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partial[p * gridDim.x + blockIdx.x] = s;
}
__global__ void k_norm2b(int B, int nb, const double* __restrict__ partial, double* __restrict__ out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= B) return;
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += partial[(int64_t)p * nb + b];
    out[p] = s;
}
template <typename T>
void lz_norm2(cudaStream_t st, int B, int64_t n, const T* x, int64_t xs, double* partial, double* out) {
    TMG_LAUNCH(k_norm2a<T>, dim3(LZ_DOT_BLOCKS, B), 256, 0, st, n, x, xs, partial);
    TMG_LAUNCH(k_norm2b, (unsigned)ceil_div(B, 128), 128, 0, st, B, LZ_DOT_BLOCKS, partial, out);
    TMG_CHECK_LAUNCH();
}

#define TMG_LZ_INST(T)                                                                                                 \
    template void lz_spmv<T>(cudaStream_t, int, const DevCsr<T>&, const T*, int64_t, T*, int64_t, int, int64_t, bool); \
    template void lz_multidot<T>(cudaStream_t, int, int64_t, const T*, int64_t, int64_t, int, const T*, int64_t, T*, T*); \
    template void lz_three_term<T>(cudaStream_t, int, int64_t, int, const T*, double*, const double*, int, const T*,  \
                                   int64_t, T*, int64_t);                                                           \
    template void lz_gemv_sub<T>(cudaStream_t, int, int64_t, int, const T*, int64_t, const T*, int, T*, int64_t);     \
    template void lz_beta_scale<T>(cudaStream_t, int, int64_t, int, const T*, const T*, const T*, int64_t, T*, T*,    \
                                   int64_t, double*, int, int*);                                                    \
    template void lz_scale_first<T>(cudaStream_t, int, int64_t, const T*, T*, T*, int64_t);                          \
    template void lz_gemm_real<T>(cudaStream_t, int, int64_t, int, int, const T*, int64_t, const double*, int64_t, int, \
                                  T*, int64_t);                                                                     \
    template void lz_combine_f<T>(cudaStream_t, int, int64_t, const T*, int64_t, const T*, int64_t, const double*,    \
                                  int, int, int, const double*, T*, int64_t);                                       \
    template void lz_restart_norm<T>(cudaStream_t, int, int64_t, int, const T*, const T*, const T*, int64_t, T*, T*,  \
                                     int64_t, double*, int);                                                        \
    template void lz_copy<T>(cudaStream_t, int64_t, const T*, T*);                                                   \
    template void lz_norm2<T>(cudaStream_t, int, int64_t, const T*, int64_t, double*, double*);
TMG_LZ_INST(double)
TMG_LZ_INST(zd)

}  // namespace tmg
