// Dense generalized Hermitian eigensolver for small harmonic problems (n <= 200), one CTA
// per problem, FP64.  Restates the reference's solve_dense (src/hermitian_lanczos.cpp:68-110,
// used for n <= 200 at :283): K and M are made exactly Hermitian ((A + A^H) / 2), the problem
// K x = lambda M x is reduced with the Cholesky factor M = L L^H to C = L^-1 K L^-H, C is
// brought to real symmetric tridiagonal form (Householder reflectors, then a diagonal phase
// scaling of the off-diagonal), the tridiagonal problem is solved by implicit QL with
// eigenvectors, and the nev smallest eigenpairs are transformed back to x = L^-H y
// (M-orthonormal, as Eigen's GeneralizedSelfAdjointEigenSolver returns them).
#include "dense.cuh"

namespace tmg {

namespace {

constexpr int DN_MAX = 200;
constexpr int DN_THREADS = 512;

__device__ __forceinline__ zd zmul(zd a, zd b) { return zd{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ zd zconj(zd a) { return zd{a.x, -a.y}; }
__device__ __forceinline__ zd zsub(zd a, zd b) { return zd{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ zd zadd(zd a, zd b) { return zd{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ zd zscale(double s, zd a) { return zd{s * a.x, s * a.y}; }

// Column-major n x n matrices in global workspace; A(i, j) = A[j * n + i].
__global__ void __launch_bounds__(DN_THREADS) k_dense_geig(int n, int nev, const zd* __restrict__ Kin,
                                                           const zd* __restrict__ Min, zd* __restrict__ work,
                                                           double* __restrict__ lam_out, zd* __restrict__ X,
                                                           double* __restrict__ res_out, int* __restrict__ status) {
    const int p = blockIdx.x;
    const int64_t nn = (int64_t)n * n;
    const zd* K0 = Kin + p * nn;
    const zd* M0 = Min + p * nn;
    zd* A = work + p * 5 * nn;       // Hermitian K, later C and the reflectors
    zd* L = A + nn;                  // Cholesky factor of M (lower)
    zd* W = L + nn;                  // L^-1 K, then scratch
    zd* Mh = W + nn;                 // Hermitian M (kept for residuals)
    zd* Kh = Mh + nn;                // Hermitian K (kept for residuals)
    X += (int64_t)p * n * nev;
    const int tid = threadIdx.x;
    __shared__ double d[DN_MAX + 8], e[DN_MAX + 8], rc[DN_MAX + 8], rs[DN_MAX + 8], lamv[DN_MAX + 8];
    __shared__ zd v[DN_MAX + 8], pv[DN_MAX + 8], ph[DN_MAX + 8], ev[DN_MAX + 8];
    __shared__ int perm[DN_MAX + 8];
    __shared__ double s_scal[4];
    __shared__ int s_m, s_go, s_lo, s_hi, s_bad;
    if (tid == 0) s_bad = 0;
    // 1. Hermitian parts
    for (int64_t q = tid; q < nn; q += blockDim.x) {
        const int i = (int)(q % n), j = (int)(q / n);
        const zd a = K0[q], b = zconj(K0[(int64_t)i * n + j]);
        const zd c = M0[q], dd = zconj(M0[(int64_t)i * n + j]);
        const zd kh = zscale(0.5, zadd(a, b)), mh = zscale(0.5, zadd(c, dd));
        A[q] = kh; Kh[q] = kh; Mh[q] = mh; L[q] = mh;
    }
    __syncthreads();
    // 2. Cholesky M = L L^H (right-looking, lower triangle)
    for (int j = 0; j < n; j++) {
        if (tid == 0) {
            const double djj = L[(int64_t)j * n + j].x;
            if (!(djj > 0.0)) s_bad = 1;
            s_scal[0] = djj > 0.0 ? sqrt(djj) : 1.0;
        }
        __syncthreads();
        const double dj = s_scal[0];
        for (int i = j + tid; i < n; i += blockDim.x) L[(int64_t)j * n + i] = zscale(1.0 / dj, L[(int64_t)j * n + i]);
        __syncthreads();
        const int t = n - j - 1;
        for (int64_t q = tid; q < (int64_t)t * t; q += blockDim.x) {
            const int i = j + 1 + (int)(q % t), k = j + 1 + (int)(q / t);
            if (k <= i) L[(int64_t)k * n + i] = zsub(L[(int64_t)k * n + i],
                                                     zmul(L[(int64_t)j * n + i], zconj(L[(int64_t)j * n + k])));
        }
        __syncthreads();
    }
    if (s_bad) { if (tid == 0) status[p] = 1; return; }
    // 3. W = L^-1 K (forward substitution on every column), C = L^-1 W^H
    for (int pass = 0; pass < 2; pass++) {
        zd* src = pass == 0 ? A : W;
        zd* dst = pass == 0 ? W : A;
        for (int64_t q = tid; q < nn; q += blockDim.x) {
            const int i = (int)(q % n), j = (int)(q / n);
            dst[q] = pass == 0 ? src[q] : zconj(src[(int64_t)i * n + j]);
        }
        __syncthreads();
        for (int i = 0; i < n; i++) {
            const double li = L[(int64_t)i * n + i].x;
            for (int c = tid; c < n; c += blockDim.x) dst[(int64_t)c * n + i] = zscale(1.0 / li, dst[(int64_t)c * n + i]);
            __syncthreads();
            const int t = n - i - 1;
            for (int64_t q = tid; q < (int64_t)t * n; q += blockDim.x) {
                const int r = i + 1 + (int)(q % t), c = (int)(q / t);
                dst[(int64_t)c * n + r] = zsub(dst[(int64_t)c * n + r], zmul(L[(int64_t)i * n + r], dst[(int64_t)c * n + i]));
            }
            __syncthreads();
        }
    }
    // exact Hermitian C
    for (int64_t q = tid; q < nn; q += blockDim.x) {
        const int i = (int)(q % n), j = (int)(q / n);
        if (i > j) {
            const zd h = zscale(0.5, zadd(A[q], zconj(A[(int64_t)i * n + j])));
            A[q] = h;
            A[(int64_t)i * n + j] = zconj(h);
        } else if (i == j) {
            A[q].y = 0.0;
        }
    }
    __syncthreads();
    // 4. Householder tridiagonalisation: column k, reflector H = I - 2 u u^H on rows k+1..n-1
    for (int k = 0; k < n - 2; k++) {
        const int t = n - k - 1;           // length of the column below the diagonal
        if (tid < t) v[tid] = A[(int64_t)k * n + k + 1 + tid];
        __syncthreads();
        if (tid == 0) {
            double nrm = 0.0;
            for (int i = 0; i < t; i++) nrm += v[i].x * v[i].x + v[i].y * v[i].y;
            nrm = sqrt(nrm);
            const double a0 = hypot(v[0].x, v[0].y);
            zd phase = a0 > 0.0 ? zd{v[0].x / a0, v[0].y / a0} : zd{1.0, 0.0};
            const zd alpha = zscale(-nrm, phase);          // H x = alpha e1
            ev[k] = alpha;
            s_scal[1] = 0.0;
            if (nrm > 0.0) {
                v[0] = zsub(v[0], alpha);
                double un = 0.0;
                for (int i = 0; i < t; i++) un += v[i].x * v[i].x + v[i].y * v[i].y;
                s_scal[1] = un > 0.0 ? 1.0 / sqrt(un) : 0.0;
            }
        }
        __syncthreads();
        if (tid < t) v[tid] = zscale(s_scal[1], v[tid]);
        __syncthreads();
        // p = B u (B trailing block), then w = p - (u^H p) u, B -= 2 (u w^H + w u^H)
        for (int i = tid; i < t; i += blockDim.x) {
            zd acc{0.0, 0.0};
            for (int j = 0; j < t; j++) acc = zadd(acc, zmul(A[(int64_t)(k + 1 + j) * n + k + 1 + i], v[j]));
            pv[i] = acc;
        }
        __syncthreads();
        if (tid == 0) {
            zd up{0.0, 0.0};
            for (int i = 0; i < t; i++) up = zadd(up, zmul(zconj(v[i]), pv[i]));
            s_scal[2] = up.x;
            s_scal[3] = up.y;
        }
        __syncthreads();
        const zd up{s_scal[2], s_scal[3]};
        if (tid < t) pv[tid] = zsub(pv[tid], zmul(up, v[tid]));
        __syncthreads();
        for (int64_t q = tid; q < (int64_t)t * t; q += blockDim.x) {
            const int i = (int)(q % t), j = (int)(q / t);
            zd* a = &A[(int64_t)(k + 1 + j) * n + k + 1 + i];
            const zd upd = zadd(zmul(v[i], zconj(pv[j])), zmul(pv[i], zconj(v[j])));
            *a = zsub(*a, zscale(2.0, upd));
        }
        __syncthreads();
        // keep the reflector in column k below the subdiagonal slot (rows k+1..n-1)
        if (tid < t) A[(int64_t)k * n + k + 1 + tid] = v[tid];
        __syncthreads();
    }
    // tridiagonal: diagonal d, off-diagonal ev (complex) -> real |e| with phases ph
    if (tid == 0) {
        for (int i = 0; i < n; i++) d[i] = A[(int64_t)i * n + i].x;
        if (n >= 2) ev[n - 2] = A[(int64_t)(n - 2) * n + n - 1];
        ph[0] = zd{1.0, 0.0};
        for (int i = 0; i + 1 < n; i++) {
            const double a = hypot(ev[i].x, ev[i].y);
            e[i] = a;
            const zd u = a > 0.0 ? zd{ev[i].x / a, ev[i].y / a} : zd{1.0, 0.0};
            ph[i + 1] = zmul(ph[i], u);        // T = P S P^H with S real symmetric
        }
        e[n - 1] = 0.0;
    }
    __syncthreads();
    // 5. implicit QL with eigenvectors on (d, e): Zr (n x n, column-major) in W's storage
    double* Zr = reinterpret_cast<double*>(W);
    for (int64_t q = tid; q < nn; q += blockDim.x) Zr[q] = (q % n) == (q / n) ? 1.0 : 0.0;
    __syncthreads();
    const double eps = 2.220446049250313e-16;
    double f = 0.0, tst1 = 0.0;
    for (int l = 0; l < n; l++) {
        if (tid == 0) {
            tst1 = fmax(tst1, fabs(d[l]) + fabs(e[l]));
            int mm = l;
            while (mm < n) {
                if (fabs(e[mm]) <= eps * tst1) break;
                mm++;
            }
            if (mm >= n) mm = n - 1;
            s_m = mm;
            s_go = mm > l ? 1 : 0;
        }
        __syncthreads();
        int iter = 0;
        while (s_go) {
            if (tid == 0) {
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
                for (int i = l + 2; i < n; i++) d[i] -= h;
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
            for (int k = tid; k < n; k += blockDim.x)
                for (int i = s_hi; i >= s_lo; i--) {
                    const double c = rc[i], s = rs[i];
                    const double h = Zr[(int64_t)(i + 1) * n + k];
                    const double zi = Zr[(int64_t)i * n + k];
                    Zr[(int64_t)(i + 1) * n + k] = s * zi + c * h;
                    Zr[(int64_t)i * n + k] = c * zi - s * h;
                }
            __syncthreads();
        }
        if (tid == 0) { d[l] = d[l] + f; e[l] = 0.0; }
        __syncthreads();
    }
    // ascending order (stable)
    if (tid == 0) {
        for (int i = 0; i < n; i++) perm[i] = i;
        for (int i = 1; i < n; i++) {
            const int pv_ = perm[i];
            int j = i - 1;
            while (j >= 0 && d[perm[j]] > d[pv_]) { perm[j + 1] = perm[j]; j--; }
            perm[j + 1] = pv_;
        }
        for (int i = 0; i < nev; i++) lamv[i] = d[perm[i]];
    }
    __syncthreads();
    // 6. eigenvectors: y = H_0 ... H_{n-3} P z, x = L^-H y; one thread per selected pair
    for (int s = tid; s < nev; s += blockDim.x) {
        const int c = perm[s];
        zd* x = X + (int64_t)s * n;
        for (int i = 0; i < n; i++) x[i] = zmul(ph[i], zd{Zr[(int64_t)c * n + i], 0.0});
        for (int k = n - 3; k >= 0; k--) {          // y <- H_k y on rows k+1..n-1
            const int t = n - k - 1;
            zd dot{0.0, 0.0};
            for (int i = 0; i < t; i++) dot = zadd(dot, zmul(zconj(A[(int64_t)k * n + k + 1 + i]), x[k + 1 + i]));
            for (int i = 0; i < t; i++)
                x[k + 1 + i] = zsub(x[k + 1 + i], zscale(2.0, zmul(A[(int64_t)k * n + k + 1 + i], dot)));
        }
        for (int i = n - 1; i >= 0; i--) {         // L^H x = y
            zd a = x[i];
            for (int k = i + 1; k < n; k++) a = zsub(a, zmul(zconj(L[(int64_t)i * n + k]), x[k]));
            x[i] = zscale(1.0 / L[(int64_t)i * n + i].x, a);
        }
    }
    __syncthreads();
    // 7. eigenvalues and residuals ||K x - lambda M x|| / ||K x|| (cyclic_solver.cpp:1099-1114)
    for (int s = tid; s < nev; s += blockDim.x) {
        const zd* x = X + (int64_t)s * n;
        double rn = 0.0, kn = 0.0;
        for (int i = 0; i < n; i++) {
            zd kx{0.0, 0.0}, mx{0.0, 0.0};
            for (int j = 0; j < n; j++) {
                kx = zadd(kx, zmul(Kh[(int64_t)j * n + i], x[j]));
                mx = zadd(mx, zmul(Mh[(int64_t)j * n + i], x[j]));
            }
            const zd r = zsub(kx, zscale(lamv[s], mx));
            rn += r.x * r.x + r.y * r.y;
            kn += kx.x * kx.x + kx.y * kx.y;
        }
        lam_out[(int64_t)p * nev + s] = lamv[s];
        res_out[(int64_t)p * nev + s] = kn > 0.0 ? sqrt(rn / kn) : sqrt(rn);
    }
    if (tid == 0) status[p] = 0;
}

// Scatter a CSC matrix (complex values) into a dense column-major block.
__global__ void k_csc_to_dense(int32_t n, const int64_t* __restrict__ cp, const int32_t* __restrict__ ri,
                               const zd* __restrict__ v, zd* __restrict__ D) {
    const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int64_t q = cp[j]; q < cp[j + 1]; q++) D[(int64_t)j * n + ri[q]] = v[q];
}

}  // namespace

void dense_csc_to_dense(cudaStream_t st, int32_t n, const int64_t* cp, const int32_t* ri, const zd* v, zd* D) {
    TMG_CUDA(cudaMemsetAsync(D, 0, (size_t)n * n * sizeof(zd), st));
    if (n) TMG_LAUNCH(k_csc_to_dense, (unsigned)ceil_div(n, 128), 128, 0, st, n, cp, ri, v, D);
    TMG_CHECK_LAUNCH();
}

void dense_geig(cudaStream_t st, int B, int n, int nev, const zd* K, const zd* M, zd* work, double* lam, zd* X,
                double* res, int* status) {
    if (n > DN_MAX || nev > n || nev < 1) throw std::invalid_argument("dense eigensolver: size out of range");
    TMG_LAUNCH(k_dense_geig, B, DN_THREADS, 0, st, n, nev, K, M, work, lam, X, res, status);
    TMG_CHECK_LAUNCH();
}

}  // namespace tmg
