// Batched supernodal multifrontal LDL^H (no pivoting, D real) and its triangular solves.
//
// The supernodal tree is processed level by level (leaves first).  For every level: the
// level's update blocks are zeroed, children's update blocks are added into their parents
// (one launch per child rank, so no two writers touch one entry and the sums run in a fixed
// order), then each front is partially factorised by 32-wide pivot blocks: diagonal block
// (one CTA per front), panel rows (CTA per 64 rows), and the Schur update of the trailing
// lower triangle (CTA per 64x64 tile).  Every launch covers all problems of the batch
// (grid y or z = problem).  The reference factorises the same operator with Eigen's
// simplicial up-looking LDL^T (src/hermitian_lanczos.cpp:12-56); the supernodal form has the
// same L and D in exact arithmetic.
#include <algorithm>
#include <map>

#include "mf.cuh"

namespace tmg {

int64_t g_kernel_launches = 0;

template <typename T>
__device__ __forceinline__ T dev_div(T a, typename real_of<T>::type d) { return a / d; }
template <>
__device__ __forceinline__ double dev_div<double>(double a, double d) { return a / d; }
template <>
__device__ __forceinline__ float dev_div<float>(float a, float d) { return a / d; }

// Entry (i, j), i >= j, of front s: the L panel for j < w, the update block otherwise.
template <typename T>
__device__ __forceinline__ T* fent(const SnDev& S, T* L, T* U, int s, int64_t m, int w, int64_t i, int64_t j) {
    if (j < w) return L + S.loff[s] + j * m + i;
    const int64_t u = m - w;
    return U + S.uoff[s] + (j - w) * u + (i - w);
}

// ------------------------------------------------------------------------------------
template <typename T>
__global__ void k_scatter(int64_t n, const T* __restrict__ vals, const int64_t* __restrict__ dest,
                          const uint8_t* __restrict__ cj, T* __restrict__ L, int64_t lstride) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    const int64_t p = blockIdx.y;
    const int64_t d = dest[q];
    if (d < 0) return;
    const T v = vals[p * n + q];
    L[p * lstride + d] = cj[q] ? conj(v) : v;
}

template <typename T>
__global__ void k_uzero(const int32_t* __restrict__ items, int nitems, SnDev S, T* __restrict__ U, int64_t ustride) {
    const int64_t p = blockIdx.z;
    for (int it = blockIdx.y; it < nitems; it += gridDim.y) {
        const int s = items[it];
        const int64_t u = (S.row_ptr[s + 1] - S.row_ptr[s]) - (S.first[s + 1] - S.first[s]);
        T* Us = U + p * ustride + S.uoff[s];
        for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < u * u; q += (int64_t)gridDim.x * blockDim.x)
            Us[q] = zero_of<T>();
    }
}

template <typename T>
__global__ void k_extend_add(const int32_t* __restrict__ items, int nitems, SnDev S, T* __restrict__ L,
                             T* __restrict__ U, int64_t lstride, int64_t ustride) {
    const int64_t p = blockIdx.z;
    T* Lp = L + p * lstride;
    T* Up = U + p * ustride;
    for (int it = blockIdx.y; it < nitems; it += gridDim.y) {
        const int par = items[2 * it], c = items[2 * it + 1];
        const int64_t mc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int64_t wc = S.first[c + 1] - S.first[c];
        const int64_t u = mc - wc;
        const int64_t mp = S.row_ptr[par + 1] - S.row_ptr[par];
        const int wp = S.first[par + 1] - S.first[par];
        const int32_t* rl = S.rel + S.rel_ptr[c];
        const T* Uc = Up + S.uoff[c];
        for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < u * u;
             idx += (int64_t)gridDim.x * blockDim.x) {
            const int64_t a = idx % u, b = idx / u;
            if (a < b) continue;
            *fent(S, Lp, Up, par, mp, wp, rl[a], rl[b]) += Uc[b * u + a];
        }
    }
}

// Factor the 32x32 diagonal block of pivot block kb of every listed front.
template <typename T>
__global__ void __launch_bounds__(256) k_diag(const int32_t* __restrict__ items, int kb, SnDev S, T* __restrict__ L,
                                              int64_t lstride, int* __restrict__ status) {
    using R = typename real_of<T>::type;
    __shared__ T A[MF_NB][MF_NB + 1];
    const int64_t p = blockIdx.y;
    const int s = items[blockIdx.x];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const int k0 = kb * MF_NB;
    const int nb = min(MF_NB, w - k0);
    T* Fs = L + p * lstride + S.loff[s];
    for (int q = threadIdx.x; q < MF_NB * MF_NB; q += blockDim.x) {
        const int i = q % MF_NB, j = q / MF_NB;
        if (i < nb && j <= i) A[i][j] = Fs[(int64_t)(k0 + j) * m + k0 + i];
    }
    __syncthreads();
    for (int j = 0; j < nb; j++) {
        const R d = re(A[j][j]);
        if (d == R(0)) {
            if (threadIdx.x == 0) atomicCAS(status + p, 0, S.first[s] + k0 + j + 1);
            return;
        }
        const int t = nb - j - 1;
        for (int q = threadIdx.x; q < t * t; q += blockDim.x) {
            const int i = j + 1 + q % t, k = j + 1 + q / t;
            if (k <= i) A[i][k] -= dev_div(A[i][j] * conj(A[k][j]), d);
        }
        __syncthreads();
        for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) A[i][j] = dev_div(A[i][j], d);
        if (threadIdx.x == 0) { T dd = zero_of<T>(); reinterpret_cast<R*>(&dd)[0] = d; A[j][j] = dd; }
        __syncthreads();
    }
    for (int q = threadIdx.x; q < MF_NB * MF_NB; q += blockDim.x) {
        const int i = q % MF_NB, j = q / MF_NB;
        if (i < nb && j <= i) Fs[(int64_t)(k0 + j) * m + k0 + i] = A[i][j];
    }
}

// Panel rows below the diagonal block: L(i, blk) = A(i, blk) (D L_kk^H)^-1
template <typename T>
__global__ void __launch_bounds__(64) k_panel(const int32_t* __restrict__ items, int kb, SnDev S, T* __restrict__ L,
                                              int64_t lstride) {
    using R = typename real_of<T>::type;
    __shared__ T Lk[MF_NB][MF_NB + 1];
    __shared__ R dk[MF_NB];
    const int64_t p = blockIdx.y;
    const int s = items[2 * blockIdx.x];
    const int r0 = items[2 * blockIdx.x + 1];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const int k0 = kb * MF_NB;
    const int nb = min(MF_NB, w - k0);
    T* Fs = L + p * lstride + S.loff[s];
    for (int q = threadIdx.x; q < MF_NB * MF_NB; q += blockDim.x) {
        const int i = q % MF_NB, j = q / MF_NB;
        if (i < nb && j < i) Lk[i][j] = Fs[(int64_t)(k0 + j) * m + k0 + i];
    }
    for (int j = threadIdx.x; j < nb; j += blockDim.x) dk[j] = re(Fs[(int64_t)(k0 + j) * m + k0 + j]);
    __syncthreads();
    const int64_t i = r0 + threadIdx.x;
    if (i >= m) return;
    T x[MF_NB];
#pragma unroll
    for (int j = 0; j < MF_NB; j++) x[j] = j < nb ? Fs[(int64_t)(k0 + j) * m + i] : zero_of<T>();
#pragma unroll
    for (int j = 0; j < MF_NB; j++) {
        if (j < nb) {
            T a = x[j];
#pragma unroll
            for (int l = 0; l < MF_NB; l++)
                if (l < j) a -= (dk[l] * x[l]) * conj(Lk[j][l]);
            x[j] = dev_div(a, dk[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < MF_NB; j++)
        if (j < nb) Fs[(int64_t)(k0 + j) * m + i] = x[j];
}

// Trailing lower-triangle update: C(i,j) -= sum_l L(i,l) d_l conj(L(j,l)) over the pivot block
template <typename T>
__global__ void __launch_bounds__(256) k_update(const int32_t* __restrict__ items, int kb, SnDev S, T* __restrict__ L,
                                                T* __restrict__ U, int64_t lstride, int64_t ustride) {
    using R = typename real_of<T>::type;
    extern __shared__ unsigned char smem_raw[];
    T* Li = reinterpret_cast<T*>(smem_raw);                  // [MF_NB][MF_TILE]
    T* Lj = Li + MF_NB * MF_TILE;                            // [MF_NB][MF_TILE], scaled by d
    const int64_t p = blockIdx.y;
    const int s = items[3 * blockIdx.x];
    const int ti = items[3 * blockIdx.x + 1], tj = items[3 * blockIdx.x + 2];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const int k0 = kb * MF_NB;
    const int nb = min(MF_NB, w - k0);
    const int64_t t0 = k0 + nb;
    const int64_t i0 = t0 + (int64_t)ti * MF_TILE, j0 = t0 + (int64_t)tj * MF_TILE;
    T* Lp = L + p * lstride;
    T* Up = U + p * ustride;
    const T* Fs = Lp + S.loff[s];
    for (int q = threadIdx.x; q < MF_NB * MF_TILE; q += blockDim.x) {
        const int r = q % MF_TILE, l = q / MF_TILE;
        T a = zero_of<T>(), b = zero_of<T>();
        if (l < nb) {
            if (i0 + r < m) a = Fs[(int64_t)(k0 + l) * m + i0 + r];
            if (j0 + r < m) {
                const R d = re(Fs[(int64_t)(k0 + l) * m + k0 + l]);
                b = d * Fs[(int64_t)(k0 + l) * m + j0 + r];
            }
        }
        Li[l * MF_TILE + r] = a;
        Lj[l * MF_TILE + r] = b;
    }
    __syncthreads();
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = zero_of<T>();
    for (int l = 0; l < nb; l++) {
        T av[4], bv[4];
#pragma unroll
        for (int a = 0; a < 4; a++) av[a] = Li[l * MF_TILE + ty + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; b++) bv[b] = conj(Lj[l * MF_TILE + tx + 16 * b]);
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] += av[a] * bv[b];
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int64_t i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
            if (i < m && j < m && i >= j) *fent(S, Lp, Up, s, m, w, i, j) -= acc[a][b];
        }
}

template <typename T>
__global__ void k_count_nonpos(int32_t ns, SnDev S, const T* __restrict__ L, int64_t lstride, int* __restrict__ cnt) {
    const int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (s >= ns) return;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const T* Fs = L + p * lstride + S.loff[s];
    int c = 0;
    for (int j = 0; j < w; j++)
        if (!(re(Fs[(int64_t)j * m + j]) > 0)) c++;
    if (c) atomicAdd(cnt + p, c);
}

// ------------------------------------------------------------------------------------
// Triangular solves, level by level.  Forward: gather the front vector (own entries +
// children's update vectors, children in fixed order), then sweep 64-wide column blocks:
// every CTA of a front re-solves the small diagonal block (staged in shared memory) from
// the final block entries and updates its own 256 rows below it, so a large front is spread
// over many CTAs and the only sequential chain is the column-block loop.  Backward:
// off-diagonal products with the ancestors' solution (warp per column), then column blocks
// from the last one, each CTA re-solving the diagonal block and updating its own columns to
// the left.  grid y = problem.
template <typename T>
__device__ __forceinline__ T shfl_t(T v, int src) {
    using R = typename real_of<T>::type;
    T o;
    reinterpret_cast<R*>(&o)[0] = __shfl_sync(0xffffffff, reinterpret_cast<R*>(&v)[0], src);
    if constexpr (sizeof(T) == 2 * sizeof(R))
        reinterpret_cast<R*>(&o)[1] = __shfl_sync(0xffffffff, reinterpret_cast<R*>(&v)[1], src);
    return o;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    using R = typename real_of<T>::type;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        R* q = reinterpret_cast<R*>(&v);
        q[0] += __shfl_xor_sync(0xffffffff, q[0], o);
        if constexpr (sizeof(T) == 2 * sizeof(R)) q[1] += __shfl_xor_sync(0xffffffff, q[1], o);
    }
    return v;
}

struct SolveArgs {
    int64_t lstride, xstride, tstride;
};

template <typename T>
__global__ void __launch_bounds__(256) k_fwd_gather(const int32_t* __restrict__ lvl, SnDev S, SolveArgs A,
                                                    const T* __restrict__ x, T* __restrict__ tbuf) {
    const int64_t p = blockIdx.y;
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = lvl[blockIdx.x];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    T* t = tbuf + S.row_ptr[s];
    for (int64_t r = threadIdx.x; r < m; r += blockDim.x) t[r] = r < w ? x[f + r] : zero_of<T>();
    __syncthreads();
    for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
        const int ch = S.child_list[c];
        const int64_t mc = S.row_ptr[ch + 1] - S.row_ptr[ch];
        const int wc = S.first[ch + 1] - S.first[ch];
        const T* tc = tbuf + S.row_ptr[ch] + wc;
        const int32_t* rl = S.rel + S.rel_ptr[ch];
        for (int64_t a = threadIdx.x; a < mc - wc; a += blockDim.x) t[rl[a]] += tc[a];
        __syncthreads();
    }
}

// item = (s, row0): rows [row0, row0 + SV_RC) below the diagonal block of column block b
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_block(const int32_t* __restrict__ items, int b, SnDev S, SolveArgs A,
                                                   const T* __restrict__ L, T* __restrict__ x, T* __restrict__ tbuf) {
    __shared__ T y[SV_B];
    extern __shared__ unsigned char sv_smem[];
    T (*Lb)[SV_B + 1] = reinterpret_cast<T (*)[SV_B + 1]>(sv_smem);
    const int64_t p = blockIdx.y;
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int64_t row0 = items[2 * blockIdx.x + 1];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int b0 = b * SV_B;
    const int nbb = min(SV_B, w - b0);
    const T* Fs = L + p * A.lstride + S.loff[s];
    T* t = tbuf + S.row_ptr[s];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < SV_B * SV_B; q += blockDim.x) {
        const int i = q % SV_B, j = q / SV_B;
        if (i < nbb && j < i) Lb[i][j] = Fs[(int64_t)(b0 + j) * m + b0 + i];
    }
    if (threadIdx.x < nbb) y[threadIdx.x] = t[b0 + threadIdx.x];
    __syncthreads();
    if (warp == 0) {
        T v0 = lane < nbb ? y[lane] : zero_of<T>();
        T v1 = lane + 32 < nbb ? y[lane + 32] : zero_of<T>();
        for (int j = 0; j < nbb; j++) {
            const T yj = j < 32 ? shfl_t(v0, j) : shfl_t(v1, j - 32);
            if (lane > j && lane < nbb) v0 -= Lb[lane][j] * yj;
            if (lane + 32 > j && lane + 32 < nbb) v1 -= Lb[lane + 32][j] * yj;
        }
        if (lane < nbb) y[lane] = v0;
        if (lane + 32 < nbb) y[lane + 32] = v1;
    }
    __syncthreads();
    if (row0 == b0 + nbb)   // the first chunk of this front stores the scaled block solution
        for (int j = threadIdx.x; j < nbb; j += blockDim.x)
            x[f + b0 + j] = dev_div(y[j], re(Fs[(int64_t)(b0 + j) * m + b0 + j]));
    const int64_t r = row0 + threadIdx.x;
    if (r < m && r < row0 + SV_RC) {
        T a = t[r];
        for (int j = 0; j < nbb; j++) a -= Fs[(int64_t)(b0 + j) * m + r] * y[j];
        t[r] = a;
    }
}

// item = (s, col0): z_j = x[f + j] - sum_{r >= w} conj(L(r, j)) x[rows[r]], j in [col0, col0+32)
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_offdiag(const int32_t* __restrict__ items, SnDev S, SolveArgs A,
                                                     const T* __restrict__ L, const T* __restrict__ x,
                                                     T* __restrict__ tbuf) {
    const int64_t p = blockIdx.y;
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int col0 = items[2 * blockIdx.x + 1];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const T* Fs = L + p * A.lstride + S.loff[s];
    const int32_t* rows = S.rows + S.row_ptr[s];
    T* t = tbuf + S.row_ptr[s];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int jj = warp; jj < SV_CC; jj += 8) {
        const int j = col0 + jj;
        if (j >= w) break;
        T a = zero_of<T>();
        for (int64_t r = w + lane; r < m; r += 32) a += conj(Fs[(int64_t)j * m + r]) * x[rows[r]];
        a = warp_sum(a);
        if (lane == 0) t[j] = x[f + j] - a;
    }
}

// item = (s, col0): solve L_bb^H x_b = z_b, then z_j -= sum_{r in b} conj(L(r, j)) x_r for
// the CTA's columns j in [col0, col0+32), j < b0
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_block(const int32_t* __restrict__ items, int b, SnDev S, SolveArgs A,
                                                   const T* __restrict__ L, T* __restrict__ x, T* __restrict__ tbuf) {
    __shared__ T xb[SV_B];
    extern __shared__ unsigned char sv_smem[];
    T (*Lb)[SV_B + 1] = reinterpret_cast<T (*)[SV_B + 1]>(sv_smem);
    const int64_t p = blockIdx.y;
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int col0 = items[2 * blockIdx.x + 1];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int b0 = b * SV_B;
    const int nbb = min(SV_B, w - b0);
    const T* Fs = L + p * A.lstride + S.loff[s];
    T* t = tbuf + S.row_ptr[s];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < SV_B * SV_B; q += blockDim.x) {
        const int i = q % SV_B, j = q / SV_B;
        if (i < nbb && j < i) Lb[i][j] = Fs[(int64_t)(b0 + j) * m + b0 + i];
    }
    if (threadIdx.x < nbb) xb[threadIdx.x] = t[b0 + threadIdx.x];
    __syncthreads();
    if (warp == 0) {
        T v0 = lane < nbb ? xb[lane] : zero_of<T>();
        T v1 = lane + 32 < nbb ? xb[lane + 32] : zero_of<T>();
        for (int j = nbb - 1; j >= 0; j--) {
            const T yj = j < 32 ? shfl_t(v0, j) : shfl_t(v1, j - 32);
            if (lane < j) v0 -= conj(Lb[j][lane]) * yj;
            if (lane + 32 < j) v1 -= conj(Lb[j][lane + 32]) * yj;
        }
        if (lane < nbb) xb[lane] = v0;
        if (lane + 32 < nbb) xb[lane + 32] = v1;
    }
    __syncthreads();
    if (col0 == 0)
        for (int j = threadIdx.x; j < nbb; j += blockDim.x) x[f + b0 + j] = xb[j];
    for (int jj = warp; jj < SV_CC; jj += 8) {
        const int j = col0 + jj;
        if (j >= b0) break;
        T a = zero_of<T>();
        for (int r = lane; r < nbb; r += 32) a += conj(Fs[(int64_t)j * m + b0 + r]) * xb[r];
        a = warp_sum(a);
        if (lane == 0) t[j] -= a;
    }
}

template <typename T, typename U>
__global__ void k_perm_in(int n, const int32_t* __restrict__ perm, const U* __restrict__ b, int64_t ldb,
                          T* __restrict__ x, const double* __restrict__ scale) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (j >= n) return;
    const int32_t o = perm[j];
    U val = b[p * ldb + o];
    if (scale) val = scale[p * n + o] * val;
    x[p * n + j] = conv<T, U>(val);
}

template <typename T, typename U>
__global__ void k_perm_out(int n, const int32_t* __restrict__ perm, const T* __restrict__ x, U* __restrict__ out,
                           int64_t ldo, const double* __restrict__ scale) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (j >= n) return;
    const int32_t o = perm[j];
    U val = conv<U, T>(x[p * n + j]);
    if (scale) val = scale[p * n + o] * val;
    out[p * ldo + o] = val;
}

// ------------------------------------------------------------------------------------
namespace {

// First-fit plan of the update-block workspace (entries).
struct FirstFit {
    std::map<int64_t, int64_t> free_;   // start -> length
    int64_t top = 0, peak = 0;
    int64_t alloc(int64_t sz) {
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= sz) {
                const int64_t off = it->first;
                const int64_t rest = it->second - sz;
                free_.erase(it);
                if (rest) free_[off + sz] = rest;
                return off;
            }
        const int64_t off = top;
        top += sz;
        peak = std::max(peak, top);
        return off;
    }
    void release(int64_t off, int64_t sz) {
        auto it = free_.emplace(off, sz).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); it = pv; }
        }
        if (it->first + it->second == top) { top = it->first; free_.erase(it); }
    }
};

}  // namespace

void DevSymbolic::upload(const Symbolic& S, const std::vector<int64_t>& dest_h, const std::vector<uint8_t>& conj_h) {
    release();
    n = S.n; ns = S.ns; max_front = S.max_front;
    flops = 4.0 * S.flops_real;
    std::vector<int64_t> lo(ns + 1, 0), uo(ns, 0);
    l_stored = 0;
    for (int s = 0; s < ns; s++) {
        const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
        const int64_t w = S.sn_first[s + 1] - S.sn_first[s];
        lo[s + 1] = lo[s] + m * w;
        l_stored += m * w - w * (w - 1) / 2;
    }
    l_entries = lo[ns];
    t_entries = S.sn_row_ptr[ns];
    // update-block plan: allocate a level's blocks before its extend-add, release the
    // children's blocks after it
    const int nlev = (int)S.level_ptr.size() - 1;
    FirstFit ff;
    auto usz = [&](int s) {
        const int64_t u = (S.sn_row_ptr[s + 1] - S.sn_row_ptr[s]) - (S.sn_first[s + 1] - S.sn_first[s]);
        return u * u;
    };
    for (int l = 0; l < nlev; l++) {
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sn[q];
            if (usz(s) > 0) uo[s] = ff.alloc(usz(s));
        }
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sn[q];
            for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
                const int ch = S.child_list[c];
                if (usz(ch) > 0) ff.release(uo[ch], usz(ch));
            }
        }
    }
    u_entries = std::max<int64_t>(ff.peak, 1);
    auto put = [&](auto*& dptr, const auto& vec) {
        using E = typename std::decay<decltype(vec[0])>::type;
        const size_t b = std::max<size_t>(1, vec.size()) * sizeof(E);
        TMG_CUDA(cudaMalloc((void**)&dptr, b));
        if (!vec.empty()) TMG_CUDA(cudaMemcpy(dptr, vec.data(), vec.size() * sizeof(E), cudaMemcpyHostToDevice));
        bytes += b;
    };
    put(sn_first, S.sn_first); put(sn_rows, S.sn_rows); put(rel, S.rel); put(child_ptr, S.child_ptr);
    put(child_list, S.child_list); put(sn_row_ptr, S.sn_row_ptr); put(loff, lo); put(uoff, uo);
    put(rel_ptr, S.rel_ptr); put(perm, S.perm); put(level_sn, S.level_sn);
    // scatter destinations are front offsets (m*m fronts); map them onto the L panels
    std::vector<int64_t> d2(dest_h.size(), -1);
    for (size_t q = 0; q < dest_h.size(); q++) {
        const int64_t d = dest_h[q];
        if (d < 0) continue;
        const int s = (int)(std::upper_bound(S.front_off.begin(), S.front_off.end(), d) - S.front_off.begin()) - 1;
        d2[q] = lo[s] + (d - S.front_off[s]);      // column < w: the offset stays inside the panel
    }
    put(dest, d2); put(conj, conj_h);
    nlower = (int64_t)dest_h.size();
    level_ptr = S.level_ptr;
    // factorisation schedule
    std::vector<int32_t> it;
    steps.clear();
    for (int l = 0; l < nlev; l++) {
        int maxw = 0, maxch = 0;
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sn[q];
            maxw = std::max(maxw, S.sn_first[s + 1] - S.sn_first[s]);
            maxch = std::max(maxch, S.child_ptr[s + 1] - S.child_ptr[s]);
        }
        const int nkb = (maxw + MF_NB - 1) / MF_NB;
        for (int kb = 0; kb < nkb; kb++) {
            Step st{};
            st.level = l;
            st.kb = kb;
            if (kb == 0) {
                st.uzero_off = (int64_t)it.size();
                for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                    const int s = S.level_sn[q];
                    if (usz(s) > 0) { it.push_back(s); st.uzero_cnt++; st.uzero_max = std::max(st.uzero_max, usz(s)); }
                }
                for (int r = 0; r < maxch; r++) {
                    st.ext_off.push_back((int64_t)it.size());
                    int cnt = 0;
                    int64_t umax = 0;
                    for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                        const int s = S.level_sn[q];
                        if (S.child_ptr[s + 1] - S.child_ptr[s] > r) {
                            const int c = S.child_list[S.child_ptr[s] + r];
                            it.push_back(s); it.push_back(c);
                            cnt++;
                            const int64_t u = (S.sn_row_ptr[c + 1] - S.sn_row_ptr[c]) - (S.sn_first[c + 1] - S.sn_first[c]);
                            umax = std::max<int64_t>(umax, u);
                        }
                    }
                    st.ext_cnt.push_back(cnt);
                    st.ext_max.push_back((int32_t)umax);
                }
            }
            st.diag_off = (int64_t)it.size();
            for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                const int s = S.level_sn[q];
                if (S.sn_first[s + 1] - S.sn_first[s] > kb * MF_NB) { it.push_back(s); st.diag_cnt++; }
            }
            st.panel_off = (int64_t)it.size();
            for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                const int s = S.level_sn[q];
                const int w = S.sn_first[s + 1] - S.sn_first[s];
                if (w <= kb * MF_NB) continue;
                const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                const int64_t r0 = kb * MF_NB + std::min(MF_NB, w - kb * MF_NB);
                for (int64_t r = r0; r < m; r += 64) { it.push_back(s); it.push_back((int32_t)r); st.panel_cnt++; }
            }
            st.upd_off = (int64_t)it.size();
            for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                const int s = S.level_sn[q];
                const int w = S.sn_first[s + 1] - S.sn_first[s];
                if (w <= kb * MF_NB) continue;
                const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                const int64_t t0 = kb * MF_NB + std::min(MF_NB, w - kb * MF_NB);
                const int64_t T = (m - t0 + MF_TILE - 1) / MF_TILE;
                for (int64_t a = 0; a < T; a++)
                    for (int64_t b = 0; b <= a; b++) {
                        it.push_back(s); it.push_back((int32_t)a); it.push_back((int32_t)b);
                        st.upd_cnt++;
                    }
            }
            steps.push_back(st);
        }
    }
    put(items, it);
    // triangular-solve schedule
    std::vector<int32_t> si;
    solve_levels.assign(nlev, SolveLevel{});
    for (int l = 0; l < nlev; l++) {
        SolveLevel& L = solve_levels[l];
        int maxw = 0;
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sn[q];
            maxw = std::max(maxw, S.sn_first[s + 1] - S.sn_first[s]);
        }
        const int nbk = (maxw + SV_B - 1) / SV_B;
        for (int b = 0; b < nbk; b++) {
            L.fwd_off.push_back((int64_t)si.size());
            int cnt = 0;
            for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                const int s = S.level_sn[q];
                const int w = S.sn_first[s + 1] - S.sn_first[s];
                if (w <= b * SV_B) continue;
                const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                const int64_t r0 = b * SV_B + std::min(SV_B, w - b * SV_B);
                if (r0 >= m) { si.push_back(s); si.push_back((int32_t)r0); cnt++; continue; }
                for (int64_t r = r0; r < m; r += SV_RC) { si.push_back(s); si.push_back((int32_t)r); cnt++; }
            }
            L.fwd_cnt.push_back(cnt);
        }
        L.off_items = (int64_t)si.size();
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
            const int s = S.level_sn[q];
            const int w = S.sn_first[s + 1] - S.sn_first[s];
            for (int c0 = 0; c0 < w; c0 += SV_CC) { si.push_back(s); si.push_back(c0); L.off_cnt++; }
        }
        for (int b = 0; b < nbk; b++) {
            L.bwd_off.push_back((int64_t)si.size());
            int cnt = 0;
            for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                const int s = S.level_sn[q];
                const int w = S.sn_first[s + 1] - S.sn_first[s];
                if (w <= b * SV_B) continue;
                si.push_back(s); si.push_back(0); cnt++;
                for (int c0 = SV_CC; c0 < b * SV_B; c0 += SV_CC) { si.push_back(s); si.push_back(c0); cnt++; }
            }
            L.bwd_cnt.push_back(cnt);
        }
    }
    put(sitems, si);
}

void DevSymbolic::release() {
    for (void* p : {(void*)sn_first, (void*)sn_rows, (void*)rel, (void*)child_ptr, (void*)child_list,
                    (void*)sn_row_ptr, (void*)loff, (void*)uoff, (void*)rel_ptr, (void*)perm, (void*)level_sn,
                    (void*)items, (void*)sitems, (void*)dest, (void*)conj})
        if (p) cudaFree(p);
    sn_first = sn_rows = rel = child_ptr = child_list = perm = level_sn = items = sitems = nullptr;
    sn_row_ptr = loff = uoff = rel_ptr = dest = nullptr;
    conj = nullptr;
    bytes = 0;
}

template <typename T>
void mf_scatter(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, const T* vals) {
    if (S.nlower == 0) return;
    TMG_LAUNCH(k_scatter<T>, dim3((unsigned)ceil_div(S.nlower, 256), bt.B), 256, 0, st, S.nlower, vals, S.dest, S.conj,
               bt.L, bt.lstride);
    TMG_CHECK_LAUNCH();
}

template <typename T>
void mf_factor(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, int* status) {
    static bool attr_set = false;
    const size_t upd_smem = 2 * MF_NB * MF_TILE * sizeof(T);
    if (!attr_set) {
        TMG_CUDA(cudaFuncSetAttribute(k_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem));
        attr_set = true;
    }
    const SnDev sn = S.sn();
    const unsigned B = bt.B;
    for (const auto& stp : S.steps) {
        if (stp.uzero_cnt) {
            const unsigned gx = (unsigned)std::min<int64_t>(std::max<int64_t>(1, ceil_div(stp.uzero_max, 256)), 2048);
            const unsigned gy = (unsigned)std::min<int64_t>(stp.uzero_cnt, 65535);
            TMG_LAUNCH(k_uzero<T>, dim3(gx, gy, B), 256, 0, st, S.items + stp.uzero_off, stp.uzero_cnt, sn, bt.U,
                       bt.ustride);
        }
        for (size_t r = 0; r < stp.ext_off.size(); r++) {
            if (stp.ext_cnt[r] == 0) continue;
            const int64_t ent = (int64_t)stp.ext_max[r] * stp.ext_max[r];
            const unsigned gx = (unsigned)std::min<int64_t>(std::max<int64_t>(1, ceil_div(ent, 256)), 2048);
            const unsigned gy = (unsigned)std::min<int64_t>(stp.ext_cnt[r], 65535);
            TMG_LAUNCH(k_extend_add<T>, dim3(gx, gy, B), 256, 0, st, S.items + stp.ext_off[r], stp.ext_cnt[r], sn, bt.L,
                       bt.U, bt.lstride, bt.ustride);
        }
        if (stp.diag_cnt)
            TMG_LAUNCH(k_diag<T>, dim3(stp.diag_cnt, B), 256, 0, st, S.items + stp.diag_off, stp.kb, sn, bt.L, bt.lstride,
                       status);
        if (stp.panel_cnt)
            TMG_LAUNCH(k_panel<T>, dim3(stp.panel_cnt, B), 64, 0, st, S.items + stp.panel_off, stp.kb, sn, bt.L,
                       bt.lstride);
        if (stp.upd_cnt)
            TMG_LAUNCH(k_update<T>, dim3(stp.upd_cnt, B), 256, upd_smem, st, S.items + stp.upd_off, stp.kb, sn, bt.L, bt.U,
                       bt.lstride, bt.ustride);
    }
    TMG_CHECK_LAUNCH();
}

template <typename T>
void mf_solve(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, T* x, T* tbuf) {
    const int nlev = (int)S.level_ptr.size() - 1;
    static bool attr_set = false;
    const size_t sv_smem = (size_t)SV_B * (SV_B + 1) * sizeof(T);
    if (!attr_set) {
        TMG_CUDA(cudaFuncSetAttribute(k_fwd_block<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sv_smem));
        TMG_CUDA(cudaFuncSetAttribute(k_bwd_block<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sv_smem));
        attr_set = true;
    }
    const SnDev sn = S.sn();
    const SolveArgs A{bt.lstride, (int64_t)S.n, S.t_entries};
    const unsigned B = bt.B;
    for (int l = 0; l < nlev; l++) {
        const int cnt = S.level_ptr[l + 1] - S.level_ptr[l];
        if (!cnt) continue;
        TMG_LAUNCH(k_fwd_gather<T>, dim3(cnt, B), 256, 0, st, S.level_sn + S.level_ptr[l], sn, A, x, tbuf);
        const auto& L = S.solve_levels[l];
        for (size_t b = 0; b < L.fwd_off.size(); b++)
            if (L.fwd_cnt[b])
                TMG_LAUNCH(k_fwd_block<T>, dim3(L.fwd_cnt[b], B), 256, sv_smem, st, S.sitems + L.fwd_off[b], (int)b, sn, A,
                           bt.L, x, tbuf);
    }
    for (int l = nlev - 1; l >= 0; l--) {
        const auto& L = S.solve_levels[l];
        if (L.off_cnt)
            TMG_LAUNCH(k_bwd_offdiag<T>, dim3(L.off_cnt, B), 256, 0, st, S.sitems + L.off_items, sn, A, bt.L, x, tbuf);
        for (int b = (int)L.bwd_off.size() - 1; b >= 0; b--)
            if (L.bwd_cnt[b])
                TMG_LAUNCH(k_bwd_block<T>, dim3(L.bwd_cnt[b], B), 256, sv_smem, st, S.sitems + L.bwd_off[b], b, sn, A,
                           bt.L, x, tbuf);
    }
    TMG_CHECK_LAUNCH();
}

template <typename T, typename U>
void mf_permute_in(cudaStream_t st, const DevSymbolic& S, int B, const U* b, int64_t ldb, T* x, const double* scale) {
    if (!S.n) return;
    TMG_LAUNCH((k_perm_in<T, U>), dim3((unsigned)ceil_div(S.n, 256), B), 256, 0, st, S.n, S.perm, b, ldb, x, scale);
    TMG_CHECK_LAUNCH();
}
template <typename T, typename U>
void mf_permute_out(cudaStream_t st, const DevSymbolic& S, int B, const T* x, U* out, int64_t ldo, const double* scale) {
    if (!S.n) return;
    TMG_LAUNCH((k_perm_out<T, U>), dim3((unsigned)ceil_div(S.n, 256), B), 256, 0, st, S.n, S.perm, x, out, ldo, scale);
    TMG_CHECK_LAUNCH();
}

template <typename T>
void mf_count_nonpos(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, int* cnt) {
    TMG_LAUNCH(k_count_nonpos<T>, dim3((unsigned)ceil_div(S.ns, 128), bt.B), 128, 0, st, S.ns, S.sn(), bt.L, bt.lstride,
               cnt);
    TMG_CHECK_LAUNCH();
}

#define TMG_INST(T)                                                                          \
    template void mf_factor<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, int*);     \
    template void mf_scatter<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, const T*); \
    template void mf_solve<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, T*, T*);    \
    template void mf_count_nonpos<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, int*);
TMG_INST(double)
TMG_INST(float)
TMG_INST(zd)
TMG_INST(zf)
#define TMG_PINST(T, U)                                                                                          \
    template void mf_permute_in<T, U>(cudaStream_t, const DevSymbolic&, int, const U*, int64_t, T*, const double*); \
    template void mf_permute_out<T, U>(cudaStream_t, const DevSymbolic&, int, const T*, U*, int64_t, const double*);
TMG_PINST(double, double)
TMG_PINST(float, double)
TMG_PINST(zd, zd)
TMG_PINST(zf, zd)

}  // namespace tmg
