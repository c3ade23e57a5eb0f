// Batched supernodal multifrontal LDL^H (no pivoting, D real) and its triangular solves.
//
// The supernodal tree is processed level by level (leaves first).  For every level: the
// level's update blocks are zeroed, children's update blocks are added into their parents
// (one launch per child rank, so no two writers touch one entry and the sums run in a fixed
// order), then each front is partially factorised by 32-wide pivot blocks: diagonal block
// (one CTA per front), panel rows (CTA per 64 rows), and the Schur update (CTA per 64x64
// tile) in two levels: a pivot block updates only the rest of its 256-column super-block,
// and when a super-block is complete one update with K = 256 covers everything right of it
// (remaining panel columns and the update block), so the large trailing matrices are read
// and written once per super-block.  Every launch covers all problems of the batch
// (grid y or z = problem).  The reference factorises the same operator with Eigen's
// simplicial up-looking LDL^T (src/hermitian_lanczos.cpp:12-56); the supernodal form has the
// same L and D in exact arithmetic.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>

#include "mf.cuh"
#include "mf_tc.cuh"

namespace tmg {

thread_local int64_t g_kernel_launches = 0;
thread_local cudaStream_t g_stream = nullptr;
thread_local ByteCount* g_bytes = nullptr;

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

// Zero the lower triangle (row >= column: the only part the Schur updates write and the
// extend-add reads) of every listed front's update block; one warp per column.
template <typename T>
__global__ void k_uzero(const int32_t* __restrict__ items, int nitems, SnDev S, T* __restrict__ U, int64_t ustride) {
    const int64_t p = blockIdx.z;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int it = blockIdx.y; it < nitems; it += gridDim.y) {
        const int s = items[it];
        const int64_t u = (S.row_ptr[s + 1] - S.row_ptr[s]) - (S.first[s + 1] - S.first[s]);
        T* Us = U + p * ustride + S.uoff[s];
        for (int64_t b = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); b < u; b += warps)
            for (int64_t a = b + lane; a < u; a += 32) Us[b * u + a] = zero_of<T>();
    }
}

// Add each listed child's update block (lower triangle, column by column: one warp per column)
// into its parent's front, through the child's row map.
template <typename T>
__global__ void k_extend_add(const int32_t* __restrict__ items, int nitems, SnDev S, T* __restrict__ L,
                             T* __restrict__ U, int64_t lstride, int64_t ustride) {
    const int64_t p = blockIdx.z;
    T* Lp = L + p * lstride;
    T* Up = U + p * ustride;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int it = blockIdx.y; it < nitems; it += gridDim.y) {
        const int par = items[2 * it], c = items[2 * it + 1];
        const int64_t mc = S.row_ptr[c + 1] - S.row_ptr[c];
        const int64_t wc = S.first[c + 1] - S.first[c];
        const int64_t u = mc - wc;
        const int64_t mp = S.row_ptr[par + 1] - S.row_ptr[par];
        const int wp = S.first[par + 1] - S.first[par];
        const int32_t* rl = S.rel + S.rel_ptr[c];
        const T* Uc = Up + S.uoff[c];
        for (int64_t b = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); b < u; b += warps) {
            const int32_t jb = rl[b];
            for (int64_t a = b + lane; a < u; a += 32) *fent(S, Lp, Up, par, mp, wp, rl[a], jb) += Uc[b * u + a];
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

// Lower-triangle update of one 64x64 tile at front rows [i0, i0+64), columns [j0, j0+64):
//   C(i, j) -= sum_{l in [kl, kh)} L(i, l) d_l conj(L(j, l)),  i >= j, j < jmax,
// with kh = min(kl + kw, w), the K range staged through shared memory 32 columns at a time.
// Pivot mode (trail == 0): kl is one pivot block and jmax ends the block's 256-column
// super-block (updates stay inside it).  Trail mode: [kl, kh) is a whole super-block and
// the tile lies right of it (panel columns beyond it and the update block).
template <typename T>
__global__ void __launch_bounds__(256) k_update(const int32_t* __restrict__ items, int kl, int kw, int trail, SnDev S,
                                                T* __restrict__ L, T* __restrict__ U, int64_t lstride,
                                                int64_t ustride) {
    using R = typename real_of<T>::type;
    extern __shared__ unsigned char smem_raw[];
    T* Li = reinterpret_cast<T*>(smem_raw);                  // [MF_NB][MF_TILE]
    T* Lj = Li + MF_NB * MF_TILE;                            // [MF_NB][MF_TILE], scaled by d
    const int64_t p = blockIdx.y;
    const int s = items[3 * blockIdx.x];
    const int64_t i0 = items[3 * blockIdx.x + 1], j0 = items[3 * blockIdx.x + 2];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const int kh = min(kl + kw, w);
    const int64_t jmax = trail ? m : (int64_t)min((kl / MF_SB + 1) * MF_SB, w);
    T* Lp = L + p * lstride;
    T* Up = U + p * ustride;
    const T* Fs = Lp + S.loff[s];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = zero_of<T>();
    for (int k0 = kl; k0 < kh; k0 += MF_NB) {
        const int nb = min(MF_NB, kh - k0);
        __syncthreads();
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
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int64_t i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
            if (i < m && j < jmax && i >= j) *fent(S, Lp, Up, s, m, w, i, j) -= acc[a][b];
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
// Diagonal-block inverses.  After the numeric factorisation, every diagonal block of width
// NB (the block of columns [b*NB, b*NB + nbb) and the same rows) is replaced below its
// diagonal by the strict lower part of its unit-lower inverse X = L_bb^-1, computed by
// forward substitution on the columns of the identity (lanes hold rows, warp shuffles carry
// the solved entry).  The triangular solves then apply a block as one dense product, with
// no sequential dependency inside it.
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

// warps (items) per CTA of k_inv_small: its shared block copies stay under 48 KB
template <typename T>
constexpr int inv_wpc() { return sizeof(T) >= 16 ? 2 : 4; }

// item = (s, b) with a block of at most 32 columns; one warp per item
template <typename T, int NB>
__global__ void __launch_bounds__(128) k_inv_small(const int32_t* __restrict__ items, int cnt, SnDev S,
                                                   T* __restrict__ L, int64_t lstride) {
    __shared__ T Lb[inv_wpc<T>()][32][33];
    const int64_t p = blockIdx.y;
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int it = blockIdx.x * inv_wpc<T>() + wi;
    if (it >= cnt) return;                       // uniform per warp; only warp-level sync below
    const int s = items[2 * it], b = items[2 * it + 1];
    const int w = S.first[s + 1] - S.first[s];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int b0 = b * NB;
    const int nbb = min(NB, w - b0);             // <= 32 by construction of the item list
    if (nbb < 2 || nbb > 32) return;             // guard: this kernel's shared tiles hold 32 rows
    T* Fs = L + p * lstride + S.loff[s];
    for (int k = 0; k < nbb; k++)
        if (lane > k && lane < nbb) Lb[wi][lane][k] = Fs[(int64_t)(b0 + k) * m + b0 + lane];
    __syncwarp();
    for (int j = 0; j < nbb - 1; j++) {
        T v = lane == j ? one_of<T>() : zero_of<T>();
        for (int k = j; k < nbb - 1; k++) {
            const T xk = shfl_t(v, k);
            if (lane > k && lane < nbb) v -= Lb[wi][lane][k] * xk;
        }
        if (lane > j && lane < nbb) Fs[(int64_t)(b0 + j) * m + b0 + lane] = v;
    }
}

// item = (s, b) with a block wider than 32 columns; one CTA per item, warp per column
template <typename T, int NB>
__global__ void __launch_bounds__(256) k_inv_large(const int32_t* __restrict__ items, SnDev S, T* __restrict__ L,
                                                   int64_t lstride) {
    extern __shared__ unsigned char inv_smem[];
    T* Lb = reinterpret_cast<T*>(inv_smem);      // Lb[i * (NB + 1) + k] = L(b0 + i, b0 + k)
    constexpr int R = NB / 32;                   // rows per lane
    const int64_t p = blockIdx.y;
    const int s = items[2 * blockIdx.x], b = items[2 * blockIdx.x + 1];
    const int w = S.first[s + 1] - S.first[s];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int b0 = b * NB;
    const int nbb = min(NB, w - b0);
    if (nbb <= 0) return;
    T* Fs = L + p * lstride + S.loff[s];
    for (int q = threadIdx.x; q < NB * NB; q += blockDim.x) {
        const int i = q % NB, k = q / NB;
        if (i < nbb && k < i) Lb[i * (NB + 1) + k] = Fs[(int64_t)(b0 + k) * m + b0 + i];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = warp; j < nbb - 1; j += 8) {
        T v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = lane + 32 * r == j ? one_of<T>() : zero_of<T>();
        for (int k = j; k < nbb - 1; k++) {
            T src = v[0];
#pragma unroll
            for (int r = 1; r < R; r++)
                if ((k >> 5) == r) src = v[r];   // uniform across the warp
            const T xk = shfl_t(src, k & 31);
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int i = lane + 32 * r;
                if (i > k && i < nbb) v[r] -= Lb[i * (NB + 1) + k] * xk;
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int i = lane + 32 * r;
            if (i > j && i < nbb) Fs[(int64_t)(b0 + j) * m + b0 + i] = v[r];
        }
    }
}

// ------------------------------------------------------------------------------------
// Triangular solves, level by level (grid y = problem).  Front s has w pivot columns and m
// rows; its panel is L(r, j) = Fs[j * m + r] and its solve vector t (m entries) holds the
// pivot part first and the update for the parent after it.
//
// Forward, per level: gather assembles t from x and the children's updates and applies the
// first diagonal block (y_0 = X_0 t_0); each triangle launch b subtracts block b's product
// from the triangle rows below it, and the CTA holding block b+1's rows then applies X_{b+1}
// (look-ahead), so the next launch finds y_{b+1} ready; one rectangle launch then forms the
// parent update t[w..m) -= L21 y.  x receives D^-1 y.
// Backward, per level (top first): one rectangle launch forms z = x - L21^H x(rows) per
// column chunk and applies X^H to the last block; each triangle launch b subtracts block b's
// contribution from the columns left of it, and the CTA holding block b-1 applies X_{b-1}^H.
struct SolveArgs {
    int64_t lstride, xstride, tstride;
    const int* skip;   // per problem: nonzero = leave this problem's vectors alone (may be null)
};

constexpr int XS_LD = 65;                        // padded leading dimension of a staged 64x64 block

// Stage the strict lower part of the inverse block at column c0 (nbk <= 64 columns) into
// Xs[k * XS_LD + i] = X(i, k); every thread issues its loads at once.
template <typename T>
__device__ __forceinline__ void stage_x(const T* Fs, int64_t m, int c0, int nbk, T* Xs) {
#pragma unroll 4
    for (int q = threadIdx.x; q < 64 * 64; q += 256) {
        const int i = q & 63, k = q >> 6;
        if (k < nbk && i > k && i < nbk) Xs[k * XS_LD + i] = Fs[(int64_t)(c0 + k) * m + c0 + i];
    }
}

// v = X u (unit lower X staged in Xs, u in shared memory, nbk entries); four threads per row,
// red: 256 shared scratch entries.  Result for row i in v[i].  Called by all 256 threads.
template <typename T>
__device__ __forceinline__ void apply_x(const T* Xs, const T* u, int nbk, T* red, T* v) {
    const int i = threadIdx.x & 63, pi = threadIdx.x >> 6;
    T a = zero_of<T>();
    if (i < nbk)
        for (int k = pi; k < i; k += 4) a += Xs[k * XS_LD + i] * u[k];
    red[threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.x < nbk) v[i] = u[i] + ((red[i] + red[i + 64]) + (red[i + 128] + red[i + 192]));
}

// v = X^H u, same layout
template <typename T>
__device__ __forceinline__ void apply_xh(const T* Xs, const T* u, int nbk, T* red, T* v) {
    const int i = threadIdx.x & 63, pi = threadIdx.x >> 6;
    T a = zero_of<T>();
    if (i < nbk)
        for (int k = i + 1 + pi; k < nbk; k += 4) a += conj(Xs[i * XS_LD + k]) * u[k];
    red[threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.x < nbk) v[i] = u[i] + ((red[i] + red[i + 64]) + (red[i + 128] + red[i + 192]));
}

template <typename T>
__global__ void __launch_bounds__(256) k_fwd_gather(const int32_t* __restrict__ lvl, SnDev S, SolveArgs A,
                                                    const T* __restrict__ L, T* __restrict__ x, T* __restrict__ tbuf) {
    extern __shared__ unsigned char sv_smem[];
    T* Xs = reinterpret_cast<T*>(sv_smem);
    __shared__ T tv[64], yv[64], red[256];
    pdl_trigger();
    const int64_t p = blockIdx.y;
    const bool skp = A.skip && A.skip[p];
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = lvl[blockIdx.x];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const T* Fs = L + p * A.lstride + S.loff[s];
    const int nb0 = min(64, w);
    if (!skp) stage_x(Fs, m, 0, nb0, Xs);        // factor data: staged before the predecessor ends
    pdl_wait();
    if (skp) return;
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
    if (threadIdx.x < nb0) tv[threadIdx.x] = t[threadIdx.x];
    __syncthreads();
    apply_x(Xs, tv, nb0, red, yv);
    if (threadIdx.x < nb0) {
        const T y = yv[threadIdx.x];
        t[threadIdx.x] = y;
        x[f + threadIdx.x] = dev_div(y, re(Fs[(int64_t)threadIdx.x * m + threadIdx.x]));
    }
}

// item = (s, r0): triangle rows [r0, min(r0 + 64, w)) below full block b (r0 >= b*64 + 64)
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_tri(const int32_t* __restrict__ items, int b, SnDev S, SolveArgs A,
                                                 const T* __restrict__ L, T* __restrict__ x, T* __restrict__ tbuf) {
    extern __shared__ unsigned char sv_smem[];
    T* Xs = reinterpret_cast<T*>(sv_smem);
    __shared__ T ys[64], tn[64], yn[64], red[256];
    pdl_trigger();
    const int64_t p = blockIdx.y;
    const bool skp = A.skip && A.skip[p];
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int r0 = items[2 * blockIdx.x + 1];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int b0 = b * 64;
    const T* Fs = L + p * A.lstride + S.loff[s];
    T* t = tbuf + S.row_ptr[s];
    const int rend = min(r0 + 64, w);
    const bool la = r0 == b0 + 64;               // this CTA holds block b+1: look-ahead
    const int rl = threadIdx.x & 63, pi = threadIdx.x >> 6;
    const int r = r0 + rl;
    T lv[16];                                    // factor entries of this thread's product
#pragma unroll
    for (int u = 0; u < 16; u++) lv[u] = zero_of<T>();
    if (!skp) {
        if (la) stage_x(Fs, m, r0, rend - r0, Xs);
        if (r < rend) {
            const T* col = Fs + (int64_t)b0 * m + r;
#pragma unroll
            for (int u = 0; u < 16; u++) lv[u] = col[(int64_t)(pi + 4 * u) * m];
        }
    }
    pdl_wait();
    if (skp) return;
    if (threadIdx.x < 64) ys[threadIdx.x] = t[b0 + threadIdx.x];
    __syncthreads();
    T a = zero_of<T>();
#pragma unroll
    for (int u = 0; u < 16; u++) a += lv[u] * ys[pi + 4 * u];
    red[threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.x < 64 && r < rend) {
        const T v = t[r] - ((red[rl] + red[rl + 64]) + (red[rl + 128] + red[rl + 192]));
        t[r] = v;
        tn[rl] = v;
    }
    if (la) {
        __syncthreads();
        apply_x(Xs, tn, rend - r0, red, yn);
        if (threadIdx.x < rend - r0) {
            const T y = yn[threadIdx.x];
            t[r0 + threadIdx.x] = y;
            x[f + r0 + threadIdx.x] = dev_div(y, re(Fs[(int64_t)(r0 + threadIdx.x) * m + r0 + threadIdx.x]));
        }
    }
}

// item = (s, r0): rows [r0, min(r0 + SV_RR, m)) below the triangle (r0 >= w): t -= L21 y
template <typename T>
__global__ void __launch_bounds__(256) k_fwd_rect(const int32_t* __restrict__ items, SnDev S, SolveArgs A,
                                                  const T* __restrict__ L, T* __restrict__ tbuf) {
    constexpr int G = 256 / SV_RR;               // column groups
    __shared__ T part[256];
    pdl_trigger();
    const int64_t p = blockIdx.y;
    const bool skp = A.skip && A.skip[p];
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int r0 = items[2 * blockIdx.x + 1];
    const int w = S.first[s + 1] - S.first[s];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const T* Fs = L + p * A.lstride + S.loff[s];
    T* t = tbuf + S.row_ptr[s];
    pdl_wait();
    if (skp) return;
    const int rl = threadIdx.x % SV_RR, pi = threadIdx.x / SV_RR;
    const int64_t r = r0 + rl;
    T a = zero_of<T>();
    if (r < m) {
        const T* col = Fs + r;
        int j = pi;
        for (; j + 7 * G < w; j += 8 * G) {      // eight independent loads in flight per thread
            T lv[8], yv[8];
#pragma unroll
            for (int u = 0; u < 8; u++) { lv[u] = col[(int64_t)(j + u * G) * m]; yv[u] = t[j + u * G]; }
#pragma unroll
            for (int u = 0; u < 8; u++) a += lv[u] * yv[u];
        }
        for (; j < w; j += G) a += col[(int64_t)j * m] * t[j];
    }
    part[threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.x < SV_RR && r < m) {
        T sum = part[threadIdx.x];
#pragma unroll
        for (int q = 1; q < G; q++) sum += part[threadIdx.x + q * SV_RR];
        t[r] -= sum;
    }
}

// item = (s, c0): columns [c0, min(c0 + 64, w)); z_j = x_j - sum_{r >= w} conj(L(r, j)) x(rows[r]);
// each warp carries eight columns through the row loop; the CTA holding the front's last
// block then applies X^H
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_rect(const int32_t* __restrict__ items, SnDev S, SolveArgs A,
                                                  const T* __restrict__ L, T* __restrict__ x, T* __restrict__ tbuf,
                                                  int chunk) {
    // dynamic shared memory: `chunk` gathered solution entries, then the staged inverse block
    extern __shared__ unsigned char sv_smem[];
    T* xs = reinterpret_cast<T*>(sv_smem);
    T* Xs = xs + chunk;
    __shared__ T zs[64], xo[64], red[256];
    pdl_trigger();
    const int64_t p = blockIdx.y;
    const bool skp = A.skip && A.skip[p];
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int c0 = items[2 * blockIdx.x + 1];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const T* Fs = L + p * A.lstride + S.loff[s];
    const int32_t* rows = S.rows + S.row_ptr[s];
    T* t = tbuf + S.row_ptr[s];
    const int nc = min(64, w - c0);
    const bool last = c0 + nc == w;
    if (last && !skp) stage_x(Fs, m, c0, nc, Xs);
    pdl_wait();
    if (skp) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j0 = warp * 8;                     // this warp's columns: c0 + j0 .. c0 + j0 + 7
    T acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = zero_of<T>();
    for (int64_t q0 = w; q0 < m; q0 += chunk) {
        const int len = (int)(m - q0 < chunk ? m - q0 : chunk);
        __syncthreads();
        for (int q = threadIdx.x; q < len; q += blockDim.x) xs[q] = x[rows[q0 + q]];
        __syncthreads();
        if (j0 < nc) {
            const T* col = Fs + (int64_t)(c0 + j0) * m + q0;
            const int ncw = min(8, nc - j0);
            for (int q = lane; q < len; q += 64) {     // two rows per lane and step: 16 loads in flight
                const bool h1 = q + 32 < len;
                T l0[8], l1[8];
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    l0[c] = c < ncw ? col[(int64_t)c * m + q] : zero_of<T>();
                    l1[c] = c < ncw && h1 ? col[(int64_t)c * m + q + 32] : zero_of<T>();
                }
                const T x0 = xs[q], x1 = h1 ? xs[q + 32] : zero_of<T>();
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    acc[c] += conj(l0[c]) * x0;
                    acc[c] += conj(l1[c]) * x1;
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = warp_sum(acc[c]);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 8; c++)
            if (j0 + c < nc) {
                const T z = x[f + c0 + j0 + c] - acc[c];
                t[c0 + j0 + c] = z;
                zs[j0 + c] = z;
            }
    if (last) {
        __syncthreads();
        apply_xh(Xs, zs, nc, red, xo);
        if (threadIdx.x < nc) x[f + c0 + threadIdx.x] = xo[threadIdx.x];
    }
}

// item = (s, c0): columns [c0, c0 + 64) left of block b (c0 + 64 <= b*64):
// z_j -= sum_{r in block b} conj(L(r, j)) x_r; the CTA holding block b-1 then applies X^H
template <typename T>
__global__ void __launch_bounds__(256) k_bwd_tri(const int32_t* __restrict__ items, int b, SnDev S, SolveArgs A,
                                                 const T* __restrict__ L, T* __restrict__ x, T* __restrict__ tbuf) {
    extern __shared__ unsigned char sv_smem[];
    T* Xs = reinterpret_cast<T*>(sv_smem);
    __shared__ T xb[64], zs[64], xo[64], red[256];
    pdl_trigger();
    const int64_t p = blockIdx.y;
    const bool skp = A.skip && A.skip[p];
    x += p * A.xstride;
    tbuf += p * A.tstride;
    const int s = items[2 * blockIdx.x];
    const int c0 = items[2 * blockIdx.x + 1];
    const int f = S.first[s];
    const int w = S.first[s + 1] - f;
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int b0 = b * 64;
    const int nbb = min(64, w - b0);
    const T* Fs = L + p * A.lstride + S.loff[s];
    T* t = tbuf + S.row_ptr[s];
    const bool la = c0 + 64 == b0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j0 = warp * 8;
    T lv[2][8];                                  // factor entries of this lane's products
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int c = 0; c < 8; c++) lv[h][c] = zero_of<T>();
    if (!skp) {
        if (la) stage_x(Fs, m, c0, 64, Xs);
        const T* col = Fs + (int64_t)(c0 + j0) * m + b0;
#pragma unroll
        for (int h = 0; h < 2; h++)
            if (lane + 32 * h < nbb)
#pragma unroll
                for (int c = 0; c < 8; c++) lv[h][c] = col[(int64_t)c * m + lane + 32 * h];
    }
    pdl_wait();
    if (skp) return;
    if (threadIdx.x < nbb) xb[threadIdx.x] = x[f + b0 + threadIdx.x];
    __syncthreads();
    T acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = zero_of<T>();
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int r = lane + 32 * h;
        if (r < nbb) {
            const T xv = xb[r];
#pragma unroll
            for (int c = 0; c < 8; c++) acc[c] += conj(lv[h][c]) * xv;
        }
    }
#pragma unroll
    for (int c = 0; c < 8; c++) acc[c] = warp_sum(acc[c]);
    if (lane == 0)
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const T z = t[c0 + j0 + c] - acc[c];
            t[c0 + j0 + c] = z;
            zs[j0 + c] = z;
        }
    if (la) {
        __syncthreads();
        apply_xh(Xs, zs, 64, red, xo);
        if (threadIdx.x < 64) x[f + c0 + threadIdx.x] = xo[threadIdx.x];
    }
}

// Subtree solves.  One warp carries a whole subtree of narrow fronts (w <= 64: one diagonal
// block) through the forward solve in postorder and back through the backward solve in
// reverse postorder, with no grid-wide step between its fronts.  Lane i holds the pivot rows
// i and i + 32 of the current front in registers; the update rows stay in tbuf, where the
// parent's assembly (same warp, after __syncwarp) reads them.
constexpr int SUB_WARPS = 4;                     // subtrees (warps) per CTA

// task = (first, root): forward over the supernodes first..root
template <typename T>
__global__ void __launch_bounds__(32 * SUB_WARPS) k_sub_fwd(const int32_t* __restrict__ tasks, int ntasks, SnDev S,
                                                           SolveArgs A, const T* __restrict__ L, T* __restrict__ x,
                                                           T* __restrict__ tbuf) {
    pdl_trigger();
    const int task = blockIdx.x * SUB_WARPS + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int64_t p = blockIdx.y;
    pdl_wait();
    if (task >= ntasks || (A.skip && A.skip[p])) return;
    x += p * A.xstride;
    tbuf += p * A.tstride;
    L += p * A.lstride;
    const int s0 = tasks[2 * task], s1 = tasks[2 * task + 1];
    for (int s = s0; s <= s1; s++) {
        const int f = S.first[s];
        const int w = S.first[s + 1] - f;
        const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
        const T* Fs = L + S.loff[s];
        T* t = tbuf + S.row_ptr[s];
        // assemble t: pivot rows from x, update rows zero, plus every child's update rows
        for (int64_t r = lane; r < m; r += 32) t[r] = r < w ? x[f + r] : zero_of<T>();
        __syncwarp();
        for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
            const int ch = S.child_list[c];
            const int64_t nu = (S.row_ptr[ch + 1] - S.row_ptr[ch]) - (S.first[ch + 1] - S.first[ch]);
            const T* tc = tbuf + S.row_ptr[ch + 1] - nu;
            const int32_t* rl = S.rel + S.rel_ptr[ch];
            for (int64_t a = lane; a < nu; a += 32) t[rl[a]] += tc[a];
            __syncwarp();
        }
        const T d0 = lane < w ? Fs[(int64_t)lane * m + lane] : one_of<T>();
        const T d1 = lane + 32 < w ? Fs[(int64_t)(lane + 32) * m + lane + 32] : one_of<T>();
        const T t0 = lane < w ? t[lane] : zero_of<T>();
        const T t1 = lane + 32 < w ? t[lane + 32] : zero_of<T>();
        // y = X t (X: the block's unit-lower inverse, stored below the diagonal), eight columns
        // of X per step; y_i = 0 for i >= w
        T y0 = t0, y1 = t1;
        for (int k0 = 0; k0 + 1 < w; k0 += 8) {
            T xa[8], xb[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int k = k0 + u;
                xa[u] = lane > k && lane < w ? Fs[(int64_t)k * m + lane] : zero_of<T>();
                xb[u] = lane + 32 > k && lane + 32 < w ? Fs[(int64_t)k * m + lane + 32] : zero_of<T>();
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int k = k0 + u;
                const T tk = shfl_t(k < 32 ? t0 : t1, k & 31);
                y0 += xa[u] * tk;
                y1 += xb[u] * tk;
            }
        }
        if (lane < w) x[f + lane] = dev_div(y0, re(d0));
        if (lane + 32 < w) x[f + lane + 32] = dev_div(y1, re(d1));
        // update rows: t[r] -= sum_j L(r, j) y_j, two rows per lane, eight columns per step
        for (int64_t r0 = w; r0 < m; r0 += 64) {
            const int64_t ra = r0 + lane, rb = ra + 32;
            const bool ha = ra < m, hb = rb < m;
            T aa = zero_of<T>(), ab = zero_of<T>();
            for (int j0 = 0; j0 < w; j0 += 8) {
                T la[8], lb[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int j = j0 + u;
                    la[u] = ha && j < w ? Fs[(int64_t)j * m + ra] : zero_of<T>();
                    lb[u] = hb && j < w ? Fs[(int64_t)j * m + rb] : zero_of<T>();
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int j = j0 + u;
                    const T yj = shfl_t(j < 32 ? y0 : y1, j & 31);
                    aa += la[u] * yj;
                    ab += lb[u] * yj;
                }
            }
            if (ha) t[ra] -= aa;
            if (hb) t[rb] -= ab;
        }
        __syncwarp();
    }
}

// task = (first, root): backward over the supernodes root..first
template <typename T>
__global__ void __launch_bounds__(32 * SUB_WARPS) k_sub_bwd(const int32_t* __restrict__ tasks, int ntasks, SnDev S,
                                                           SolveArgs A, const T* __restrict__ L, T* __restrict__ x) {
    pdl_trigger();
    const int task = blockIdx.x * SUB_WARPS + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    const int64_t p = blockIdx.y;
    pdl_wait();
    if (task >= ntasks || (A.skip && A.skip[p])) return;
    x += p * A.xstride;
    L += p * A.lstride;
    const int s0 = tasks[2 * task], s1 = tasks[2 * task + 1];
    for (int s = s1; s >= s0; s--) {
        const int f = S.first[s];
        const int w = S.first[s + 1] - f;
        const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
        const T* Fs = L + S.loff[s];
        const int32_t* rows = S.rows + S.row_ptr[s];
        // z_j = x_j - sum_{r >= w} conj(L(r, j)) x(rows[r]), eight columns per pass
        T z0 = lane < w ? x[f + lane] : zero_of<T>();
        T z1 = lane + 32 < w ? x[f + lane + 32] : zero_of<T>();
        for (int j0 = 0; j0 < w; j0 += 8) {
            T acc[8];
#pragma unroll
            for (int u = 0; u < 8; u++) acc[u] = zero_of<T>();
            for (int64_t r = w + lane; r < m; r += 64) {
                const bool h1 = r + 32 < m;
                const T xa = x[rows[r]];
                const T xb = h1 ? x[rows[r + 32]] : zero_of<T>();
                T la[8], lb[8];
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const bool hj = j0 + u < w;
                    la[u] = hj ? Fs[(int64_t)(j0 + u) * m + r] : zero_of<T>();
                    lb[u] = hj && h1 ? Fs[(int64_t)(j0 + u) * m + r + 32] : zero_of<T>();
                }
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    acc[u] += conj(la[u]) * xa;
                    acc[u] += conj(lb[u]) * xb;
                }
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const T v = warp_sum(acc[u]);
                if (j0 + u == lane) z0 -= v;
                if (j0 + u == lane + 32) z1 -= v;
            }
        }
        // x = X^H z: x_i = z_i + sum_{k > i} conj(X(k, i)) z_k, X(k, i) = Fs[i m + k]
        T o0 = z0, o1 = z1;
        for (int i0 = 0; i0 + 1 < w; i0 += 8) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = i0 + u;
                T a = zero_of<T>();
                if (lane > i && lane < w) a = conj(Fs[(int64_t)i * m + lane]) * z0;
                if (lane + 32 > i && lane + 32 < w) a += conj(Fs[(int64_t)i * m + lane + 32]) * z1;
                v[u] = a;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const T sum = warp_sum(v[u]);
                if (i0 + u == lane) o0 += sum;
                if (i0 + u == lane + 32) o1 += sum;
            }
        }
        if (lane < w) x[f + lane] = o0;
        if (lane + 32 < w) x[f + lane + 32] = o1;
        __syncwarp();
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
    alloc_stream = g_stream;
    cnt = g_bytes;
    auto put = [&](auto*& dptr, const auto& vec) {
        using E = typename std::decay<decltype(vec[0])>::type;
        const size_t b = std::max<size_t>(1, vec.size()) * sizeof(E);
        TMG_CUDA(pool_malloc((void**)&dptr, b, alloc_stream));
        if (cnt) cnt->add((int64_t)b);
        if (!vec.empty())
            TMG_CUDA(cudaMemcpyAsync(dptr, vec.data(), vec.size() * sizeof(E), cudaMemcpyHostToDevice, alloc_stream));
        TMG_CUDA(cudaStreamSynchronize(alloc_stream));   // the host vectors are temporaries
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
    tc_rows = 0;
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
                const int64_t s1 = std::min<int64_t>((kb * MF_NB / MF_SB + 1) * MF_SB, w);
                for (int64_t j0 = t0; j0 < s1; j0 += MF_TILE)
                    for (int64_t i0 = j0; i0 < m; i0 += MF_TILE) {
                        it.push_back(s); it.push_back((int32_t)i0); it.push_back((int32_t)j0);
                        st.upd_cnt++;
                    }
            }
            st.trail_off = (int64_t)it.size();
            std::vector<int> tcf;   // fronts of this step that qualify for the tensor-core update
            for (int pass = 0; pass < 2; pass++)
                for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++) {
                    const int s = S.level_sn[q];
                    const int w = S.sn_first[s + 1] - S.sn_first[s];
                    if (w <= kb * MF_NB) continue;
                    const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                    const int64_t kend = std::min<int64_t>((int64_t)(kb + 1) * MF_NB, w);
                    const bool sb_end = kend == w || kend % MF_SB == 0;   // this pivot block closes a super-block
                    if (!sb_end) continue;
                    const bool tc = m - kend >= tc_min_rows;
                    if (tc != (pass == 1)) continue;
                    if (tc) tcf.push_back(s);
                    for (int64_t j0 = kend; j0 < m; j0 += MF_TILE)
                        for (int64_t i0 = j0; i0 < m; i0 += MF_TILE) {
                            it.push_back(s); it.push_back((int32_t)i0); it.push_back((int32_t)j0);
                            st.trail_cnt++;
                        }
                    if (pass == 0) st.trail_simt = st.trail_cnt;
                }
            // tensor-core groups: fronts packed in order while their staged rows fit the group
            for (size_t f = 0; f < tcf.size();) {
                Step::TcGroup g;
                std::vector<std::pair<int, int64_t>> mem;   // (front, staging offset)
                int64_t rows = 0;
                while (f < tcf.size()) {
                    const int s = tcf[f];
                    const int w = S.sn_first[s + 1] - S.sn_first[s];
                    const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                    const int64_t kend = std::min<int64_t>((int64_t)(kb + 1) * MF_NB, w);
                    if (!mem.empty() && rows + (m - kend) > MF_TC_GROUP_ROWS) break;
                    mem.push_back({s, rows});
                    rows += m - kend;
                    f++;
                }
                tc_rows = std::max(tc_rows, rows);
                g.stage_off = (int64_t)it.size();
                for (auto [s, off] : mem) {
                    const int w = S.sn_first[s + 1] - S.sn_first[s];
                    const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                    const int64_t kend = std::min<int64_t>((int64_t)(kb + 1) * MF_NB, w);
                    for (int64_t r0 = kend; r0 < m; r0 += 16) {
                        it.push_back(s); it.push_back((int32_t)r0); it.push_back((int32_t)(off + r0 - kend));
                        g.stage_cnt++;
                    }
                }
                g.upd_off = (int64_t)it.size();
                for (auto [s, off] : mem) {
                    const int w = S.sn_first[s + 1] - S.sn_first[s];
                    const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
                    const int64_t kend = std::min<int64_t>((int64_t)(kb + 1) * MF_NB, w);
                    for (int64_t j0 = kend; j0 < m; j0 += MF_TILE)
                        for (int64_t i0 = j0; i0 < m; i0 += MF_TILE) {
                            it.push_back(s); it.push_back((int32_t)i0); it.push_back((int32_t)j0);
                            it.push_back((int32_t)(off + i0 - kend)); it.push_back((int32_t)(off + j0 - kend));
                            g.upd_cnt++;
                        }
                }
                st.tc.push_back(g);
            }
            steps.push_back(st);
        }
    }
    put(items, it);
    if (std::getenv("TMG_VERBOSE")) {
        int64_t simt = 0, tct = 0, groups = 0;
        for (const auto& st : steps) {
            simt += st.trail_simt;
            for (const auto& g : st.tc) { tct += g.upd_cnt; groups++; }
        }
        std::fprintf(stderr, "[tmg] factor plan n=%d: %lld trail tiles on the SIMT pipe, %lld on the tensor cores "
                     "(%lld groups, %lld staging rows)\n", n, (long long)simt, (long long)tct, (long long)groups,
                     (long long)tc_rows);
    }
    // triangular-solve schedule (64-wide diagonal blocks)
    std::vector<int32_t> si;
    plan64 = build_solve_plan(S, 64, SV_RR, si);
    put(sitems, si);
    if (std::getenv("TMG_VERBOSE")) {
        int64_t launches = 0;
        for (const auto& L : plan64.levels) {
            if (!L.gath_cnt) continue;
            launches += 3;
            for (size_t b = 0; b < L.ftri_cnt.size(); b++) launches += (L.ftri_cnt[b] > 0) + (L.btri_cnt[b] > 0);
        }
        std::fprintf(stderr, "[tmg] solve plan n=%d: %d subtrees hold %d of %d fronts; %lld launches per solve\n", n,
                     plan64.sub_cnt, plan64.sub_fronts, ns, (long long)(launches + 2 * (plan64.sub_cnt > 0)));
    }
}

void DevSymbolic::swap(DevSymbolic& o) noexcept {
    using std::swap;
    swap(n, o.n); swap(ns, o.ns); swap(max_front, o.max_front);
    swap(l_entries, o.l_entries); swap(u_entries, o.u_entries); swap(t_entries, o.t_entries);
    swap(l_stored, o.l_stored);
    swap(sn_first, o.sn_first); swap(sn_rows, o.sn_rows); swap(rel, o.rel); swap(child_ptr, o.child_ptr);
    swap(child_list, o.child_list); swap(sn_row_ptr, o.sn_row_ptr); swap(loff, o.loff); swap(uoff, o.uoff);
    swap(rel_ptr, o.rel_ptr); swap(perm, o.perm); swap(level_sn, o.level_sn); swap(items, o.items);
    swap(sitems, o.sitems); swap(dest, o.dest); swap(conj, o.conj); swap(nlower, o.nlower); swap(flops, o.flops);
    swap(bytes, o.bytes); swap(alloc_stream, o.alloc_stream); swap(cnt, o.cnt); swap(steps, o.steps);
    swap(tc_rows, o.tc_rows); swap(tc_min_rows, o.tc_min_rows); swap(plan64, o.plan64); swap(level_ptr, o.level_ptr);
}

void DevSymbolic::release() {
    if (bytes && cnt) cnt->cur -= (int64_t)bytes;
    for (void* p : {(void*)sn_first, (void*)sn_rows, (void*)rel, (void*)child_ptr, (void*)child_list,
                    (void*)sn_row_ptr, (void*)loff, (void*)uoff, (void*)rel_ptr, (void*)perm, (void*)level_sn,
                    (void*)items, (void*)sitems, (void*)dest, (void*)conj})
        if (p) cudaFreeAsync(p, alloc_stream);
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
void mf_invert_diag(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt);

template <typename T>
void mf_factor(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, int* status, bool tensor_cores) {
    const bool tc = tensor_cores && std::is_same<T, zf>::value && S.tc_rows > 0;
    TcWork wk;
    const size_t upd_smem = 2 * MF_NB * MF_TILE * sizeof(T);
    static std::once_flag attr_once;
    std::call_once(attr_once, [&]() {
        TMG_CUDA(cudaFuncSetAttribute(k_update<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)upd_smem));
    });
    const SnDev sn = S.sn();
    const unsigned B = bt.B;
    for (const auto& stp : S.steps) {
        if (stp.uzero_cnt) {
            // one warp per column of the largest update block of the step (8 per CTA; uzero_max
            // counts its entries)
            const int64_t ucols = (int64_t)std::ceil(std::sqrt((double)stp.uzero_max));
            const unsigned gx = (unsigned)std::min<int64_t>(std::max<int64_t>(1, ceil_div(ucols, 8)), 2048);
            const unsigned gy = (unsigned)std::min<int64_t>(stp.uzero_cnt, 65535);
            TMG_LAUNCH(k_uzero<T>, dim3(gx, gy, B), 256, 0, st, S.items + stp.uzero_off, stp.uzero_cnt, sn, bt.U,
                       bt.ustride);
        }
        for (size_t r = 0; r < stp.ext_off.size(); r++) {
            if (stp.ext_cnt[r] == 0) continue;
            const unsigned gx = (unsigned)std::min<int64_t>(std::max<int64_t>(1, ceil_div(stp.ext_max[r], 8)), 2048);
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
            TMG_LAUNCH(k_update<T>, dim3(stp.upd_cnt, B), 256, upd_smem, st, S.items + stp.upd_off, stp.kb * MF_NB, MF_NB,
                       0, sn, bt.L, bt.U, bt.lstride, bt.ustride);
        const int32_t ntrail = tc ? stp.trail_simt : stp.trail_cnt;
        if (ntrail)
            TMG_LAUNCH(k_update<T>, dim3(ntrail, B), 256, upd_smem, st, S.items + stp.trail_off,
                       (stp.kb * MF_NB / MF_SB) * MF_SB, MF_SB, 1, sn, bt.L, bt.U, bt.lstride, bt.ustride);
        if constexpr (std::is_same<T, zf>::value) {
            if (tc) mf_trail_tc(st, S, bt, stp, wk);
        }
    }
    TMG_CHECK_LAUNCH();
    if (tc) {
        const int e = wk.read_error(st);
        if (e) throw cuda_error("tensor-core Schur update: a bounded wait expired (code " + std::to_string(e) + ")");
    }
    mf_invert_diag<T>(st, S, bt);
}

template <typename T>
void mf_invert_diag(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt) {
    constexpr int NB = sv_nb<T>();
    const auto& P = S.plan64;
    const SnDev sn = S.sn();
    const unsigned B = bt.B;
    if (P.inv_small_cnt)
        TMG_LAUNCH((k_inv_small<T, NB>), dim3((unsigned)ceil_div(P.inv_small_cnt, inv_wpc<T>()), B),
                   32 * inv_wpc<T>(), 0, st,
                   S.sitems + P.inv_small_off, P.inv_small_cnt, sn, bt.L, bt.lstride);
    if (P.inv_large_cnt) {
        const size_t smem = (size_t)NB * (NB + 1) * sizeof(T);
        static std::once_flag attr_once;
        std::call_once(attr_once, [&]() {
            TMG_CUDA(cudaFuncSetAttribute(k_inv_large<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        });
        TMG_LAUNCH((k_inv_large<T, NB>), dim3(P.inv_large_cnt, B), 256, smem, st, S.sitems + P.inv_large_off, sn, bt.L,
                   bt.lstride);
    }
    TMG_CHECK_LAUNCH();
}

template <typename T>
void mf_solve(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, T* x, T* tbuf, const int* skip) {
    static_assert(sv_nb<T>() == 64, "the solve kernels work on 64-wide diagonal blocks");
    const auto& P = S.plan64;
    const int nlev = (int)S.level_ptr.size() - 1;
    const SnDev sn = S.sn();
    const SolveArgs A{bt.lstride, (int64_t)S.n, S.t_entries, skip};
    const unsigned B = bt.B;
    const size_t xs = (size_t)64 * XS_LD * sizeof(T);
    static std::once_flag attr_once;
    std::call_once(attr_once, [&]() {
        TMG_CUDA(cudaFuncSetAttribute(k_fwd_gather<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs));
        TMG_CUDA(cudaFuncSetAttribute(k_fwd_tri<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs));
        TMG_CUDA(cudaFuncSetAttribute(k_bwd_rect<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(xs + SV_CH * sizeof(T))));
        TMG_CUDA(cudaFuncSetAttribute(k_bwd_tri<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xs));
    });
    // the levels near the leaves hold narrow fronts: their staged blocks are sized to the
    // level's widest front (and the gathered rows to its largest rectangle), so more CTAs fit
    auto xs_of = [&](const DevSymbolic::SolveLevel& L) {
        return (size_t)std::min(64, std::max(1, L.maxw)) * XS_LD * sizeof(T);
    };
    auto chunk_of = [&](const DevSymbolic::SolveLevel& L) {
        return (int)std::max<int64_t>(1, std::min<int64_t>(SV_CH, L.maxu));
    };
    const unsigned sub_grid = (unsigned)ceil_div(P.sub_cnt, SUB_WARPS);
    if (P.sub_cnt)
        TMG_LAUNCH_PDL(k_sub_fwd<T>, dim3(sub_grid, B), 32 * SUB_WARPS, 0, st, S.sitems + P.sub_off, P.sub_cnt, sn, A,
                       bt.L, x, tbuf);
    for (int l = 0; l < nlev; l++) {
        const auto& L = P.levels[l];
        if (!L.gath_cnt) continue;
        TMG_LAUNCH_PDL(k_fwd_gather<T>, dim3(L.gath_cnt, B), 256, xs_of(L), st, S.sitems + L.gath_off, sn, A, bt.L, x,
                       tbuf);
        for (size_t b = 0; b < L.ftri_cnt.size(); b++)
            if (L.ftri_cnt[b])
                TMG_LAUNCH_PDL(k_fwd_tri<T>, dim3(L.ftri_cnt[b], B), 256, xs, st, S.sitems + L.ftri_off[b], (int)b, sn, A,
                               bt.L, x, tbuf);
        if (L.frect_cnt)
            TMG_LAUNCH_PDL(k_fwd_rect<T>, dim3(L.frect_cnt, B), 256, 0, st, S.sitems + L.frect_off, sn, A, bt.L, tbuf);
    }
    for (int l = nlev - 1; l >= 0; l--) {
        const auto& L = P.levels[l];
        if (L.brect_cnt)
            TMG_LAUNCH_PDL(k_bwd_rect<T>, dim3(L.brect_cnt, B), 256, xs_of(L) + chunk_of(L) * sizeof(T), st,
                           S.sitems + L.brect_off, sn, A, bt.L, x, tbuf, chunk_of(L));
        for (int b = (int)L.btri_cnt.size() - 1; b >= 1; b--)
            if (L.btri_cnt[b])
                TMG_LAUNCH_PDL(k_bwd_tri<T>, dim3(L.btri_cnt[b], B), 256, xs, st, S.sitems + L.btri_off[b], b, sn, A, bt.L,
                               x, tbuf);
    }
    if (P.sub_cnt)
        TMG_LAUNCH_PDL(k_sub_bwd<T>, dim3(sub_grid, B), 32 * SUB_WARPS, 0, st, S.sitems + P.sub_off, P.sub_cnt, sn, A,
                       bt.L, x);
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
    template void mf_factor<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, int*, bool); \
    template void mf_scatter<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, const T*); \
    template void mf_solve<T>(cudaStream_t, const DevSymbolic&, const Batch<T>&, T*, T*, const int*); \
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
