// Host runtime + C ABI of the GB300 cyclic-symmetry modal solve.
//
// Data flow for one speed (reference: src/cyclic_solver.cpp:725-1357):
//   element kernels -> candidate-pattern gathers (K, M, Komega, G, Ksigma)      [device]
//   static prestress: (Tr^T K Tr) projection, supernodal LDL^T, solve            [device]
//   cyclic projections Kc/Kp/Mc/Mp (+Gc/Gp): two-stage gathers with pruning      [device]
//   per harmonic: operator K_k - sigma M_k formed on the union pattern, scattered
//   into fronts, multifrontal LDL^H (FP64, or FP32 + FP64 refinement), Lanczos    [device]
//   small sectors (n <= 200): dense generalized eigensolver, one CTA per problem   [device]
//   with Coriolis, k > 0: the Lancaster pencil on the 2n block pattern, dense or
//   shift-invert Lanczos, forward / backward selection                            [device]
// Host work is pattern-only (symbolic analysis, cached per pattern) plus the small
// per-restart control decisions.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>
#include <random>
#include <set>
#include <thread>

#include "../../include/turbomodal_gb300.h"
#include "engine.hpp"
#include "dense.cuh"
#include "fe.cuh"

namespace tmg {

constexpr double PI = 3.14159265358979323846;

// ------------------------------------------------------------------------------------
// small device kernels of the runtime
// ------------------------------------------------------------------------------------
__global__ void k_proj1(int64_t n, const int64_t* __restrict__ p, const int64_t* __restrict__ src,
                        const double* __restrict__ coef, const double* __restrict__ A, double* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    double acc = 0.0;
    for (int64_t q = p[e]; q < p[e + 1]; q++) {
        const double t = coef[q] * A[src[q]];
        acc = (q == p[e]) ? t : acc + t;
    }
    out[e] = acc;
}

__global__ void k_proj2(int64_t n, const int64_t* __restrict__ p, const int64_t* __restrict__ src,
                        const double* __restrict__ coef, const double* __restrict__ I, double tol,
                        double* __restrict__ out, uint8_t* __restrict__ flag) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    double acc = 0.0;
    for (int64_t q = p[e]; q < p[e + 1]; q++) {
        const double t = I[src[q]] * coef[q];
        acc = (q == p[e]) ? t : acc + t;
    }
    out[e] = acc;
    flag[e] = fabs(acc) > tol ? 1 : 0;
}

__global__ void k_gather(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ src,
                         double* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) out[e] = idx[e] >= 0 ? src[idx[e]] : 0.0;
}

__global__ void k_gather_masked(int64_t n, const int64_t* __restrict__ idx, const double* __restrict__ v,
                                const uint8_t* __restrict__ keep, double* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) out[e] = keep[idx[e]] ? v[idx[e]] : 0.0;
}

__global__ void k_mask_values(int64_t n, const double* __restrict__ v, const uint8_t* __restrict__ keep,
                              double* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) out[e] = keep[e] ? v[e] : 0.0;
}

template <typename T>
__global__ void k_gather_t(int64_t n, const int64_t* __restrict__ idx, const T* __restrict__ src, T* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) out[e] = src[idx[e]];
}

template <typename T, typename U>
__global__ void k_gather_conv(int64_t n, const int64_t* __restrict__ idx, const U* __restrict__ src, T* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e < n) out[e] = conv<T, U>(src[idx[e]]);
}

// Complex harmonic operator on the union pattern:
//   ((kc + P kp) + conj(P) kph) - sigma ((mc + P mp) + conj(P) mph)
// with missing constituents read as exact zeros (the reference's sparse-sum semantics,
// src/cyclic_solver.cpp:946-947, src/hermitian_lanczos.cpp:15).
__global__ void k_form_complex(int64_t n, const int64_t* __restrict__ ikc, const int64_t* __restrict__ ikp,
                               const int64_t* __restrict__ ikh, const int64_t* __restrict__ imc,
                               const int64_t* __restrict__ imp, const int64_t* __restrict__ imh,
                               const double* __restrict__ kc, const double* __restrict__ kp,
                               const double* __restrict__ mc, const double* __restrict__ mp, double Pr, double Pi,
                               double sigma, double kscale, zd* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double a = ikc[e] >= 0 ? kc[ikc[e]] : 0.0;
    const double b = ikp[e] >= 0 ? kp[ikp[e]] : 0.0;
    const double c = ikh[e] >= 0 ? kp[ikh[e]] : 0.0;
    const double am = imc[e] >= 0 ? mc[imc[e]] : 0.0;
    const double bm = imp[e] >= 0 ? mp[imp[e]] : 0.0;
    const double cm = imh[e] >= 0 ? mp[imh[e]] : 0.0;
    const zd P{Pr, Pi}, Pc{Pr, -Pi};
    const zd kk = (zd{a, 0.0} + P * zd{b, 0.0}) + Pc * zd{c, 0.0};
    const zd mm = (zd{am, 0.0} + P * zd{bm, 0.0}) + Pc * zd{cm, 0.0};
    out[e] = kscale * kk - sigma * mm;
}

// Real (k = 0 or N/2) sums (kc + s kp) + s kph and their |v| > 1e-15 flags.
__global__ void k_form_real_sum(int64_t n, const int64_t* __restrict__ ic, const int64_t* __restrict__ ip,
                                const int64_t* __restrict__ ih, const double* __restrict__ c,
                                const double* __restrict__ p, double s, double* __restrict__ out,
                                uint8_t* __restrict__ flag) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double a = ic[e] >= 0 ? c[ic[e]] : 0.0;
    const double b = ip[e] >= 0 ? p[ip[e]] : 0.0;
    const double h = ih[e] >= 0 ? p[ih[e]] : 0.0;
    const double v = (a + s * b) + s * h;
    out[e] = v;
    flag[e] = fabs(v) > 1e-15 ? 1 : 0;
}

__global__ void k_form_real_op(int64_t n, const int64_t* __restrict__ ik, const int64_t* __restrict__ im,
                               const double* __restrict__ kv, const double* __restrict__ mv, double sigma,
                               double kscale, double* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double a = ik[e] >= 0 ? kv[ik[e]] : 0.0;
    const double b = im[e] >= 0 ? mv[im[e]] : 0.0;
    out[e] = kscale * a - sigma * b;
}

// u_red (reduced numbering) = scatter of x_free; out_full = T0 u_red with right rows * P
__global__ void k_expand(int32_t nfull, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                         const double* __restrict__ tv, const uint8_t* __restrict__ isr, const int32_t* __restrict__ r2f,
                         const zd* __restrict__ x, int64_t ldx, zd P, zd* __restrict__ out, int64_t ldo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nfull) return;
    const int64_t v = blockIdx.y;
    zd s{0.0, 0.0};
    for (int64_t q = rp[i]; q < rp[i + 1]; q++) {
        const int32_t f = r2f[ci[q]];
        if (f >= 0) s += tv[q] * x[v * ldx + f];
    }
    out[v * ldo + i] = isr[i] ? s * P : s;
}

// Modal mass N Re(phi^H M phi) of every expanded mode (python/turbomodal/solver.py:91-103): one
// warp per sector column j forms (M phi)_j over the candidate pattern (M is symmetric, so its
// CSC columns are its rows) and multiplies by conj(phi_j); each CTA writes its partial sum,
// and k_mass_sum adds the partials in a fixed order (deterministic).
constexpr int MASS_BLOCKS = 304;
__global__ void __launch_bounds__(256) k_mass_part(int32_t ndof, const int64_t* __restrict__ cp,
                                                   const int32_t* __restrict__ ci, const double* __restrict__ mv,
                                                   const zd* __restrict__ phi, int64_t ldp, double* __restrict__ part) {
    __shared__ double red[8];
    const int64_t v = blockIdx.y;
    const zd* f = phi + v * ldp;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc = 0.0;
    for (int64_t j = (int64_t)blockIdx.x * 8 + warp; j < ndof; j += (int64_t)gridDim.x * 8) {
        zd y{0.0, 0.0};
        for (int64_t q = cp[j] + lane; q < cp[j + 1]; q += 32) y += mv[q] * f[ci[q]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            y.x += __shfl_xor_sync(0xffffffffu, y.x, o);
            y.y += __shfl_xor_sync(0xffffffffu, y.y, o);
        }
        acc += f[j].x * y.x + f[j].y * y.y;   // Re(conj(phi_j) y_j)
    }
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int q = 0; q < 8; q++) t += red[q];
        part[v * gridDim.x + blockIdx.x] = t;
    }
}

__global__ void k_mass_sum(int nb, const double* __restrict__ part, double scale, double* __restrict__ out) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    for (int q = 0; q < nb; q++) t += part[(int64_t)v * nb + q];
    out[v] = scale * t;
}

__global__ void k_real_to_complex(int64_t n, const double* __restrict__ a, zd* __restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = zd{a[i], 0.0};
}

// F_cyc = Tr^T F (gather over the transposed transformation), and u = Tr u_cyc
__global__ void k_csr_real(int32_t nrows, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                           const double* __restrict__ v, const double* __restrict__ x, double* __restrict__ y) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= nrows) return;
    double s = 0.0;
    for (int64_t q = rp[i]; q < rp[i + 1]; q++) s += v[q] * x[ci[q]];
    y[i] = s;
}

template <typename T>
__global__ void k_restart_norm(int64_t n, int nev, const T* __restrict__ dot, const T* __restrict__ f,
                               const T* __restrict__ Mf, T* __restrict__ V, T* __restrict__ MV,
                               double* __restrict__ beta) {
    const double b = sqrt(fabs(re(dot[0])));
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (b > 1e-14) {
        if (i == 0) beta[nev - 1] = b;
        if (i < n) {
            V[(int64_t)nev * n + i] = f[i] / b;
            MV[(int64_t)nev * n + i] = Mf[i] / b;
        }
    } else if (i == 0) {
        beta[nev - 1] = 0.0;
    }
}

template <typename T, typename U>
__global__ void k_conv_copy(int64_t n, const U* __restrict__ a, T* __restrict__ b) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = conv<T, U>(a[i]);
}

template <typename T>
__global__ void k_gather_i32(int64_t n, const int32_t* __restrict__ idx, const T* __restrict__ src, T* __restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

template <typename T>
__global__ void k_scatter_vec(int64_t n, const int32_t* __restrict__ idx, const T* __restrict__ src, T* __restrict__ dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) dst[idx[i]] = src[i];
}

// ------------------------------------------------------------------------------------
// host helpers
// ------------------------------------------------------------------------------------
inline unsigned nblk(int64_t n, int b = 256) { return (unsigned)std::max<int64_t>(1, ceil_div(n, b)); }

Pattern transpose_map(const Pattern& A, std::vector<int64_t>& map) {
    Pattern B;
    B.nrows = A.ncols; B.ncols = A.nrows;
    B.p.assign(B.ncols + 1, 0);
    for (int32_t r : A.i) B.p[r + 1]++;
    for (int32_t c = 0; c < B.ncols; c++) B.p[c + 1] += B.p[c];
    B.i.resize(A.i.size());
    map.assign(A.i.size(), -1);
    std::vector<int64_t> pos(B.p.begin(), B.p.end() - 1);
    for (int32_t j = 0; j < A.ncols; j++)
        for (int64_t q = A.p[j]; q < A.p[j + 1]; q++) {
            const int64_t d = pos[A.i[q]]++;
            B.i[d] = j;
            map[d] = q;
        }
    return B;
}

Flagged flagged(const Pattern& cand, const std::vector<uint8_t>& f) {
    Flagged F;
    F.pat.nrows = cand.nrows; F.pat.ncols = cand.ncols;
    F.pat.p.assign(cand.ncols + 1, 0);
    for (int32_t j = 0; j < cand.ncols; j++) {
        for (int64_t q = cand.p[j]; q < cand.p[j + 1]; q++)
            if (f[q]) { F.pat.i.push_back(cand.i[q]); F.cand.push_back(q); }
        F.pat.p[j + 1] = (int64_t)F.pat.i.size();
    }
    return F;
}

// Sub-pattern selection by a predicate on (row, col), keeping the source slot index.
template <typename Pred>
Flagged select(const Pattern& A, const std::vector<int64_t>& src, Pred pred) {
    Flagged F;
    F.pat.nrows = A.nrows; F.pat.ncols = A.ncols;
    F.pat.p.assign(A.ncols + 1, 0);
    for (int32_t j = 0; j < A.ncols; j++) {
        for (int64_t q = A.p[j]; q < A.p[j + 1]; q++)
            if (pred(A.i[q], j)) { F.pat.i.push_back(A.i[q]); F.cand.push_back(src.empty() ? q : src[q]); }
        F.pat.p[j + 1] = (int64_t)F.pat.i.size();
    }
    return F;
}

// Build the projection chain for C = (Tt * A) * T where A's entries live at `asrc`
// positions of a device value array.
void build_chain(ProjChain& ch, const Pattern& Tt, const std::vector<double>& Ttv, const Flagged& A,
                 const Pattern& T, const std::vector<double>& Tv) {
    Product P1 = product(Tt, A.pat);
    Product P2 = product(P1.C, T);
    ch.C = P2.C;
    ch.n1 = P1.C.nnz();
    ch.n2 = P2.C.nnz();
    std::vector<int64_t> src1(P1.a_slot.size()), src2(P2.a_slot.size());
    std::vector<double> c1(P1.a_slot.size()), c2(P2.a_slot.size());
    for (size_t q = 0; q < P1.a_slot.size(); q++) { c1[q] = Ttv[P1.a_slot[q]]; src1[q] = A.cand[P1.b_slot[q]]; }
    for (size_t q = 0; q < P2.a_slot.size(); q++) { src2[q] = P2.a_slot[q]; c2[q] = Tv[P2.b_slot[q]]; }
    ch.p1.upload(P1.cptr); ch.src1.upload(src1); ch.coef1.upload(c1);
    ch.p2.upload(P2.cptr); ch.src2.upload(src2); ch.coef2.upload(c2);
    ch.I.alloc(ch.n1); ch.Cv.alloc(ch.n2); ch.Cf.alloc(ch.n2);
}

void run_chain(cudaStream_t st, ProjChain& ch, const double* A, double tol) {
    if (ch.n1) TMG_LAUNCH(k_proj1, nblk(ch.n1), 256, 0, st, ch.n1, ch.p1.p, ch.src1.p, ch.coef1.p, A, ch.I.p);
    if (ch.n2) TMG_LAUNCH(k_proj2, nblk(ch.n2), 256, 0, st, ch.n2, ch.p2.p, ch.src2.p, ch.coef2.p, ch.I.p, tol, ch.Cv.p, ch.Cf.p);
    TMG_CHECK_LAUNCH();
}

// Free-space extraction of the pruned projection (src/cyclic_solver.cpp:644-658).
void extract_free(cudaStream_t st, const ProjChain& ch, const std::vector<int32_t>& r2free, int32_t nfree,
                  FreeMat& out) {
    std::vector<uint8_t> f = ch.Cf.download();
    out.pat.nrows = out.pat.ncols = nfree;
    out.pat.p.assign(nfree + 1, 0);
    out.pat.i.clear();
    std::vector<int64_t> idx;
    for (int32_t j = 0; j < ch.C.ncols; j++) {
        const int32_t fj = r2free[j];
        if (fj < 0) continue;
        for (int64_t q = ch.C.p[j]; q < ch.C.p[j + 1]; q++) {
            const int32_t fi = r2free[ch.C.i[q]];
            if (fi >= 0 && f[q]) { out.pat.i.push_back(fi); idx.push_back(q); }
        }
        out.pat.p[fj + 1] = (int64_t)out.pat.i.size();
    }
    for (int32_t j = 0; j < nfree; j++) out.pat.p[j + 1] = std::max(out.pat.p[j + 1], out.pat.p[j]);
    out.idx.upload(idx);
    out.v.alloc(idx.size());
    if (!idx.empty()) TMG_LAUNCH(k_gather, nblk(idx.size()), 256, 0, st, (int64_t)idx.size(), out.idx.p, ch.Cv.p, out.v.p);
    TMG_CHECK_LAUNCH();
}

// Structural free-space pattern of a projection chain (every product entry, before pruning).
void struct_free(const ProjChain& ch, const std::vector<int32_t>& r2free, int32_t nfree, FreeMat& out) {
    out.spat.nrows = out.spat.ncols = nfree;
    out.spat.p.assign(nfree + 1, 0);
    out.spat.i.clear();
    std::vector<int64_t> idx;
    for (int32_t j = 0; j < ch.C.ncols; j++) {
        const int32_t fj = r2free[j];
        if (fj < 0) continue;
        for (int64_t q = ch.C.p[j]; q < ch.C.p[j + 1]; q++) {
            const int32_t fi = r2free[ch.C.i[q]];
            if (fi >= 0) { out.spat.i.push_back(fi); idx.push_back(q); }
        }
        out.spat.p[fj + 1] = (int64_t)out.spat.i.size();
    }
    for (int32_t j = 0; j < nfree; j++) out.spat.p[j + 1] = std::max(out.spat.p[j + 1], out.spat.p[j]);
    out.sidx.upload(idx);
    out.sv.alloc(idx.size());
}

// Values on the structural pattern: the pruned value where the entry survives, else 0.
void struct_values(cudaStream_t st, const ProjChain& ch, FreeMat& out) {
    if (out.sv.n)
        TMG_LAUNCH(k_gather_masked, nblk(out.sv.n), 256, 0, st, (int64_t)out.sv.n, out.sidx.p, ch.Cv.p, ch.Cf.p,
                   out.sv.p);
    TMG_CHECK_LAUNCH();
}

// Union of patterns with per-constituent index maps, CSR view and lower triangle.
void build_union(UnionMaps& um, const std::vector<const Pattern*>& parts) {
    um.U = pattern_union(parts);
    um.maps.clear();
    for (const Pattern* P : parts) {
        std::vector<int64_t> loc = locate(um.U, *P);
        std::vector<int64_t> m(um.U.nnz(), -1);
        for (size_t q = 0; q < loc.size(); q++) m[loc[q]] = (int64_t)q;
        DVec<int64_t> d;
        d.upload(m);
        um.maps.push_back(std::move(d));
    }
    std::vector<int64_t> tmap;
    Pattern Ut = transpose_map(um.U, tmap);   // CSC of U^T == CSR of U
    um.csr2csc.upload(tmap);
    um.csr_rowptr.upload(Ut.p);
    um.csr_col.upload(Ut.i);
    um.lower = lower_triangle(um.U);
    std::vector<int64_t> l2c;
    std::vector<int32_t> lr, lc;
    for (int32_t j = 0; j < um.U.ncols; j++)
        for (int64_t q = um.U.p[j]; q < um.U.p[j + 1]; q++)
            if (um.U.i[q] >= j) { l2c.push_back(q); lr.push_back(um.U.i[q]); lc.push_back(j); }
    um.lower2csc.upload(l2c);
    um.low_row.upload(lr);
    um.low_col.upload(lc);
}

}  // namespace tmg

// =====================================================================================
// Context
// =====================================================================================
using namespace tmg;

// Supernode shapes the autotuner chooses between: relaxed amalgamation of the fundamental
// supernodes (explicit zeros within `relax` of the stored entries, fronts at most `maxw`
// columns wide, 0 = no cap) and the row threshold of the tensor-core trailing update.
struct TuneCand {
    double relax = 0.0;
    int32_t maxw = 0;
    int32_t tc_min = MF_TC_MIN_ROWS;
};
struct TuneRow {
    TuneCand cand;
    double factor_ms = 0.0, solve_ms = 0.0, score_ms = 0.0;
    int64_t stored = 0;           // L entries per problem
    int32_t supernodes = 0;
};

struct ResultHost {
    int32_t k = 0;
    double rpm = 0.0;
    std::vector<double> freqs;
    std::vector<int32_t> whirl;
    std::vector<zd> shapes;          // ndof x m
    std::vector<double> modal_mass;  // N Re(phi^H M phi) per mode (full annulus)
    int32_t converged = 0, iterations = 0, status = 0;
    double max_residual = 0.0, refine_residual = 0.0;
    int64_t solves = 0, applies = 0;
};

struct tmg_context {
    // device bytes this context holds (current, peak); first member, so it outlives every
    // buffer that counts itself in it during destruction
    ByteCount bytes;
    std::mutex mu;                // phase timings and the error text, written by a batch's helper thread too
    cudaStream_t st2 = nullptr;   // stream of the real-harmonic batch run beside the complex one
    int device = 0;
    cudaStream_t st = nullptr;
    size_t budget = 0;
    std::string err;
    std::unique_ptr<Sector> sec;
    // candidate-pattern matrices
    CandMat K, M, Kw, G, Ks, Keff;
    bool have_KM = false;
    double kw_omega = -1.0;
    // static prestress operator (k = 0 reduced stiffness without hub DOFs)
    bool static_ready = false;
    ProjChain stat_chain;
    FreeMat stat_free;
    OpSymbolic stat_sym;
    UnionMaps stat_union;
    DVec<double> stat_L, stat_t, stat_x, stat_vals;
    std::vector<int32_t> stat_free_idx;     // free position -> reduced index
    DVec<int32_t> dstat_free_idx;
    DVec<double> u_static;
    // prepared speed
    bool prepared = false;
    double rpm = 0.0;
    bool coriolis = false;
    ProjChain chK[2], chM[2], chG[2];
    Flagged fK, fM, fG;
    FreeMat Kcf, Kpf, Mcf, Mpf, Gcf, Gpf;
    std::vector<int64_t> kpT, mpT;
    Pattern KpfH, MpfH;
    // operators
    UnionMaps opC, opMC;                 // complex harmonic operator and its mass part
    OpSymbolic symC;
    std::string symC_key;
    UnionMaps W0, WM0;                   // real-sum domains (Kc + s Kp + s Kp^H)
    Symbolic symRef[3];                  // analyses of the reference patterns (tmg_symbolic)
    std::string symRef_key[3];
    struct RealOp {
        FreeMat Kr, Mr;                   // filtered matrices (reference patterns)
        DVec<double> Ks, Ms;              // the same values on the structural domains W, W_M
        bool valid = false;
    } real[2];                            // 0: k = 0, 1: k = N/2
    // k = 0 and k = N/2 solved as one batch: operator on W, mass on W_M (structural domains)
    UnionMaps pairOp, pairM;
    OpSymbolic pairSym;
    std::string pair_key;
    // the operator-pattern state of the other regime (rest vs speed) last seen, kept so that a
    // sweep that returns to it reuses its unions, maps and symbolic analyses
    struct PatternState {
        std::string key;
        UnionMaps opC, opMC, W0, WM0, pairOp, pairM;
        OpSymbolic symC, pairSym;
        TuneCand tune_choice;
        std::string tuned_key;
    } stash;
    // Coriolis QEP: gyroscopic sum domain W_G = Gc u Gp u Gp^H and the Lancaster block maps
    // of the shifted operator L1 - sigma L2 and of L2 over (W, W_M, W_G)
    std::vector<int64_t> gpT;
    Pattern GpfH;
    UnionMaps WG0;
    // Refinement deflation across the speeds of a sweep (off unless the environment sets
    // TMG_DEFLATE when the context is created): the DEFL_M lowest eigenvectors of every complex
    // harmonic from the last solve, valid while the operator pattern keeps `recycle_key`.
    bool deflate = false;
    bool autotune = false;        // tune the complex operator's supernode shapes on first use
    std::vector<TuneRow> tune_rows;   // trials of the last tuning (empty: none ran)
    TuneCand tune_choice;         // shapes of the current complex analysis
    double solves_per_factor = 0.0;   // FP32 solves per factorisation seen in the last mixed batch
    std::string tuned_key;        // pattern the current complex analysis was tuned for
    double shift = 1.0;           // sigma of the standard path (cyclic_solver.cpp:1017)
    bool tensor_cores = false;    // tcgen05 trailing updates in the complex FP32 factorisation
    double refine_tol = 1e-10;    // relative residual target of a refined (mixed) solve
    std::string recycle_key;
    std::map<int, DVec<zd>> recycle;
    struct Qep {
        DVec<int64_t> sk, sm, sg, sk2, sm2, sg2;
        DVec<int8_t> blk, blk2;
        UnionMaps op, l2;
        OpSymbolic sym;
        std::string key;
    } qep;
    std::vector<ResultHost> results;
    double phase_ms[9] = {0};
    int64_t launches = 0;
    // expansion maps (CSR of T(0), right-DOF flags, reduced -> free)
    DVec<int64_t> dT0_rp;
    DVec<int32_t> dT0_ci, d_r2free;
    DVec<double> dT0_v;
    DVec<uint8_t> d_isr;
    // profiling mode: CUDA-event timing of every triangular-solve graph launch
    bool profile = false;
    double solve_ms = 0.0, solve_bytes = 0.0;
    int64_t solve_count = 0;
    cudaEvent_t pev0 = nullptr, pev1 = nullptr;
};

namespace {

// Free device memory plus what this process's stream-ordered pool holds unused.
size_t device_free_bytes(int device) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t reserved = 0, used = 0;
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used);
        if (reserved > used) fr += (size_t)(reserved - used);
    }
    return fr;
}

// error text written while a batch's helper thread may also write it
void note_err(tmg_context* c, const std::string& m) {
    std::lock_guard<std::mutex> lk(c->mu);
    c->err = m;
}

int set_err(tmg_context* c, int code, const std::string& m) {
    if (c) c->err = m;
    return code;
}

template <typename F>
int guarded(tmg_context* c, F&& fn) {
    try {
        cudaSetDevice(c->device);
        g_stream = c->st;
        g_bytes = &c->bytes;
        struct Reset { ~Reset() { g_bytes = nullptr; } } reset;
        return fn();
    } catch (const cuda_error& e) {
        return set_err(c, TMG_ERR_CUDA, e.what());
    } catch (const numeric_error& e) {
        return set_err(c, TMG_ERR_NUMERIC, e.what());
    } catch (const std::bad_alloc&) {
        return set_err(c, TMG_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return set_err(c, TMG_ERR_ARG, e.what());
    }
}

// ---- sector set-up -------------------------------------------------------------------
void setup_sector(tmg_context* c, const tmg_sector_desc* d) {
    auto S = std::make_unique<Sector>();
    S->nn = d->num_nodes; S->ne = d->num_elements; S->ns = d->num_sectors; S->axis = d->rotation_axis;
    S->E = d->E; S->nu = d->nu; S->rho = d->rho;
    if (S->nn <= 0 || S->ne <= 0) throw std::invalid_argument("empty mesh");
    if (S->ns <= 0) throw std::invalid_argument("num_sectors must be positive");
    if (S->axis < 0 || S->axis > 2) throw std::invalid_argument("rotation_axis must be 0, 1 or 2");
    if (S->E <= 0.0) throw std::invalid_argument("Young's modulus E must be positive");
    if (S->nu <= 0.0 || S->nu >= 0.5) throw std::invalid_argument("Poisson's ratio nu must be in (0, 0.5)");
    if (S->rho <= 0.0) throw std::invalid_argument("Density rho must be positive");
    S->X.assign(d->coords, d->coords + (size_t)3 * S->nn);
    S->conn.assign(d->connectivity, d->connectivity + (size_t)10 * S->ne);
    for (int32_t v : S->conn)
        if (v < 0 || v >= S->nn) throw std::invalid_argument("connectivity references an unknown node");
    S->left.assign(d->left_nodes, d->left_nodes + d->num_left);
    S->right.assign(d->right_nodes, d->right_nodes + d->num_right);
    for (int k = 0; k < d->num_pairs; k++) S->pairs.push_back({d->pairs[2 * k], d->pairs[2 * k + 1]});
    S->hub.assign(d->constrained_nodes, d->constrained_nodes + d->num_constrained);
    const int32_t nn = S->nn, ndof = 3 * nn;
    // DOF classes (src/cyclic_solver.cpp:214-238)
    std::vector<uint8_t> isl(nn, 0), isr(nn, 0);
    for (int32_t v : S->left) isl.at(v) = 1;
    for (int32_t v : S->right) isr.at(v) = 1;
    S->is_right.assign(ndof, 0);
    for (int32_t i = 0; i < nn; i++)
        for (int dd = 0; dd < 3; dd++) {
            const int32_t dof = 3 * i + dd;
            if (isr[i]) { S->right_dofs.push_back(dof); S->is_right[dof] = 1; }
            else if (isl[i]) S->left_dofs.push_back(dof);
            else S->interior_dofs.push_back(dof);
        }
    S->f2r.assign(ndof, -1);
    int32_t idx = 0;
    for (int32_t dof : S->interior_dofs) S->f2r[dof] = idx++;
    for (int32_t dof : S->left_dofs) S->f2r[dof] = idx++;
    S->n_reduced = idx;
    std::set<int32_t> cons;
    for (int32_t nid : S->hub) { cons.insert(3 * nid); cons.insert(3 * nid + 1); cons.insert(3 * nid + 2); }
    std::vector<int32_t> r2full;
    r2full.insert(r2full.end(), S->interior_dofs.begin(), S->interior_dofs.end());
    r2full.insert(r2full.end(), S->left_dofs.begin(), S->left_dofs.end());
    S->r2free.assign(S->n_reduced, -1);
    for (int32_t r = 0; r < S->n_reduced; r++)
        if (!cons.count(r2full[r])) { S->r2free[r] = (int32_t)S->free_reduced_map.size(); S->free_reduced_map.push_back(r); }
    S->n_free = (int32_t)S->free_reduced_map.size();
    // T(0): identity on interior + left, rotation on right rows (src/cyclic_solver.cpp:240-330)
    {
        const double alpha = 2.0 * PI / S->ns;
        const double ca = std::cos(alpha), sa = std::sin(alpha);
        int c1, c2, cax;
        if (S->axis == 0) { c1 = 1; c2 = 2; cax = 0; }
        else if (S->axis == 1) { c1 = 0; c2 = 2; cax = 1; }
        else { c1 = 0; c2 = 1; cax = 2; }
        std::vector<int32_t> r2l(nn, -1);
        for (auto& pr : S->pairs) r2l.at(pr.second) = pr.first;
        // (row, col, value) triplets, unique positions
        std::vector<std::vector<std::pair<int32_t, double>>> rows(ndof);
        for (int32_t dof : S->interior_dofs) rows[dof].push_back({S->f2r[dof], 1.0});
        for (int32_t dof : S->left_dofs) rows[dof].push_back({S->f2r[dof], 1.0});
        std::vector<uint8_t> done(nn, 0);
        for (int32_t rd : S->right_dofs) {
            const int32_t rn = rd / 3;
            if (done[rn]) continue;
            done[rn] = 1;
            const int32_t ln = r2l[rn];
            if (ln < 0) throw std::invalid_argument("Right boundary node " + std::to_string(rn) + " has no matched left partner");
            const int32_t l1 = S->f2r[3 * ln + c1], l2 = S->f2r[3 * ln + c2], lax = S->f2r[3 * ln + cax];
            if (l1 < 0 || l2 < 0 || lax < 0) throw std::invalid_argument("matched left node is on the right boundary");
            const int32_t rb = 3 * rn;
            rows[rb + c1].push_back({l1, ca}); rows[rb + c1].push_back({l2, -sa});
            rows[rb + c2].push_back({l1, sa}); rows[rb + c2].push_back({l2, ca});
            rows[rb + cax].push_back({lax, 1.0});
        }
        // CSC of T (full x reduced) and of its real filtered copy (|v| > 1e-15)
        auto build = [&](bool filt, Pattern& T, std::vector<double>& Tv) {
            T.nrows = ndof; T.ncols = S->n_reduced;
            T.p.assign(S->n_reduced + 1, 0);
            std::vector<std::vector<std::pair<int32_t, double>>> cols(S->n_reduced);
            for (int32_t r = 0; r < ndof; r++)
                for (auto& e : rows[r])
                    if (!filt || std::fabs(e.second) > 1e-15) cols[e.first].push_back({r, e.second});
            T.i.clear(); Tv.clear();
            for (int32_t cc = 0; cc < S->n_reduced; cc++) {
                std::sort(cols[cc].begin(), cols[cc].end());
                for (auto& e : cols[cc]) { T.i.push_back(e.first); Tv.push_back(e.second); }
                T.p[cc + 1] = (int64_t)T.i.size();
            }
        };
        build(false, S->T0, S->T0v);
        build(true, S->Tr, S->Trv);
        std::vector<int64_t> mp;
        S->T0t = transpose_map(S->T0, mp);
        S->T0tv.resize(mp.size());
        for (size_t q = 0; q < mp.size(); q++) S->T0tv[q] = S->T0v[mp[q]];
        S->Trt = transpose_map(S->Tr, mp);
        S->Trtv.resize(mp.size());
        for (size_t q = 0; q < mp.size(); q++) S->Trtv[q] = S->Trv[mp[q]];
    }
    // node adjacency -> candidate pattern
    {
        std::vector<std::vector<int32_t>> adj(nn);
        for (int32_t e = 0; e < S->ne; e++)
            for (int a = 0; a < 10; a++)
                for (int b = 0; b < 10; b++) adj[S->conn[(size_t)e * 10 + b]].push_back(S->conn[(size_t)e * 10 + a]);
        S->nadj_p.assign(nn + 1, 0);
        for (int32_t v = 0; v < nn; v++) {
            auto& L = adj[v];
            std::sort(L.begin(), L.end());
            L.erase(std::unique(L.begin(), L.end()), L.end());
            S->nadj_p[v + 1] = S->nadj_p[v] + (int64_t)L.size();
        }
        S->nadj_i.resize(S->nadj_p[nn]);
        for (int32_t v = 0; v < nn; v++) std::copy(adj[v].begin(), adj[v].end(), S->nadj_i.begin() + S->nadj_p[v]);
        S->npairs = S->nadj_p[nn];
        Pattern& C = S->cand;
        C.nrows = C.ncols = ndof;
        C.p.assign(ndof + 1, 0);
        C.i.resize(9 * S->npairs);
        std::vector<int64_t> candp(ndof + 1, 0);
        for (int32_t nb = 0; nb < nn; nb++) {
            const int64_t deg = S->nadj_p[nb + 1] - S->nadj_p[nb];
            for (int dd = 0; dd < 3; dd++) {
                const int64_t base = 9 * S->nadj_p[nb] + 3 * deg * dd;
                C.p[3 * nb + dd] = base;
                for (int64_t t = 0; t < deg; t++)
                    for (int cc = 0; cc < 3; cc++) C.i[base + 3 * t + cc] = 3 * S->nadj_i[S->nadj_p[nb] + t] + cc;
            }
        }
        C.p[ndof] = 9 * S->npairs;
        std::vector<int32_t> pcol(S->npairs), ppos(S->npairs);
        for (int32_t nb = 0; nb < nn; nb++)
            for (int64_t q = S->nadj_p[nb]; q < S->nadj_p[nb + 1]; q++) { pcol[q] = nb; ppos[q] = (int32_t)(q - S->nadj_p[nb]); }
        // contributions per node pair in element order
        std::vector<int64_t> cnt(S->npairs + 1, 0);
        auto pair_of = [&](int32_t na, int32_t nb) -> int64_t {
            const int32_t* b = S->nadj_i.data() + S->nadj_p[nb];
            const int32_t* e = S->nadj_i.data() + S->nadj_p[nb + 1];
            return S->nadj_p[nb] + (std::lower_bound(b, e, na) - b);
        };
        for (int32_t e = 0; e < S->ne; e++)
            for (int a = 0; a < 10; a++)
                for (int b = 0; b < 10; b++) cnt[pair_of(S->conn[(size_t)e * 10 + a], S->conn[(size_t)e * 10 + b]) + 1]++;
        for (int64_t q = 0; q < S->npairs; q++) cnt[q + 1] += cnt[q];
        std::vector<int32_t> cl(cnt[S->npairs]);
        std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
        for (int32_t e = 0; e < S->ne; e++)
            for (int a = 0; a < 10; a++)
                for (int b = 0; b < 10; b++)
                    cl[pos[pair_of(S->conn[(size_t)e * 10 + a], S->conn[(size_t)e * 10 + b])]++] = e * 100 + a * 10 + b;
        // node -> (element, local node) in element order, for load vectors
        std::vector<int64_t> np(nn + 1, 0);
        for (int32_t v : S->conn) np[v + 1]++;
        for (int32_t v = 0; v < nn; v++) np[v + 1] += np[v];
        std::vector<int32_t> nl(np[nn]);
        std::vector<int64_t> npos(np.begin(), np.end() - 1);
        for (int32_t e = 0; e < S->ne; e++)
            for (int a = 0; a < 10; a++) nl[npos[S->conn[(size_t)e * 10 + a]]++] = e * 10 + a;
        S->dX.upload(S->X);
        S->dconn.upload(S->conn);
        S->pair_col.upload(pcol);
        S->pair_pos.upload(ppos);
        S->clist.upload(cl);
        S->cptr.upload(cnt);
        S->dnadj_p.upload(S->nadj_p);
        std::vector<int64_t> cp(C.p.begin(), C.p.end());
        S->dcand_p.upload(cp);
        S->nptr.upload(np);
        S->nlist.upload(nl);
    }
    c->dT0_rp.upload(S->T0t.p);
    c->dT0_ci.upload(S->T0t.i);
    c->dT0_v.upload(S->T0tv);
    c->d_isr.upload(S->is_right);
    c->d_r2free.upload(S->r2free);
    c->sec = std::move(S);
    c->have_KM = false;
    c->static_ready = false;
    c->prepared = false;
    c->kw_omega = -1.0;
    c->symC.valid = false;
    c->symC_key.clear();
    c->stash.key.clear();
    c->real[0].valid = c->real[1].valid = false;
    c->results.clear();
}

void ensure_elem_buffers(Sector& S) {
    S.Kel.alloc((size_t)S.ne * 900);
    S.Mel.alloc((size_t)S.ne * 900);
}

void gather_into(tmg_context* c, const double* Kel, CandMat& out) {
    Sector& S = *c->sec;
    out.v.alloc(S.cand.nnz());
    out.f.alloc(S.cand.nnz());
    launch_gather_blocks(c->st, S.npairs, S.pair_col.p, S.pair_pos.p, S.dnadj_p.p, S.cptr.p, S.clist.p, S.dcand_p.p,
                         Kel, out.v.p, out.f.p);
}

void assemble_KM(tmg_context* c) {
    if (c->have_KM) return;
    Sector& S = *c->sec;
    ensure_elem_buffers(S);
    DVec<int> neg;
    neg.alloc(1);
    neg.zero(c->st);
    launch_elem_KM(c->st, S.ne, S.dX.p, S.dconn.p, S.E, S.nu, S.rho, S.Kel.p, S.Mel.p, neg.p);
    gather_into(c, S.Kel.p, c->K);
    gather_into(c, S.Mel.p, c->M);
    c->have_KM = true;
}

void assemble_rot(tmg_context* c, double omega) {
    if (c->kw_omega == omega) return;
    Sector& S = *c->sec;
    ensure_elem_buffers(S);
    launch_elem_rot(c->st, S.ne, S.dX.p, S.dconn.p, S.rho, omega, S.axis, S.Kel.p, S.Mel.p);
    gather_into(c, S.Kel.p, c->Kw);
    gather_into(c, S.Mel.p, c->G);
    c->kw_omega = omega;
}

// ---- factorisation + solve helpers ---------------------------------------------------
void analyze_op(OpSymbolic& os, const UnionMaps& um, const TuneCand* cand = nullptr,
                const std::vector<int32_t>* amd = nullptr) {
    os.S = analyze(um.lower, cand ? cand->relax : 0.0, cand ? cand->maxw : 0, amd);
    std::vector<int64_t> dest;
    std::vector<uint8_t> cj;
    scatter_map(os.S, um.lower, dest, cj);
    os.D.tc_min_rows = cand ? cand->tc_min : MF_TC_MIN_ROWS;
    os.D.upload(os.S, dest, cj);
    os.valid = true;
}

std::string pattern_key(const Pattern& P) {
    // cheap fingerprint of a pattern (size + rolling hash)
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { h ^= v; h *= 1099511628211ull; };
    mix((uint64_t)P.nrows); mix((uint64_t)P.nnz());
    for (int64_t v : P.p) mix((uint64_t)v);
    for (int32_t v : P.i) mix((uint64_t)v);
    return std::to_string(h);
}

// Static prestress operator: (Tr^T K Tr).pruned, hub DOFs removed (cyclic_solver.cpp:456-541)
void ensure_static(tmg_context* c) {
    if (c->static_ready) return;
    Sector& S = *c->sec;
    assemble_KM(c);
    Flagged fk = flagged(S.cand, c->K.f.download());
    build_chain(c->stat_chain, S.Trt, S.Trtv, fk, S.Tr, S.Trv);
    run_chain(c->st, c->stat_chain, c->K.v.p, 1e-15 * 1e-12);
    // free DOFs of the static solve: hub-constrained reduced DOFs removed
    extract_free(c->st, c->stat_chain, S.r2free, S.n_free, c->stat_free);
    build_union(c->stat_union, {&c->stat_free.pat});
    analyze_op(c->stat_sym, c->stat_union);
    // values -> fronts, factor (FP64 real)
    const DevSymbolic& D = c->stat_sym.D;
    c->stat_L.alloc(D.l_entries);
    c->stat_L.zero(c->st);
    DVec<double> ustore;
    ustore.alloc(D.u_entries);
    const Batch<double> bt{1, c->stat_L.p, ustore.p, D.l_entries, D.u_entries};
    c->stat_vals.alloc(c->stat_union.lower2csc.n);
    DVec<double> full;
    full.alloc(c->stat_union.U.nnz());
    if (full.n)
        TMG_LAUNCH(k_gather, nblk(full.n), 256, 0, c->st, (int64_t)full.n, c->stat_union.maps[0].p, c->stat_free.v.p, full.p);
    if (c->stat_vals.n)
        TMG_LAUNCH(k_gather_t<double>, nblk(c->stat_vals.n), 256, 0, c->st, (int64_t)c->stat_vals.n,
                   c->stat_union.lower2csc.p, full.p, c->stat_vals.p);
    mf_scatter<double>(c->st, D, bt, c->stat_vals.p);
    DVec<int> status;
    status.alloc(1);
    status.zero(c->st);
    mf_factor<double>(c->st, D, bt, status.p);
    int hs = 0;
    TMG_CUDA(cudaMemcpyAsync(&hs, status.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    TMG_CUDA(cudaStreamSynchronize(c->st));
    if (hs) throw numeric_error("static prestress factorisation hit a zero pivot");
    c->stat_t.alloc(std::max<int64_t>(1, D.t_entries));
    c->stat_x.alloc(S.n_free);
    std::vector<int32_t> fr(S.free_reduced_map.begin(), S.free_reduced_map.end());
    c->dstat_free_idx.upload(fr);
    c->static_ready = true;
}

// u(omega) = Tr u_cyc with K_cyc,free u_free = (Tr^T F)_free (cyclic_solver.cpp:461-557)
void static_solve(tmg_context* c, double omega) {
    Sector& S = *c->sec;
    ensure_static(c);
    const DevSymbolic& D = c->stat_sym.D;
    DVec<double> Fe, F, Fc, uc;
    Fe.alloc((size_t)S.ne * 30);
    F.alloc(3 * (size_t)S.nn);
    launch_elem_fc(c->st, S.ne, S.dX.p, S.dconn.p, S.rho, omega, S.axis, Fe.p);
    launch_gather_load(c->st, S.nn, S.nptr.p, S.nlist.p, Fe.p, F.p);
    DVec<int64_t> trp, trtp;
    DVec<int32_t> tri, trti;
    DVec<double> trv, trtv;
    trp.upload(S.Tr.p); tri.upload(S.Tr.i); trv.upload(S.Trv);       // CSC of Tr == CSR of Tr^T
    trtp.upload(S.Trt.p); trti.upload(S.Trt.i); trtv.upload(S.Trtv); // CSC of Tr^T == CSR of Tr
    Fc.alloc(S.n_reduced);
    TMG_LAUNCH(k_csr_real, nblk(S.n_reduced), 256, 0, c->st, S.n_reduced, trp.p, tri.p, trv.p, F.p, Fc.p);
    DVec<double> ff;
    ff.alloc(S.n_free);
    TMG_LAUNCH(k_gather_i32<double>, nblk(S.n_free), 256, 0, c->st, (int64_t)S.n_free, c->dstat_free_idx.p, Fc.p, ff.p);
    const Batch<double> bt{1, c->stat_L.p, nullptr, D.l_entries, 0};
    mf_permute_in<double, double>(c->st, D, 1, ff.p, S.n_free, c->stat_x.p, nullptr);
    mf_solve<double>(c->st, D, bt, c->stat_x.p, c->stat_t.p);
    mf_permute_out<double, double>(c->st, D, 1, c->stat_x.p, ff.p, S.n_free, nullptr);
    uc.alloc(S.n_reduced);
    uc.zero(c->st);
    TMG_LAUNCH(k_scatter_vec<double>, nblk(S.n_free), 256, 0, c->st, (int64_t)S.n_free, c->dstat_free_idx.p, ff.p, uc.p);
    c->u_static.alloc(3 * (size_t)S.nn);
    TMG_LAUNCH(k_csr_real, nblk(3 * (int64_t)S.nn), 256, 0, c->st, 3 * S.nn, trtp.p, trti.p, trtv.p, uc.p, c->u_static.p);
    TMG_CHECK_LAUNCH();
    TMG_CUDA(cudaStreamSynchronize(c->st));
}

}  // namespace

namespace {

// ---- cyclic projections ----------------------------------------------------------------
struct ChainCache {
    std::string key;
};

void project(tmg_context* c, const CandMat& A, ProjChain* ch, Flagged& fl, FreeMat& cf, FreeMat& pf, double tol) {
    Sector& S = *c->sec;
    Flagged f = flagged(S.cand, A.f.download());
    const bool same_pat = (f.pat.p == fl.pat.p) && (f.pat.i == fl.pat.i) && ch[0].n2 > 0;
    if (!same_pat) {
        fl = f;
        const std::vector<uint8_t>& isr = S.is_right;
        Flagged as = select(fl.pat, fl.cand, [&](int32_t r, int32_t cc) { return isr[r] == isr[cc]; });
        Flagged an = select(fl.pat, fl.cand, [&](int32_t r, int32_t cc) { return !isr[r] && isr[cc]; });
        build_chain(ch[0], S.T0t, S.T0tv, as, S.T0, S.T0v);
        build_chain(ch[1], S.T0t, S.T0tv, an, S.T0, S.T0v);
    }
    run_chain(c->st, ch[0], A.v.p, tol);
    run_chain(c->st, ch[1], A.v.p, tol);
    extract_free(c->st, ch[0], S.r2free, S.n_free, cf);
    extract_free(c->st, ch[1], S.r2free, S.n_free, pf);
    if (!same_pat || cf.spat.ncols != S.n_free) {
        struct_free(ch[0], S.r2free, S.n_free, cf);
        struct_free(ch[1], S.r2free, S.n_free, pf);
    }
    struct_values(c->st, ch[0], cf);
    struct_values(c->st, ch[1], pf);
}

bool same_pattern(const Pattern& a, const Pattern& b) { return a.p == b.p && a.i == b.i && a.nrows == b.nrows; }

void swap_op(OpSymbolic& a, OpSymbolic& b) {
    std::swap(a.S, b.S);
    a.D.swap(b.D);
    std::swap(a.valid, b.valid);
}

void prepare(tmg_context* c, double rpm, bool coriolis) {
    Sector& S = *c->sec;
    const double omega = rpm * 2.0 * PI / 60.0;
    auto t0 = std::chrono::steady_clock::now();
    assemble_KM(c);
    const int64_t nc = S.cand.nnz();
    c->Keff.v.alloc(nc);
    c->Keff.f.alloc(nc);
    if (std::fabs(omega) > 0.0) {
        assemble_rot(c, omega);
        if (!S.hub.empty()) {
            static_solve(c, omega);
            ensure_elem_buffers(S);
            DVec<int> bad;
            bad.alloc(1);
            bad.zero(c->st);
            launch_elem_ksig(c->st, S.ne, S.dX.p, S.dconn.p, S.E, S.nu, c->u_static.p, S.Kel.p, bad.p);
            gather_into(c, S.Kel.p, c->Ks);
            int hb = 0;
            TMG_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
            TMG_CUDA(cudaStreamSynchronize(c->st));
            if (hb) throw numeric_error("TET10::B_matrix: singular Jacobian (degenerate element)");
            launch_cand_axpy3(c->st, nc, 1.0, c->K.v.p, c->K.f.p, -1.0, c->Kw.v.p, c->Kw.f.p, 1.0, c->Ks.v.p,
                              c->Ks.f.p, c->Keff.v.p, c->Keff.f.p);
        } else {
            launch_cand_axpy3(c->st, nc, 1.0, c->K.v.p, c->K.f.p, -1.0, c->Kw.v.p, c->Kw.f.p, 0.0, nullptr, nullptr,
                              c->Keff.v.p, c->Keff.f.p);
        }
    } else {
        launch_cand_axpy3(c->st, nc, 1.0, c->K.v.p, c->K.f.p, 0.0, nullptr, nullptr, 0.0, nullptr, nullptr,
                          c->Keff.v.p, c->Keff.f.p);
    }
    project(c, c->Keff, c->chK, c->fK, c->Kcf, c->Kpf, 1e-27);
    project(c, c->M, c->chM, c->fM, c->Mcf, c->Mpf, 1e-27);
    c->coriolis = coriolis && std::fabs(omega) > 0.0;
    if (c->coriolis) project(c, c->G, c->chG, c->fG, c->Gcf, c->Gpf, 1e-27);
    // Operators are built on the structural patterns of the projections (entries the reference
    // prunes as roundoff are exact zeros there), which do not change with the speed: the
    // unions, maps and symbolic analyses below are rebuilt only when the sector operator's own
    // pattern changes (in practice once at rest and once at speed).
    c->KpfH = transpose_map(c->Kpf.spat, c->kpT);
    c->MpfH = transpose_map(c->Mpf.spat, c->mpT);
    const std::string key = pattern_key(c->Kcf.spat) + pattern_key(c->Kpf.spat) + pattern_key(c->Mcf.spat) +
                            pattern_key(c->Mpf.spat);
    if (key != c->symC_key && c->stash.key == key) {
        // back to the pattern of the other regime: exchange the current state with the kept one
        auto& o = c->stash;
        std::swap(c->opC, o.opC); std::swap(c->opMC, o.opMC); std::swap(c->W0, o.W0); std::swap(c->WM0, o.WM0);
        std::swap(c->pairOp, o.pairOp); std::swap(c->pairM, o.pairM);
        swap_op(c->symC, o.symC);
        swap_op(c->pairSym, o.pairSym);
        std::swap(c->tune_choice, o.tune_choice); std::swap(c->tuned_key, o.tuned_key);
        o.key = c->symC_key;
        c->symC_key = key;
        c->pair_key = key;
    } else if (key != c->symC_key) {
        if (c->symC.valid && c->pairSym.valid) {   // keep the current regime's state for a later return
            auto& o = c->stash;
            std::swap(c->opC, o.opC); std::swap(c->opMC, o.opMC); std::swap(c->W0, o.W0); std::swap(c->WM0, o.WM0);
            std::swap(c->pairOp, o.pairOp); std::swap(c->pairM, o.pairM);
            swap_op(c->symC, o.symC);
            swap_op(c->pairSym, o.pairSym);
            std::swap(c->tune_choice, o.tune_choice); std::swap(c->tuned_key, o.tuned_key);
            o.key = c->symC_key;
        }
        // complex harmonic operator: union of Kc, Kp, Kp^H, Mc, Mp, Mp^H
        build_union(c->opC, {&c->Kcf.spat, &c->Kpf.spat, &c->KpfH, &c->Mcf.spat, &c->Mpf.spat, &c->MpfH});
        build_union(c->opMC, {&c->Mcf.spat, &c->Mpf.spat, &c->MpfH});
        // transposed-constituent maps must address the un-transposed value arrays
        for (int which : {2, 5}) {
            const std::vector<int64_t>& tm = which == 2 ? c->kpT : c->mpT;
            std::vector<int64_t> m = c->opC.maps[which].download();
            for (auto& v : m) if (v >= 0) v = tm[v];
            c->opC.maps[which].upload(m);
        }
        {
            std::vector<int64_t> m = c->opMC.maps[2].download();
            for (auto& v : m) if (v >= 0) v = c->mpT[v];
            c->opMC.maps[2].upload(m);
        }
        c->symC.valid = false;
        c->symC_key = key;
        // real sums domain W = Kc u Kp u Kp^H (and the mass analogue)
        build_union(c->W0, {&c->Kcf.spat, &c->Kpf.spat, &c->KpfH});
        build_union(c->WM0, {&c->Mcf.spat, &c->Mpf.spat, &c->MpfH});
        for (UnionMaps* w : {&c->W0, &c->WM0}) {
            const std::vector<int64_t>& tm = (w == &c->W0) ? c->kpT : c->mpT;
            std::vector<int64_t> m = w->maps[2].download();
            for (auto& v : m) if (v >= 0) v = tm[v];
            w->maps[2].upload(m);
        }
        // real harmonics k = 0 and N/2: operator K on W, mass on W_M, both problems one batch
        build_union(c->pairOp, {&c->W0.U, &c->WM0.U});
        build_union(c->pairM, {&c->WM0.U});
        c->pairSym.valid = false;
        c->pair_key = key;
    }
    // real k = 0 / N/2 matrices: filtered sums (cyclic_solver.cpp:673-723); the filtered
    // patterns are what tmg_projection reports, the masked values on W / W_M feed the solver
    for (int h = 0; h < 2; h++) {
        if (h == 1 && !(S.ns % 2 == 0 && S.ns / 2 > 0)) { c->real[h].valid = false; continue; }
        const double sgn = h == 0 ? 1.0 : -1.0;
        auto& R = c->real[h];
        for (int which = 0; which < 2; which++) {
            UnionMaps& w = which == 0 ? c->W0 : c->WM0;
            const FreeMat& cc = which == 0 ? c->Kcf : c->Mcf;
            const FreeMat& pp = which == 0 ? c->Kpf : c->Mpf;
            DVec<double> vv;
            DVec<uint8_t> ff;
            vv.alloc(w.U.nnz());
            ff.alloc(w.U.nnz());
            if (w.U.nnz())
                TMG_LAUNCH(k_form_real_sum, nblk(w.U.nnz()), 256, 0, c->st, w.U.nnz(), w.maps[0].p, w.maps[1].p,
                           w.maps[2].p, cc.sv.p, pp.sv.p, sgn, vv.p, ff.p);
            DVec<double>& sv = which == 0 ? R.Ks : R.Ms;
            sv.alloc(w.U.nnz());
            if (w.U.nnz()) TMG_LAUNCH(k_mask_values, nblk(w.U.nnz()), 256, 0, c->st, w.U.nnz(), vv.p, ff.p, sv.p);
            Flagged fl = flagged(w.U, ff.download());
            FreeMat& dst = which == 0 ? R.Kr : R.Mr;
            dst.pat = fl.pat;
            dst.idx.upload(fl.cand);
            dst.v.alloc(fl.cand.size());
            if (!fl.cand.empty())
                TMG_LAUNCH(k_gather, nblk(fl.cand.size()), 256, 0, c->st, (int64_t)fl.cand.size(), dst.idx.p, vv.p,
                           dst.v.p);
            TMG_CUDA(cudaStreamSynchronize(c->st));
        }
        R.valid = true;
    }
    TMG_CUDA(cudaStreamSynchronize(c->st));
    c->prepared = true;
    c->rpm = rpm;
    c->phase_ms[0] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Gyroscopic sum domain and Lancaster block maps of the prepared speed (built when the
// structural patterns of K, M or G change; the symbolic analysis follows lazily).
void ensure_qep(tmg_context* c) {
    const std::string key = c->symC_key + pattern_key(c->Gcf.spat) + pattern_key(c->Gpf.spat);
    if (key == c->qep.key) return;
    c->GpfH = transpose_map(c->Gpf.spat, c->gpT);
    build_union(c->WG0, {&c->Gcf.spat, &c->Gpf.spat, &c->GpfH});
    {
        std::vector<int64_t> m = c->WG0.maps[2].download();
        for (auto& v : m) if (v >= 0) v = c->gpT[v];
        c->WG0.maps[2].upload(m);
    }
    auto& Q = c->qep;
    const LancasterBlocks A = lancaster_blocks(c->W0.U, c->WM0.U, c->WG0.U, 0);
    const LancasterBlocks L2 = lancaster_blocks(c->W0.U, c->WM0.U, c->WG0.U, 1);
    build_union(Q.op, {&A.P});
    build_union(Q.l2, {&L2.P});
    Q.sk.upload(A.srcK); Q.sm.upload(A.srcM); Q.sg.upload(A.srcG); Q.blk.upload(A.blk);
    Q.sk2.upload(L2.srcK); Q.sm2.upload(L2.srcM); Q.sg2.upload(L2.srcG); Q.blk2.upload(L2.blk);
    Q.sym.valid = false;
    Q.key = key;
}

}  // namespace

namespace {

// ---- batched kernels of the harmonic solves ---------------------------------------------
// (Kc + P Kp) + conj(P) Kp^H per problem (phase p from ph[2p], ph[2p+1])
__global__ void k_form_csum(int64_t n, const int64_t* __restrict__ ic, const int64_t* __restrict__ ip,
                            const int64_t* __restrict__ ih, const double* __restrict__ c, const double* __restrict__ pv,
                            const double* __restrict__ ph, zd* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (e >= n) return;
    const double a = ic[e] >= 0 ? c[ic[e]] : 0.0;
    const double b = ip[e] >= 0 ? pv[ip[e]] : 0.0;
    const double h = ih[e] >= 0 ? pv[ih[e]] : 0.0;
    const zd P{ph[2 * p], ph[2 * p + 1]}, Pc{ph[2 * p], -ph[2 * p + 1]};
    out[p * n + e] = (zd{a, 0.0} + P * zd{b, 0.0}) + Pc * zd{h, 0.0};
}

// Complex harmonic operator on the union pattern, per problem:
//   ((kc + P kp) + conj(P) kph) - sigma ((mc + P mp) + conj(P) mph)
// with missing constituents read as exact zeros (the reference's sparse-sum semantics,
// src/cyclic_solver.cpp:946-947, src/hermitian_lanczos.cpp:15).
__global__ void k_form_complex(int64_t n, const int64_t* __restrict__ ikc, const int64_t* __restrict__ ikp,
                               const int64_t* __restrict__ ikh, const int64_t* __restrict__ imc,
                               const int64_t* __restrict__ imp, const int64_t* __restrict__ imh,
                               const double* __restrict__ kc, const double* __restrict__ kp,
                               const double* __restrict__ mc, const double* __restrict__ mp,
                               const double* __restrict__ ph, double sigma, zd* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (e >= n) return;
    const double a = ikc[e] >= 0 ? kc[ikc[e]] : 0.0;
    const double b = ikp[e] >= 0 ? kp[ikp[e]] : 0.0;
    const double c = ikh[e] >= 0 ? kp[ikh[e]] : 0.0;
    const double am = imc[e] >= 0 ? mc[imc[e]] : 0.0;
    const double bm = imp[e] >= 0 ? mp[imp[e]] : 0.0;
    const double cm = imh[e] >= 0 ? mp[imh[e]] : 0.0;
    const zd P{ph[2 * p], ph[2 * p + 1]}, Pc{ph[2 * p], -ph[2 * p + 1]};
    const zd kk = (zd{a, 0.0} + P * zd{b, 0.0}) + Pc * zd{c, 0.0};
    const zd mm = (zd{am, 0.0} + P * zd{bm, 0.0}) + Pc * zd{cm, 0.0};
    out[p * n + e] = kk - sigma * mm;
}

// Lancaster matrices of the Coriolis QEP per problem (src/modal_solver.cpp:151-198 and the
// shifted operator of src/hermitian_lanczos.cpp:15): L1 = [[D, K], [K, 0]] with
// D = (i 2 omega) G, L2 = [[M, 0], [0, K]].  mode 0: L1 - sigma_p L2, 1: L1, 2: L2.  K, M, G
// hold each problem's harmonic values on their domains (nK, nM, nG entries per problem);
// an absent block entry reads as an exact zero.
__global__ void k_form_lancaster(int64_t ne, const int64_t* __restrict__ sk, const int64_t* __restrict__ sm,
                                 const int64_t* __restrict__ sg, const int8_t* __restrict__ blk,
                                 const zd* __restrict__ K, int64_t nK, const zd* __restrict__ M, int64_t nM,
                                 const zd* __restrict__ G, int64_t nG, double two_omega,
                                 const double* __restrict__ sigma, int mode, zd* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (e >= ne) return;
    const int b = blk[e];
    const zd z{0.0, 0.0};
    const zd kv = sk[e] >= 0 ? K[p * nK + sk[e]] : z;
    zd l1 = z, l2 = z;
    if (b == 0) {
        if (sg[e] >= 0) l1 = zd{0.0, two_omega} * G[p * nG + sg[e]];
        if (sm[e] >= 0) l2 = M[p * nM + sm[e]];
    } else if (b == 3) {
        l2 = kv;
    } else {
        l1 = kv;
    }
    out[p * ne + e] = mode == 1 ? l1 : (mode == 2 ? l2 : l1 - sigma[p] * l2);
}

// free-space degenerate duplication: column m <- src m/2, conjugated when m is odd
__global__ void k_dup_conj(int64_t n, int nx, const zd* __restrict__ X, zd* __restrict__ Y) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (i >= n || m >= nx) return;
    const zd v = X[(int64_t)(m / 2) * n + i];
    Y[(int64_t)m * n + i] = (m % 2 == 0) ? v : conj(v);
}

template <typename T>
__global__ void k_resid(int64_t n, int nm, const T* __restrict__ AX, const T* __restrict__ MX, const double* __restrict__ lam,
                        double sigma, T* __restrict__ KX, T* __restrict__ R) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int m = blockIdx.y;
    if (i >= n || m >= nm) return;
    const int64_t q = (int64_t)m * n + i;
    const T kx = AX[q] + sigma * MX[q];      // K x = (K - sigma M) x + sigma M x
    KX[q] = kx;
    R[q] = kx - lam[m] * MX[q];
}

template <typename T>
__global__ void k_gather_b(int64_t n, const int64_t* __restrict__ idx, const T* __restrict__ src, int64_t ss,
                           T* __restrict__ dst, int64_t ds) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (e < n) dst[p * ds + e] = src[p * ss + idx[e]];
}

// s_i = 1/sqrt(|Re a_ii|) per problem from a CSR matrix (1 when the diagonal is absent or zero)
template <typename T>
__global__ void k_diag_scale(int32_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                             const T* __restrict__ v, int64_t vs, double* __restrict__ s) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n) return;
    double d = 0.0;
    for (int64_t q = rp[i]; q < rp[i + 1]; q++)
        if (ci[q] == i) d = fabs(re(v[p * vs + q]));
    s[p * n + i] = d > 0.0 ? 1.0 / sqrt(d) : 1.0;
}

template <typename T, typename U>
__global__ void k_scale_lower(int64_t nl, int32_t n, const int32_t* __restrict__ row, const int32_t* __restrict__ col,
                              const double* __restrict__ s, const U* __restrict__ v, T* __restrict__ out) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (q < nl) out[p * nl + q] = conv<T, U>((s[p * n + row[q]] * s[p * n + col[q]]) * v[p * nl + q]);
}

template <typename T>
__global__ void k_pcg_xr(int64_t n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ pp,
                         const T* __restrict__ q, const T* __restrict__ rz, const T* __restrict__ pq,
                         const int* __restrict__ done) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n || done[p]) return;
    const double a = re(rz[p]) / re(pq[p]);
    x[p * n + i] += a * pp[p * n + i];
    r[p * n + i] -= a * q[p * n + i];
}

template <typename T>
__global__ void k_pcg_p(int64_t n, T* __restrict__ pp, const T* __restrict__ z, const T* __restrict__ rznew,
                        const T* __restrict__ rz, const int* __restrict__ done) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n || done[p]) return;
    const double b = re(rznew[p]) / re(rz[p]);
    pp[p * n + i] = z[p * n + i] + b * pp[p * n + i];
}

template <typename T>
__global__ void k_ir_update(int64_t n, T* __restrict__ x, const T* __restrict__ d, const int* __restrict__ done) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n || done[p]) return;
    x[p * n + i] += d[p * n + i];
}

// y[p] = sgn * Einv[p] h[p] for the m x m (column-major) matrix of every problem (deflation)
// dst[p] = inv[p] * src[p] (per-problem scalar)
template <typename T>
__global__ void k_scale_into(int64_t n, const double* __restrict__ inv, const T* __restrict__ src, int64_t ss,
                             T* __restrict__ dst, int64_t ds) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t p = blockIdx.y;
    if (i >= n) return;
    dst[p * ds + i] = inv[p] * src[p * ss + i];
}

template <typename T>
__global__ void k_small_mv(int m, const T* __restrict__ Einv, const T* __restrict__ h, T* __restrict__ y, double sgn) {
    const int64_t p = blockIdx.x;
    const int i = threadIdx.x;
    if (i >= m) return;
    T acc = zero_of<T>();
    for (int j = 0; j < m; j++) acc += Einv[p * m * m + (int64_t)j * m + i] * h[p * m + j];
    y[p * m + i] = sgn * acc;
}

inline std::complex<double> to_std(double v) { return {v, 0.0}; }
inline std::complex<double> to_std(zd v) { return {v.x, v.y}; }
template <typename T> T from_std(std::complex<double> v);
template <> inline double from_std<double>(std::complex<double> v) { return v.real(); }
template <> inline zd from_std<zd>(std::complex<double> v) { return zd{v.real(), v.imag()}; }

// eigenvectors kept per complex harmonic to deflate the refinement at the next speed
constexpr int DEFL_M = 8;

// ---- shift-invert operator of a batch ----------------------------------------------------
template <typename Tv, typename Tf>
struct ShiftInvertB {
    tmg_context* c = nullptr;
    const DevSymbolic* D = nullptr;
    const UnionMaps* um = nullptr;
    int32_t n = 0;
    int B = 1;
    bool mixed = false;
    bool spd = false;             // every pivot positive: CG-accelerated refinement
    int max_iter = 30;            // refinement iterations per solve (mixed)
    double rtol = 1e-10;          // relative residual target of a refined solve (mixed)
    DevCsr<Tv> A;                 // FP64 operator K - sigma M (CSR, per-problem values)
    DVec<Tf> L, U, tb, xw;
    DVec<Tv> gin, gout, r, d, z, pp, q, sc, bin;
    DVec<double> scale, np, nrm;
    DVec<int> ddone;
    std::vector<double> worst;    // worst relative residual of a refined solve, per problem
    std::vector<int> skip;        // problems finished or failed: refinement leaves them alone
    std::vector<std::string> failed;   // per problem: why its factorisation failed ("" = fine)
    int64_t solves = 0, applies = 0, max_its = 0;
    // Deflation of the refinement CG (off unless set_deflation is called): W holds mdef vectors
    // per problem (n x mdef, problem stride n * mdef), AW = A W, Einv = (W^H A W)^-1 per problem
    // (mdef x mdef, column-major).
    int mdef = 0;
    DVec<Tv> W, AW, Einv, hdef, ydef, pdef;
    // restarted GMRES of the indefinite case: GM Krylov vectors per cycle, V ((GM+1) x n per
    // problem), preconditioned directions Z (GM x n per problem)
    static constexpr int GM = 32;
    int gmres_cycles = 4;
    DVec<Tv> GV, GZ, gh, gpart, gy;
    DVec<double> ginv;
    cudaGraphExec_t gexec = nullptr;
    int64_t launches_per_solve = 0;
    ~ShiftInvertB() { if (gexec) cudaGraphExecDestroy(gexec); }

    void factor(const Tv* lower_vals) {
        const int64_t nl = D->nlower;
        L.alloc((size_t)B * D->l_entries);
        U.alloc((size_t)B * std::max<int64_t>(D->u_entries, 1));
        L.zero(g_stream);
        const Batch<Tf> bt{B, L.p, U.p, D->l_entries, D->u_entries};
        if constexpr (std::is_same<Tv, Tf>::value) {
            mf_scatter<Tf>(g_stream, *D, bt, lower_vals);
        } else {
            scale.alloc((size_t)B * n);
            TMG_LAUNCH(k_diag_scale<Tv>, dim3(nblk(n), B), 256, 0, g_stream, n, A.rowptr, A.col, A.val, A.vstride, scale.p);
            DVec<Tf> lv;
            lv.alloc((size_t)B * nl);
            TMG_LAUNCH((k_scale_lower<Tf, Tv>), dim3(nblk(nl), B), 256, 0, g_stream, nl, n, um->low_row.p, um->low_col.p,
                       scale.p, lower_vals, lv.p);
            mf_scatter<Tf>(g_stream, *D, bt, lv.p);
            TMG_CUDA(cudaStreamSynchronize(g_stream));
        }
        DVec<int> status;
        status.alloc(2 * B);
        status.zero(g_stream);
        mf_factor<Tf>(g_stream, *D, bt, status.p, c->tensor_cores);
        mf_count_nonpos<Tf>(g_stream, *D, bt, status.p + B);
        std::vector<int> hs(2 * B);
        TMG_CUDA(cudaMemcpyAsync(hs.data(), status.p, 2 * B * sizeof(int), cudaMemcpyDeviceToHost, g_stream));
        TMG_CUDA(cudaStreamSynchronize(g_stream));
        spd = true;
        skip.assign(B, 0);
        failed.assign(B, std::string());
        int nfail = 0;
        for (int p = 0; p < B; p++) {
            if (hs[p]) {   // this problem fails alone; the rest of the batch goes on
                failed[p] = "zero pivot in LDL^H factorisation at column " + std::to_string(hs[p] - 1);
                skip[p] = 1;
                nfail++;
                continue;
            }
            if (hs[B + p]) spd = false;
        }
        if (nfail == B) throw numeric_error(failed[0]);
        U.release();                  // the update workspace is only needed while factorising
        tb.alloc((size_t)B * std::max<int64_t>(1, D->t_entries));
        xw.alloc((size_t)B * n);
        for (DVec<Tv>* v : {&gin, &gout, &r, &d, &z, &pp, &q}) v->alloc((size_t)B * n);
        sc.alloc(4 * B);
        np.alloc((size_t)B * LZ_DOT_BLOCKS);
        nrm.alloc(B);
        ddone.alloc(B);
        ddone.zero(g_stream);
        worst.assign(B, 0.0);
    }
    Batch<Tf> batch() const { return Batch<Tf>{B, L.p, nullptr, D->l_entries, 0}; }

    // Deflate the CG of every later mixed apply with m vectors per problem (Wsrc: B x n x m,
    // problem stride n * m), which should approximate the operator's lowest eigenvectors (the
    // eigenvectors of the previous speed of a sweep).  Only for the CG path (every pivot positive).
    void set_deflation(const Tv* Wsrc, int m) {
        mdef = 0;
        if (!mixed || !spd || m <= 0 || m > 32) return;
        const int64_t nm = (int64_t)n * m;
        W.alloc((size_t)B * nm);
        AW.alloc((size_t)B * nm);
        TMG_CUDA(cudaMemcpyAsync(W.p, Wsrc, (size_t)B * nm * sizeof(Tv), cudaMemcpyDeviceToDevice, g_stream));
        lz_spmv<Tv>(g_stream, B, A, W.p, nm, AW.p, nm, m, n);
        pdef.alloc((size_t)B * m * LZ_DOT_BLOCKS);
        hdef.alloc((size_t)B * m);
        ydef.alloc((size_t)B * m);
        // E = W^H A W column by column, inverted on the host (Gauss-Jordan, partial pivoting)
        std::vector<std::complex<double>> E((size_t)B * m * m);
        std::vector<Tv> col((size_t)B * m);
        for (int v = 0; v < m; v++) {
            lz_multidot<Tv>(g_stream, B, n, W.p, nm, n, m, AW.p + (int64_t)v * n, nm, pdef.p, hdef.p);
            TMG_CUDA(cudaMemcpyAsync(col.data(), hdef.p, col.size() * sizeof(Tv), cudaMemcpyDeviceToHost, g_stream));
            TMG_CUDA(cudaStreamSynchronize(g_stream));
            for (int p = 0; p < B; p++)
                for (int k = 0; k < m; k++) E[((size_t)p * m + v) * m + k] = to_std(col[(size_t)p * m + k]);
        }
        std::vector<Tv> inv((size_t)B * m * m);
        for (int p = 0; p < B; p++) {
            std::vector<std::complex<double>> a(E.begin() + (size_t)p * m * m, E.begin() + (size_t)(p + 1) * m * m);
            std::vector<std::complex<double>> x((size_t)m * m, 0.0);
            for (int i = 0; i < m; i++) x[(size_t)i * m + i] = 1.0;
            for (int c0 = 0; c0 < m; c0++) {
                int piv = c0;
                for (int r = c0 + 1; r < m; r++)
                    if (std::abs(a[(size_t)c0 * m + r]) > std::abs(a[(size_t)c0 * m + piv])) piv = r;
                if (std::abs(a[(size_t)c0 * m + piv]) == 0.0) return;   // singular: no deflation
                for (int j = 0; j < m; j++) {
                    std::swap(a[(size_t)j * m + c0], a[(size_t)j * m + piv]);
                    std::swap(x[(size_t)j * m + c0], x[(size_t)j * m + piv]);
                }
                const std::complex<double> d = a[(size_t)c0 * m + c0];
                for (int j = 0; j < m; j++) { a[(size_t)j * m + c0] /= d; x[(size_t)j * m + c0] /= d; }
                for (int r = 0; r < m; r++) {
                    if (r == c0) continue;
                    const std::complex<double> f = a[(size_t)c0 * m + r];
                    if (f == 0.0) continue;
                    for (int j = 0; j < m; j++) {
                        a[(size_t)j * m + r] -= f * a[(size_t)j * m + c0];
                        x[(size_t)j * m + r] -= f * x[(size_t)j * m + c0];
                    }
                }
            }
            for (size_t q = 0; q < (size_t)m * m; q++) inv[(size_t)p * m * m + q] = from_std<Tv>(x[q]);
        }
        Einv.upload(inv);
        mdef = m;
    }
    // z -= W Einv (AW^H z) for every problem
    void deflate(Tv* z) {
        const int64_t nm = (int64_t)n * mdef;
        lz_multidot<Tv>(g_stream, B, n, AW.p, nm, n, mdef, z, n, pdef.p, hdef.p);
        TMG_LAUNCH(k_small_mv<Tv>, B, 32, 0, g_stream, mdef, Einv.p, hdef.p, ydef.p, 1.0);
        lz_gemv_sub<Tv>(g_stream, B, n, mdef, W.p, nm, ydef.p, mdef, z, n);
    }

    // the permute / supernodal sweeps / permute sequence of one batched solve is captured
    // once into a CUDA graph over fixed buffers and replayed for every solve
    void solve1(const Tv* b, Tv* x) {
        const double* s = mixed ? scale.p : nullptr;
        if (!gexec) {
            const int64_t l0 = g_kernel_launches;
            cudaGraph_t g;
            TMG_CUDA(cudaStreamBeginCapture(g_stream, cudaStreamCaptureModeThreadLocal));
            mf_permute_in<Tf, Tv>(g_stream, *D, B, gin.p, n, xw.p, s);
            mf_solve<Tf>(g_stream, *D, batch(), xw.p, tb.p, ddone.p);
            mf_permute_out<Tf, Tv>(g_stream, *D, B, xw.p, gout.p, n, s);
            TMG_CUDA(cudaStreamEndCapture(g_stream, &g));
            TMG_CUDA(cudaGraphInstantiate(&gexec, g, 0));
            TMG_CUDA(cudaGraphDestroy(g));
            launches_per_solve = g_kernel_launches - l0;
            g_kernel_launches = l0;
        }
        TMG_CUDA(cudaMemcpyAsync(gin.p, b, (size_t)B * n * sizeof(Tv), cudaMemcpyDeviceToDevice, g_stream));
        if (c->profile) {
            if (!c->pev0) { TMG_CUDA(cudaEventCreate(&c->pev0)); TMG_CUDA(cudaEventCreate(&c->pev1)); }
            TMG_CUDA(cudaEventRecord(c->pev0, g_stream));
        }
        TMG_CUDA(cudaGraphLaunch(gexec, g_stream));
        if (c->profile) {
            TMG_CUDA(cudaEventRecord(c->pev1, g_stream));
            TMG_CUDA(cudaEventSynchronize(c->pev1));
            float ms = 0.f;
            TMG_CUDA(cudaEventElapsedTime(&ms, c->pev0, c->pev1));
            c->solve_ms += ms;
            c->solve_count++;
            // algorithmic bytes: every stored L entry read once per sweep direction, plus the
            // solution vector read and written once per direction, for each problem
            c->solve_bytes += (double)B * (2.0 * (double)D->l_stored * sizeof(Tf) + 4.0 * (double)n * sizeof(Tf));
        }
        g_kernel_launches += launches_per_solve;
        TMG_CUDA(cudaMemcpyAsync(x, gout.p, (size_t)B * n * sizeof(Tv), cudaMemcpyDeviceToDevice, g_stream));
        solves++;
    }
    std::vector<double> norms(const Tv* v) {
        std::vector<double> h(B);
        lz_norm2<Tv>(g_stream, B, n, v, n, np.p, nrm.p);
        TMG_CUDA(cudaMemcpyAsync(h.data(), nrm.p, B * sizeof(double), cudaMemcpyDeviceToHost, g_stream));
        TMG_CUDA(cudaStreamSynchronize(g_stream));
        return h;
    }
    // Restarted GMRES on A x = b, right-preconditioned by the FP32 factor (z = F^-1 v), FP64
    // Arnoldi with two classical Gram-Schmidt passes and complex Givens rotations on the host, per
    // problem.  Used when some pivot is negative (indefinite or strongly shifted operators), where
    // plain refinement x += F^-1 (b - A x) stalls as soon as the factor's error is not a
    // contraction; GMRES converges whenever the preconditioned operator's spectrum clusters with a
    // few outliers.  Each cycle ends with the true FP64 residual.  Returns the inner iterations.
    int gmres(const Tv* b, Tv* x, const std::vector<double>& bn, std::vector<int>& done, std::vector<double>& rn) {
        using cplx = std::complex<double>;
        cudaStream_t st = g_stream;
        const int64_t vs = (int64_t)(GM + 1) * n, zs = (int64_t)GM * n;
        if (!GV.p) {
            GV.alloc((size_t)B * vs);
            GZ.alloc((size_t)B * zs);
            gh.alloc((size_t)B * (GM + 1));
            gpart.alloc((size_t)B * (GM + 1) * LZ_DOT_BLOCKS);
            gy.alloc((size_t)B * GM);
            ginv.alloc(B);
        }
        TMG_CUDA(cudaMemsetAsync(x, 0, (size_t)B * n * sizeof(Tv), st));
        lz_copy<Tv>(st, (int64_t)B * n, b, r.p);
        std::vector<cplx> H((size_t)B * (GM + 1) * GM), cs((size_t)B * GM), sn((size_t)B * GM), g((size_t)B * (GM + 1));
        std::vector<double> inv(B), est(B);
        std::vector<Tv> hv((size_t)B * (GM + 1)), yv((size_t)B * GM);
        auto Hat = [&](int p, int i, int j) -> cplx& { return H[((size_t)p * GM + j) * (GM + 1) + i]; };
        auto scale_into = [&](const Tv* src, int64_t ss, Tv* dst, int64_t ds) {
            TMG_CUDA(cudaMemcpyAsync(ginv.p, inv.data(), B * sizeof(double), cudaMemcpyHostToDevice, st));
            TMG_LAUNCH(k_scale_into<Tv>, dim3(nblk(n), B), 256, 0, st, (int64_t)n, ginv.p, src, ss, dst, ds);
            TMG_CUDA(cudaStreamSynchronize(st));   // inv is a host vector reused by the next call
        };
        int total = 0;
        for (int cycle = 0; cycle < gmres_cycles; cycle++) {
            rn = norms(r.p);
            bool all = true;
            for (int p = 0; p < B; p++) {
                if (!done[p] && rn[p] <= rtol * rtol * bn[p]) done[p] = 1;
                all = all && done[p];
            }
            TMG_CUDA(cudaMemcpyAsync(ddone.p, done.data(), B * sizeof(int), cudaMemcpyHostToDevice, st));
            if (all) break;
            std::fill(H.begin(), H.end(), cplx(0.0));
            std::fill(g.begin(), g.end(), cplx(0.0));
            for (int p = 0; p < B; p++) {
                const double beta = std::sqrt(rn[p]);
                inv[p] = (!done[p] && beta > 0.0) ? 1.0 / beta : 0.0;
                g[(size_t)p * (GM + 1)] = beta;
            }
            scale_into(r.p, n, GV.p, vs);                      // v_0 = r / ||r||
            int jj = 0;
            for (int j = 0; j < GM; j++) {
                // z_j = F^-1 v_j, w = A z_j (w in z)
                TMG_CUDA(cudaMemcpy2DAsync(d.p, n * sizeof(Tv), GV.p + (int64_t)j * n, vs * sizeof(Tv), n * sizeof(Tv), B,
                                           cudaMemcpyDeviceToDevice, st));
                solve1(d.p, q.p);
                TMG_CUDA(cudaMemcpy2DAsync(GZ.p + (int64_t)j * n, zs * sizeof(Tv), q.p, n * sizeof(Tv), n * sizeof(Tv), B,
                                           cudaMemcpyDeviceToDevice, st));
                lz_spmv<Tv>(st, B, A, q.p, n, z.p, n, 1, n);
                for (int pass = 0; pass < 2; pass++) {
                    lz_multidot<Tv>(st, B, n, GV.p, vs, n, j + 1, z.p, n, gpart.p, gh.p);
                    lz_gemv_sub<Tv>(st, B, n, j + 1, GV.p, vs, gh.p, j + 1, z.p, n);
                    TMG_CUDA(cudaMemcpyAsync(hv.data(), gh.p, (size_t)B * (j + 1) * sizeof(Tv), cudaMemcpyDeviceToHost, st));
                    TMG_CUDA(cudaStreamSynchronize(st));
                    for (int p = 0; p < B; p++)
                        for (int k = 0; k <= j; k++) Hat(p, k, j) += to_std(hv[(size_t)p * (j + 1) + k]);
                }
                const std::vector<double> hn = norms(z.p);
                for (int p = 0; p < B; p++) {
                    const double h = std::sqrt(hn[p]);
                    Hat(p, j + 1, j) = h;
                    inv[p] = (!done[p] && h > 0.0) ? 1.0 / h : 0.0;
                }
                scale_into(z.p, n, GV.p + (int64_t)(j + 1) * n, vs);   // v_{j+1}
                bool conv = true;
                for (int p = 0; p < B; p++) {
                    if (done[p]) continue;
                    cplx* gp = g.data() + (size_t)p * (GM + 1);
                    for (int i = 0; i < j; i++) {   // earlier rotations on the new column
                        const cplx ci = cs[(size_t)p * GM + i], si = sn[(size_t)p * GM + i];
                        const cplx t = ci * Hat(p, i, j) + si * Hat(p, i + 1, j);
                        Hat(p, i + 1, j) = -std::conj(si) * Hat(p, i, j) + ci * Hat(p, i + 1, j);
                        Hat(p, i, j) = t;
                    }
                    const cplx a = Hat(p, j, j), bb = Hat(p, j + 1, j);
                    const double rho = std::hypot(std::abs(a), std::abs(bb));
                    cplx ci, si;
                    if (rho == 0.0) { ci = 1.0; si = 0.0; }
                    else if (std::abs(a) == 0.0) { ci = 0.0; si = std::conj(bb) / std::abs(bb); }
                    else { ci = std::abs(a) / rho; si = (a / std::abs(a)) * std::conj(bb) / rho; }
                    cs[(size_t)p * GM + j] = ci;
                    sn[(size_t)p * GM + j] = si;
                    Hat(p, j, j) = ci * a + si * bb;
                    Hat(p, j + 1, j) = 0.0;
                    gp[j + 1] = -std::conj(si) * gp[j];
                    gp[j] = ci * gp[j];
                    est[p] = std::abs(gp[j + 1]);
                    if (est[p] > 0.5 * rtol * std::sqrt(bn[p])) conv = false;
                }
                jj = j + 1;
                total++;
                if (conv) break;
            }
            // x += Z y with H y = g (back substitution per problem; converged problems add nothing)
            std::fill(yv.begin(), yv.end(), from_std<Tv>(cplx(0.0)));
            for (int p = 0; p < B; p++) {
                if (done[p]) continue;
                std::vector<cplx> y(jj);
                const cplx* gp = g.data() + (size_t)p * (GM + 1);
                for (int i = jj - 1; i >= 0; i--) {
                    cplx acc = gp[i];
                    for (int k = i + 1; k < jj; k++) acc -= Hat(p, i, k) * y[k];
                    const cplx dgl = Hat(p, i, i);
                    y[i] = std::abs(dgl) > 0.0 ? acc / dgl : cplx(0.0);
                }
                for (int i = 0; i < jj; i++) yv[(size_t)p * jj + i] = from_std<Tv>(-y[i]);
            }
            TMG_CUDA(cudaMemcpyAsync(gy.p, yv.data(), (size_t)B * jj * sizeof(Tv), cudaMemcpyHostToDevice, st));
            lz_gemv_sub<Tv>(st, B, n, jj, GZ.p, zs, gy.p, jj, x, n);
            TMG_CUDA(cudaStreamSynchronize(st));
            lz_copy<Tv>(st, (int64_t)B * n, b, r.p);
            lz_spmv<Tv>(st, B, A, x, n, r.p, n, 1, n, true);
        }
        rn = norms(r.p);
        for (int p = 0; p < B; p++)
            if (!done[p] && rn[p] <= rtol * rtol * bn[p]) done[p] = 1;
        return total;
    }

    // x = (K - sigma M)^-1 b for every problem of the batch; problem p's right-hand side
    // starts at b + p * bs, its solution at x + p * n
    void apply(const Tv* b, int64_t bs, Tv* x) {
        applies++;
        if (bs != n) {
            if (!bin.p) bin.alloc((size_t)B * n);
            TMG_CUDA(cudaMemcpy2DAsync(bin.p, n * sizeof(Tv), b, bs * sizeof(Tv), n * sizeof(Tv), B,
                                       cudaMemcpyDeviceToDevice, g_stream));
            b = bin.p;
        }
        if (!mixed) {   // finished problems are skipped by the solve kernels
            TMG_CUDA(cudaMemcpyAsync(ddone.p, skip.data(), B * sizeof(int), cudaMemcpyHostToDevice, g_stream));
            solve1(b, x);
            return;
        }
        const std::vector<double> bn = norms(b);
        std::vector<int> done(skip);
        std::vector<double> rn;
        TMG_CUDA(cudaMemcpyAsync(ddone.p, done.data(), B * sizeof(int), cudaMemcpyHostToDevice, g_stream));
        int it = 0;
        auto check = [&]() {
            rn = norms(r.p);
            bool all = true, changed = false;
            for (int p = 0; p < B; p++) {
                if (!done[p] && rn[p] <= rtol * rtol * bn[p]) { done[p] = 1; changed = true; }
                all = all && done[p];
            }
            if (changed) TMG_CUDA(cudaMemcpyAsync(ddone.p, done.data(), B * sizeof(int), cudaMemcpyHostToDevice, g_stream));
            return all;
        };
        if (spd) {
            // CG on A x = b preconditioned by the FP32 factor; FP64 operator and vectors
            TMG_CUDA(cudaMemsetAsync(x, 0, (size_t)B * n * sizeof(Tv), g_stream));
            lz_copy<Tv>(g_stream, (int64_t)B * n, b, r.p);
            if (mdef > 0) {   // deflated start x0 = W Einv W^H b, r0 = b - A x0
                const int64_t nm = (int64_t)n * mdef;
                lz_multidot<Tv>(g_stream, B, n, W.p, nm, n, mdef, b, n, pdef.p, hdef.p);
                TMG_LAUNCH(k_small_mv<Tv>, B, 32, 0, g_stream, mdef, Einv.p, hdef.p, ydef.p, -1.0);
                lz_gemv_sub<Tv>(g_stream, B, n, mdef, W.p, nm, ydef.p, mdef, x, n);
                lz_spmv<Tv>(g_stream, B, A, x, n, r.p, n, 1, n, true);
            }
            solve1(r.p, z.p);
            if (mdef > 0) deflate(z.p);
            lz_copy<Tv>(g_stream, (int64_t)B * n, z.p, pp.p);
            lz_multidot<Tv>(g_stream, B, n, r.p, n, n, 1, z.p, n, d.p, sc.p);           // rz
            for (it = 1; it <= max_iter; it++) {
                lz_spmv<Tv>(g_stream, B, A, pp.p, n, q.p, n, 1, n);
                lz_multidot<Tv>(g_stream, B, n, pp.p, n, n, 1, q.p, n, d.p, sc.p + B);   // pq
                TMG_LAUNCH(k_pcg_xr<Tv>, dim3(nblk(n), B), 256, 0, g_stream, n, x, r.p, pp.p, q.p, sc.p, sc.p + B, ddone.p);
                if (check()) break;
                solve1(r.p, z.p);
                if (mdef > 0) deflate(z.p);
                lz_multidot<Tv>(g_stream, B, n, r.p, n, n, 1, z.p, n, d.p, sc.p + 2 * B);  // rz_new
                TMG_LAUNCH(k_pcg_p<Tv>, dim3(nblk(n), B), 256, 0, g_stream, n, pp.p, z.p, sc.p + 2 * B, sc.p, ddone.p);
                TMG_CUDA(cudaMemcpyAsync(sc.p, sc.p + 2 * B, B * sizeof(Tv), cudaMemcpyDeviceToDevice, g_stream));
            }
        } else {
            it = gmres(b, x, bn, done, rn);
        }
        max_its = std::max<int64_t>(max_its, it);
        for (int p = 0; p < B; p++)
            if (!skip[p]) worst[p] = std::max(worst[p], std::sqrt(rn[p] / std::max(bn[p], 1e-300)));
    }
};

template <typename Tv>
struct EigOut {
    std::vector<double> lam;
    DVec<Tv> X;                 // n x ne
    int ne = 0, restarts = 0;
    bool converged = false, done = false;
    std::string failed;         // non-empty: the problem stopped with this error
};

template <typename Tv> Tv rnd_entry(std::mt19937& g, std::normal_distribution<double>& d);
template <> double rnd_entry<double>(std::mt19937& g, std::normal_distribution<double>& d) { return d(g); }
template <> zd rnd_entry<zd>(std::mt19937& g, std::normal_distribution<double>& d) {
    const double a = d(g);
    const double b = d(g);
    return zd{a, b};
}

// Shift-invert Lanczos (src/hermitian_lanczos.cpp:264-460) for a batch in lockstep, with
// device-resident bases and scalars; the host reads the converged counts after each
// restart cycle and extracts every problem as soon as it has converged.
template <typename Tv, typename Tf>
std::vector<EigOut<Tv>> lanczos(tmg_context* c, ShiftInvertB<Tv, Tf>& op, const DevCsr<Tv>& M, int nev, int ncv,
                                double shift, double tol, int max_restarts, const double* dshifts = nullptr) {
    const int64_t n = op.n;
    const int B = op.B;
    cudaStream_t st = g_stream;
    const int64_t vs = (int64_t)(ncv + 1) * n;
    DVec<Tv> V, MV, w, Mw, h, dot, part;
    V.alloc((size_t)B * vs); MV.alloc((size_t)B * vs);
    V.zero(st); MV.zero(st);
    w.alloc((size_t)B * n); Mw.alloc((size_t)B * n); h.alloc((size_t)B * (ncv + 1)); dot.alloc(B);
    part.alloc((size_t)B * LZ_DOT_BLOCKS * (ncv + 1));
    DVec<double> alpha, beta, theta, lam, S, Z, Q, rot;
    alpha.alloc((size_t)B * ncv); beta.alloc((size_t)B * ncv); theta.alloc((size_t)B * ncv); lam.alloc((size_t)B * ncv);
    S.alloc((size_t)B * ncv * ncv); Z.alloc((size_t)B * ncv * ncv); Q.alloc((size_t)B * ncv * ncv);
    const int64_t rs = (int64_t)2 * std::max(1, ncv - nev) * std::max(1, ncv - 1);
    rot.alloc((size_t)B * rs);
    alpha.zero(st); beta.zero(st);
    DVec<int> order, nconv, flag;
    order.alloc((size_t)B * ncv); nconv.alloc(B); flag.alloc(B);
    flag.zero(st);
    {
        std::mt19937 gen(42);
        std::normal_distribution<double> dist(0.0, 1.0);
        std::vector<Tv> v0(n);
        for (int64_t i = 0; i < n; i++) v0[i] = rnd_entry<Tv>(gen, dist);
        for (int p = 0; p < B; p++)
            TMG_CUDA(cudaMemcpyAsync(V.p + p * vs, v0.data(), n * sizeof(Tv), cudaMemcpyHostToDevice, st));
        TMG_CUDA(cudaStreamSynchronize(st));
        lz_spmv<Tv>(st, B, M, V.p, vs, MV.p, vs, 1, n);
        lz_multidot<Tv>(st, B, n, V.p, vs, n, 1, MV.p, vs, part.p, dot.p);
        lz_scale_first<Tv>(st, B, n, dot.p, V.p, MV.p, vs);
    }
    std::vector<EigOut<Tv>> out(B);
    const int m = ncv;
    int remaining = B;
    for (int p = 0; p < B; p++)
        if (!op.failed[p].empty()) { out[p].failed = op.failed[p]; out[p].done = true; remaining--; }
    for (int restart = 0; restart <= max_restarts && remaining > 0; restart++) {
        const int j0 = restart == 0 ? 0 : nev;
        for (int j = j0; j < m; j++) {
            op.apply(MV.p + (int64_t)j * n, vs, w.p);
            lz_multidot<Tv>(st, B, n, MV.p + (int64_t)j * n, vs, n, 1, w.p, n, part.p, dot.p);
            lz_three_term<Tv>(st, B, n, j, dot.p, alpha.p, beta.p, ncv, V.p, vs, w.p, n);
            lz_multidot<Tv>(st, B, n, MV.p, vs, n, j + 1, w.p, n, part.p, h.p);
            lz_gemv_sub<Tv>(st, B, n, j + 1, V.p, vs, h.p, j + 1, w.p, n);
            lz_spmv<Tv>(st, B, M, w.p, n, Mw.p, n, 1, n);
            lz_multidot<Tv>(st, B, n, w.p, n, n, 1, Mw.p, n, part.p, dot.p);
            lz_beta_scale<Tv>(st, B, n, j, dot.p, w.p, Mw.p, n, V.p, MV.p, vs, beta.p, ncv, flag.p);
        }
        std::vector<int> hflag(B), hn(B);
        TMG_CUDA(cudaMemcpyAsync(hflag.data(), flag.p, B * sizeof(int), cudaMemcpyDeviceToHost, st));
        TMG_CUDA(cudaStreamSynchronize(st));
        for (int p = 0; p < B; p++)
            if (hflag[p] && !out[p].done) {   // this problem stops alone; the batch goes on
                out[p].failed = "Lanczos breakdown (beta < 1e-14) at step " + std::to_string(hflag[p] - 1);
                out[p].done = true;
                op.skip[p] = 1;
                remaining--;
            }
        if (remaining == 0) break;
        lz_tridiag(st, B, m, ncv, nev, shift, tol, alpha.p, beta.p, theta.p, S.p, lam.p, order.p, nconv.p, Z.p,
                   dshifts);
        TMG_CUDA(cudaMemcpyAsync(hn.data(), nconv.p, B * sizeof(int), cudaMemcpyDeviceToHost, st));
        TMG_CUDA(cudaStreamSynchronize(st));
        for (int p = 0; p < B; p++) {
            if (out[p].done) continue;
            out[p].restarts = restart;
            if (!(hn[p] >= nev || restart == max_restarts)) continue;
            int ne = std::min(hn[p] > 0 ? hn[p] : nev, m);
            ne = std::min(ne, nev);
            std::vector<double> Sh((size_t)m * m), lh(m);
            std::vector<int> oh(m);
            TMG_CUDA(cudaMemcpyAsync(Sh.data(), S.p + (int64_t)p * ncv * ncv, Sh.size() * sizeof(double),
                                     cudaMemcpyDeviceToHost, st));
            TMG_CUDA(cudaMemcpyAsync(lh.data(), lam.p + (int64_t)p * ncv, m * sizeof(double), cudaMemcpyDeviceToHost, st));
            TMG_CUDA(cudaMemcpyAsync(oh.data(), order.p + (int64_t)p * ncv, m * sizeof(int), cudaMemcpyDeviceToHost, st));
            TMG_CUDA(cudaStreamSynchronize(st));
            std::vector<double> Csel((size_t)m * ne);
            out[p].lam.resize(ne);
            for (int t = 0; t < ne; t++) {
                out[p].lam[t] = lh[oh[t]];
                for (int k = 0; k < m; k++) Csel[(size_t)t * m + k] = Sh[(size_t)oh[t] * m + k];
            }
            DVec<double> dC;
            dC.upload(Csel);
            out[p].X.alloc((size_t)n * std::max(ne, 1));
            lz_gemm_real<Tv>(st, 1, n, m, ne, V.p + p * vs, 0, dC.p, 0, m, out[p].X.p, 0);
            TMG_CUDA(cudaStreamSynchronize(st));
            out[p].ne = ne;
            out[p].converged = hn[p] >= nev;
            out[p].done = true;
            op.skip[p] = 1;
            remaining--;
        }
        if (remaining == 0) break;
        // implicit restart (src/hermitian_lanczos.cpp:114-260) for the whole batch
        lz_restart_qr(st, B, m, ncv, nev, theta.p, alpha.p, beta.p, Q.p, rot.p, rs);
        DVec<Tv> Y;
        Y.alloc((size_t)B * n * (nev + 1));
        const int64_t yst = (int64_t)n * (nev + 1);
        lz_gemm_real<Tv>(st, B, n, m, nev + 1, V.p, vs, Q.p, (int64_t)ncv * ncv, m, Y.p, yst);
        lz_combine_f<Tv>(st, B, n, Y.p + (int64_t)nev * n, yst, V.p + (int64_t)m * n, vs, beta.p, ncv, nev, m, Q.p, w.p, n);
        for (int p = 0; p < B; p++) lz_copy<Tv>(st, (int64_t)nev * n, Y.p + p * yst, V.p + p * vs);
        lz_spmv<Tv>(st, B, M, w.p, n, Mw.p, n, 1, n);
        lz_multidot<Tv>(st, B, n, w.p, n, n, 1, Mw.p, n, part.p, dot.p);
        lz_restart_norm<Tv>(st, B, n, nev, dot.p, w.p, Mw.p, n, V.p, MV.p, vs, beta.p, ncv);
        lz_spmv<Tv>(st, B, M, V.p, vs, MV.p, vs, nev, n);
    }
    return out;
}

struct Problem {
    int k = 0;
    zd P{1.0, 0.0};
    bool degenerate = false;
    int nev_target = 0;
    ResultHost* R = nullptr;
};

// Mode-shape expansion u_full = T(0) u_reduced with the right-boundary rows times e^{ik alpha}
// (src/cyclic_solver.cpp:1185-1211); X holds nm free-space columns of n_free entries.
void expand_to_sector(tmg_context* c, const Problem& pr, const zd* X, int nm, ResultHost& R) {
    Sector& S = *c->sec;
    cudaStream_t st = g_stream;
    const int32_t ndof = 3 * S.nn;
    DVec<zd> full;
    full.alloc((size_t)ndof * std::max(nm, 1));
    if (nm) TMG_LAUNCH(k_expand, dim3(nblk(ndof), nm), 256, 0, st, ndof, c->dT0_rp.p, c->dT0_ci.p, c->dT0_v.p,
                       c->d_isr.p, c->d_r2free.p, X, (int64_t)S.n_free, pr.P, full.p, (int64_t)ndof);
    TMG_CHECK_LAUNCH();
    R.shapes.resize((size_t)ndof * nm);
    R.modal_mass.assign(nm, 0.0);
    if (nm) {
        // modal masses on the sector mass matrix (the one the solve assembled)
        assemble_KM(c);
        if (!S.dcand_i.p) S.dcand_i.upload(S.cand.i);
        DVec<double> part, mm;
        part.alloc((size_t)nm * MASS_BLOCKS);
        mm.alloc(nm);
        TMG_LAUNCH(k_mass_part, dim3(MASS_BLOCKS, nm), 256, 0, st, ndof, S.dcand_p.p, S.dcand_i.p, c->M.v.p, full.p,
                   (int64_t)ndof, part.p);
        TMG_LAUNCH(k_mass_sum, 1, nm, 0, st, MASS_BLOCKS, part.p, (double)S.ns, mm.p);
        TMG_CHECK_LAUNCH();
        TMG_CUDA(cudaMemcpyAsync(R.modal_mass.data(), mm.p, nm * sizeof(double), cudaMemcpyDeviceToHost, st));
        TMG_CUDA(cudaMemcpyAsync(R.shapes.data(), full.p, R.shapes.size() * sizeof(zd), cudaMemcpyDeviceToHost, st));
        TMG_CUDA(cudaStreamSynchronize(st));
    }
}

// Post-processing of one problem (cyclic_solver.cpp:1058-1211): frequencies, min-frequency
// filter, truncation, residual diagnostic, degenerate duplication, expansion to the full
// sector DOFs.
template <typename Tv>
void finish_result(tmg_context* c, const Problem& pr, EigOut<Tv>& eo, const DevCsr<Tv>& A, const DevCsr<Tv>& M,
                   double shift, int num_modes, double min_frequency, const double* residuals = nullptr) {
    Sector& S = *c->sec;
    ResultHost& R = *pr.R;
    cudaStream_t st = g_stream;
    const int64_t n = S.n_free;
    std::vector<int> keep;
    for (int t = 0; t < eo.ne; t++) {
        const double lam = eo.lam[t];
        const double f = lam > 0.0 ? std::sqrt(lam) / (2.0 * PI) : 0.0;
        if (min_frequency > 0.0 && !(f > min_frequency)) continue;
        keep.push_back(t);
    }
    if (min_frequency > 0.0 && keep.empty()) { R.status = TMG_ERR_NUMERIC; R.freqs.clear(); return; }
    if ((int)keep.size() > pr.nev_target) keep.resize(pr.nev_target);
    const int nk = (int)keep.size();
    DVec<Tv> Xk;
    Xk.alloc((size_t)n * std::max(nk, 1));
    std::vector<double> lam(nk);
    for (int t = 0; t < nk; t++) {
        lam[t] = eo.lam[keep[t]];
        lz_copy<Tv>(st, n, eo.X.p + (int64_t)keep[t] * n, Xk.p + (int64_t)t * n);
        R.freqs.push_back(lam[t] > 0.0 ? std::sqrt(lam[t]) / (2.0 * PI) : 0.0);
    }
    if (nk > 0 && residuals) {   // computed with the dense matrices
        for (int t = 0; t < nk; t++) R.max_residual = std::max(R.max_residual, residuals[keep[t]]);
    } else if (nk > 0) {   // ||K x - lambda M x|| / ||K x|| (cyclic_solver.cpp:1099-1114)
        DVec<Tv> AX, MX, KX, RR;
        DVec<double> dl, np, nr;
        AX.alloc((size_t)n * nk); MX.alloc((size_t)n * nk); KX.alloc((size_t)n * nk); RR.alloc((size_t)n * nk);
        dl.upload(lam);
        np.alloc((size_t)nk * LZ_DOT_BLOCKS); nr.alloc(nk);
        lz_spmv<Tv>(st, 1, A, Xk.p, 0, AX.p, 0, nk, n);
        lz_spmv<Tv>(st, 1, M, Xk.p, 0, MX.p, 0, nk, n);
        TMG_LAUNCH(k_resid<Tv>, dim3(nblk(n), nk), 256, 0, st, n, nk, AX.p, MX.p, dl.p, shift, KX.p, RR.p);
        std::vector<double> a(nk), b(nk);
        lz_norm2<Tv>(st, nk, n, RR.p, n, np.p, nr.p);
        TMG_CUDA(cudaMemcpyAsync(a.data(), nr.p, nk * sizeof(double), cudaMemcpyDeviceToHost, st));
        TMG_CUDA(cudaStreamSynchronize(st));
        lz_norm2<Tv>(st, nk, n, KX.p, n, np.p, nr.p);
        TMG_CUDA(cudaMemcpyAsync(b.data(), nr.p, nk * sizeof(double), cudaMemcpyDeviceToHost, st));
        TMG_CUDA(cudaStreamSynchronize(st));
        for (int t = 0; t < nk; t++)
            R.max_residual = std::max(R.max_residual, b[t] > 0 ? std::sqrt(a[t] / b[t]) : std::sqrt(a[t]));
    }
    DVec<zd> Xc;
    Xc.alloc((size_t)n * std::max(nk, 1));
    if constexpr (std::is_same<Tv, double>::value) {
        if (nk) TMG_LAUNCH(k_real_to_complex, nblk(n * nk), 256, 0, st, n * nk, Xk.p, Xc.p);
    } else {
        if (nk) lz_copy<zd>(st, n * nk, Xk.p, Xc.p);
    }
    int nm = nk;
    R.whirl.assign(nk, 0);
    DVec<zd> Xd;
    const zd* Xsrc = Xc.p;
    if (pr.degenerate && nk > 0) {
        nm = std::min(2 * nk, num_modes);
        Xd.alloc((size_t)n * nm);
        TMG_LAUNCH(k_dup_conj, dim3(nblk(n), nm), 256, 0, st, n, nm, Xc.p, Xd.p);
        std::vector<double> f2(nm);
        R.whirl.assign(nm, 0);
        for (int q = 0; q < nm; q++) { f2[q] = R.freqs[q / 2]; R.whirl[q] = (q % 2 == 0) ? 1 : -1; }
        R.freqs = f2;
        Xsrc = Xd.p;
    }
    expand_to_sector(c, pr, Xsrc, nm, R);
}

// Coriolis QEP post-processing (src/modal_solver.cpp:249-309, then src/cyclic_solver.cpp:
// 1058-1094 and :1185-1211): Ritz values |omega| < 1e-6 dropped, the lowest num_modes forward
// (omega > 0) and backward (omega < 0) values by |omega| kept and re-sorted by |omega|,
// frequencies |omega| / 2 pi, whirl +1 / -1, shapes = the first n rows of the 2n Lancaster
// vectors; then the min-frequency filter, the truncation to num_modes and the expansion to
// the sector DOFs.  The QEP has no residual check and no degenerate duplication.
void finish_qep(tmg_context* c, const Problem& pr, const EigOut<zd>& eo, int num_modes, double min_frequency) {
    Sector& S = *c->sec;
    ResultHost& R = *pr.R;
    const int64_t n = S.n_free, n2 = 2 * n;
    struct Entry { double om; int idx; int wh; };
    std::vector<Entry> ent;
    for (int i = 0; i < eo.ne; i++) {
        const double om = eo.lam[i];
        if (std::fabs(om) < 1e-6) continue;
        ent.push_back({om, i, om > 0 ? 1 : -1});
    }
    auto byabs = [](const Entry& a, const Entry& b) { return std::fabs(a.om) < std::fabs(b.om); };
    std::sort(ent.begin(), ent.end(), byabs);
    int nfw = 0, nbw = 0;
    std::vector<Entry> sel;
    for (const Entry& e : ent) {
        if (e.wh == 1 && nfw < num_modes) { sel.push_back(e); nfw++; }
        else if (e.wh == -1 && nbw < num_modes) { sel.push_back(e); nbw++; }
        if (nfw >= num_modes && nbw >= num_modes) break;
    }
    std::sort(sel.begin(), sel.end(), byabs);
    if (!eo.converged && sel.empty()) { R.status = TMG_ERR_NUMERIC; return; }
    std::vector<Entry> keep;
    for (const Entry& e : sel)
        if (!(min_frequency > 0.0) || std::fabs(e.om) / (2.0 * PI) > min_frequency) keep.push_back(e);
    if (keep.size() < sel.size() && keep.empty()) { R.status = TMG_ERR_NUMERIC; return; }
    if ((int)keep.size() > pr.nev_target) keep.resize(pr.nev_target);
    const int nm = (int)keep.size();
    DVec<zd> Xq;
    Xq.alloc((size_t)n * std::max(nm, 1));
    R.freqs.clear();
    R.whirl.clear();
    for (int t = 0; t < nm; t++) {
        R.freqs.push_back(std::fabs(keep[t].om) / (2.0 * PI));
        R.whirl.push_back(keep[t].wh);
        lz_copy<zd>(g_stream, n, eo.X.p + (int64_t)keep[t].idx * n2, Xq.p + (int64_t)t * n);
    }
    expand_to_sector(c, pr, Xq.p, nm, R);
}

// Factor and solve a batch of problems that share one symbolic analysis.
template <typename Tv, typename Tf>
void run_batch(tmg_context* c, std::vector<Problem>& probs, const OpSymbolic& os, const UnionMaps& um,
               const Tv* vals_csc, const DevCsr<Tv>& M, int nev, int ncv, double shift, int max_restarts, bool mixed,
               int num_modes, double min_frequency, const std::vector<double>* shifts = nullptr, bool qep = false,
               const Tv* Wdef = nullptr, int mdef = 0) {
    cudaStream_t st = g_stream;
    const int B = (int)probs.size();
    const int64_t nl = (int64_t)um.lower2csc.n, nU = um.U.nnz();
    DVec<Tv> lower, acsr;
    lower.alloc((size_t)B * nl);
    acsr.alloc((size_t)B * nU);
    if (nl) TMG_LAUNCH(k_gather_b<Tv>, dim3(nblk(nl), B), 256, 0, st, nl, um.lower2csc.p, vals_csc, nU, lower.p, nl);
    if (nU) TMG_LAUNCH(k_gather_b<Tv>, dim3(nblk(nU), B), 256, 0, st, nU, um.csr2csc.p, vals_csc, nU, acsr.p, nU);
    DevCsr<Tv> A;
    A.nrows = um.U.ncols; A.nnz = nU; A.rowptr = um.csr_rowptr.p; A.col = um.csr_col.p; A.val = acsr.p; A.vstride = nU;
    ShiftInvertB<Tv, Tf> op;
    op.c = c; op.D = &os.D; op.um = &um; op.n = um.U.ncols; op.B = B; op.mixed = mixed; op.A = A;
    op.rtol = c->refine_tol;
    auto t0 = std::chrono::steady_clock::now();
    op.factor(lower.p);
    lower.release();
    if (Wdef && mdef > 0) op.set_deflation(Wdef, mdef);
    auto t1 = std::chrono::steady_clock::now();
    DVec<double> dsh;
    if (shifts) dsh.upload(*shifts);
    std::vector<EigOut<Tv>> eo = lanczos<Tv, Tf>(c, op, M, nev, ncv, shift, 1e-8, max_restarts, shifts ? dsh.p : nullptr);
    auto t2 = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> lk(c->mu);
        c->phase_ms[1] += std::chrono::duration<double, std::milli>(t1 - t0).count();
        c->phase_ms[2] += std::chrono::duration<double, std::milli>(t2 - t1).count();
    }
    if constexpr (std::is_same<Tv, zd>::value) {
        if (c->deflate && !qep) {   // keep the lowest eigenvectors for the next speed
            if (c->recycle_key != c->symC_key) {
                c->recycle.clear();
                c->recycle_key = c->symC_key;
            }
            for (int p = 0; p < B; p++)
                if (eo[p].failed.empty() && eo[p].ne >= DEFL_M) {
                    DVec<zd>& w = c->recycle[probs[p].k];
                    w.alloc((size_t)op.n * DEFL_M);
                    TMG_CUDA(cudaMemcpyAsync(w.p, eo[p].X.p, w.bytes(), cudaMemcpyDeviceToDevice, st));
                }
        }
    }
    {
        std::lock_guard<std::mutex> lk(c->mu);
        c->phase_ms[5] += (double)op.solves;
        if (mixed && !qep && std::is_same<Tv, zd>::value) c->solves_per_factor = (double)op.solves;
        c->phase_ms[6] += (double)op.applies;
        c->phase_ms[7] = std::max(c->phase_ms[7], (double)op.max_its);
    }
    if (std::getenv("TMG_VERBOSE"))
        std::fprintf(stderr, "[tmg] batch B=%d n=%d %s: factor %.1f ms, lanczos %.1f ms, %lld solves (%lld launches each), "
                     "%lld applies, <=%lld refinement iterations\n", B, op.n, mixed ? "mixed" : "fp64",
                     std::chrono::duration<double, std::milli>(t1 - t0).count(),
                     std::chrono::duration<double, std::milli>(t2 - t1).count(), (long long)op.solves,
                     (long long)op.launches_per_solve, (long long)op.applies, (long long)op.max_its);
    for (int p = 0; p < B; p++) {
        ResultHost& R = *probs[p].R;
        R.converged = eo[p].converged;
        R.iterations = eo[p].restarts;
        R.refine_residual = op.worst[p];
        R.solves = op.solves;
        R.applies = op.applies;
        if (!eo[p].failed.empty()) { R.status = TMG_ERR_NUMERIC; note_err(c, eo[p].failed); continue; }
        if (!eo[p].converged && eo[p].ne == 0) { R.status = TMG_ERR_NUMERIC; continue; }
        if constexpr (std::is_same<Tv, zd>::value) {
            if (qep) { finish_qep(c, probs[p], eo[p], num_modes, min_frequency); continue; }
        }
        DevCsr<Tv> Ap = A, Mp = M;
        Ap.val = A.val + p * A.vstride;
        Mp.val = M.val + p * M.vstride;
        finish_result<Tv>(c, probs[p], eo[p], Ap, Mp, shift, num_modes, min_frequency);
    }
    auto t3 = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(c->mu);
    c->phase_ms[3] += std::chrono::duration<double, std::milli>(t3 - t2).count();
}

// ---- supernode-shape autotuner ----------------------------------------------------------
// For a new complex operator pattern (one per sector design and speed regime), each candidate
// shape is analysed (the AMD order is computed once and shared), factorised on the first batch
// of real operator values and its batched triangular solve timed, with CUDA events on the
// context's stream.  Score = factorisation + S x solve, S the FP32 solves per factorisation of
// the last mixed batch (256 before any, about what a config-1 batch needs; 45 in FP64).  The
// winner replaces the context's analysis and is cached per pattern fingerprint for every
// context of the process.
std::mutex g_tune_mu;
std::map<std::string, TuneCand> g_tune_cache;

template <typename Tf>
TuneRow tune_trial(tmg_context* c, OpSymbolic& os, const UnionMaps& um, const zd* vals_csc, int B, bool mixed) {
    cudaStream_t st = c->st;
    const int64_t nl = (int64_t)um.lower2csc.n, nU = um.U.nnz();
    DVec<zd> lower, acsr;
    lower.alloc((size_t)B * nl);
    acsr.alloc((size_t)B * nU);
    if (nl) TMG_LAUNCH(k_gather_b<zd>, dim3(nblk(nl), B), 256, 0, st, nl, um.lower2csc.p, vals_csc, nU, lower.p, nl);
    if (nU) TMG_LAUNCH(k_gather_b<zd>, dim3(nblk(nU), B), 256, 0, st, nU, um.csr2csc.p, vals_csc, nU, acsr.p, nU);
    ShiftInvertB<zd, Tf> op;
    op.c = c; op.D = &os.D; op.um = &um; op.n = um.U.ncols; op.B = B; op.mixed = mixed;
    op.A.nrows = um.U.ncols; op.A.nnz = nU; op.A.rowptr = um.csr_rowptr.p; op.A.col = um.csr_col.p;
    op.A.val = acsr.p; op.A.vstride = nU;
    cudaEvent_t ev[4];
    for (auto& e : ev) TMG_CUDA(cudaEventCreate(&e));
    TMG_CUDA(cudaEventRecord(ev[0], st));
    op.factor(lower.p);
    TMG_CUDA(cudaEventRecord(ev[1], st));
    lower.release();
    op.solve1(op.r.p, op.z.p);   // the first solve captures the graph
    TMG_CUDA(cudaEventRecord(ev[2], st));
    const int ns = 4;
    for (int q = 0; q < ns; q++) op.solve1(op.r.p, op.z.p);
    TMG_CUDA(cudaEventRecord(ev[3], st));
    TMG_CUDA(cudaEventSynchronize(ev[3]));
    TuneRow row;
    float f_ms = 0.f, s_ms = 0.f;
    TMG_CUDA(cudaEventElapsedTime(&f_ms, ev[0], ev[1]));
    TMG_CUDA(cudaEventElapsedTime(&s_ms, ev[2], ev[3]));
    row.factor_ms = f_ms;
    row.solve_ms = s_ms / ns;
    for (auto& e : ev) cudaEventDestroy(e);
    row.stored = os.D.l_entries;
    row.supernodes = os.D.ns;
    return row;
}

void tune_complex(tmg_context* c, const UnionMaps& um, const zd* vals_csc, int B, bool mixed) {
    const std::string key = c->symC_key + (mixed ? "|mixed" : "|fp64");
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            const TuneCand& w = it->second;
            if (w.relax != c->tune_choice.relax || w.maxw != c->tune_choice.maxw || w.tc_min != c->tune_choice.tc_min) {
                const std::vector<int32_t> amd = c->symC.S.amd;
                analyze_op(c->symC, um, &w, &amd);
            }
            c->tune_choice = w;
            c->tuned_key = c->symC_key;
            return;
        }
    }
    std::vector<TuneCand> cands = {{0.0, 0, MF_TC_MIN_ROWS}, {0.1, 256, MF_TC_MIN_ROWS}, {0.25, 256, MF_TC_MIN_ROWS},
                                   {0.25, 512, MF_TC_MIN_ROWS}};
    if (mixed) cands.push_back({0.0, 0, 384});
    const double S = c->solves_per_factor > 0 ? c->solves_per_factor : (mixed ? 256.0 : 45.0);
    const std::vector<int32_t> amd = c->symC.S.amd;
    c->tune_rows.clear();
    int best = -1;
    for (size_t q = 0; q < cands.size(); q++) {
        OpSymbolic os;
        analyze_op(os, um, &cands[q], &amd);
        TuneRow row = mixed ? tune_trial<zf>(c, os, um, vals_csc, B, true) : tune_trial<zd>(c, os, um, vals_csc, B, false);
        row.cand = cands[q];
        row.score_ms = row.factor_ms + S * row.solve_ms;
        c->tune_rows.push_back(row);
        if (best < 0 || row.score_ms < c->tune_rows[best].score_ms) best = (int)q;
        if (std::getenv("TMG_VERBOSE"))
            std::fprintf(stderr, "[tmg] tune relax %.2f maxw %d tc %d: factor %.1f ms, solve %.2f ms, score %.1f ms, "
                         "%lld stored, %d supernodes\n", cands[q].relax, cands[q].maxw, cands[q].tc_min,
                         row.factor_ms, row.solve_ms, row.score_ms, (long long)row.stored, row.supernodes);
    }
    const TuneCand w = cands[best];
    analyze_op(c->symC, um, &w, &amd);
    c->tune_choice = w;
    c->tuned_key = c->symC_key;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = w;
}

// Problems per batch that fit the device-memory budget.
int batch_size(tmg_context* c, const OpSymbolic& os, const UnionMaps& um, int64_t nM, int ncv, bool cplx, bool mixed,
               int nprob) {
    const double vb = cplx ? 16.0 : 8.0;                       // FP64 vector entry
    const double fb = mixed ? vb / 2 : vb;                     // factor entry
    const DevSymbolic& D = os.D;
    const double n = um.U.ncols;
    const double per = fb * (double)(D.l_entries + D.u_entries + D.t_entries + n) +
                       vb * (double)(3 * um.U.nnz() + 2 * um.lower2csc.n + 2 * nM) +
                       vb * n * (2.0 * (ncv + 1) + 12.0) + 8.0 * ncv * ncv * 4;
    const double avail = std::min<double>((double)c->budget, 0.85 * (double)device_free_bytes(c->device));
    const int b = (int)std::floor(avail / per);
    if (b < 1) throw numeric_error("device memory budget too small for one problem");
    return std::max(1, std::min(nprob, b));
}

// Coriolis harmonics k > 0: the Lancaster QEP (src/modal_solver.cpp:200-312) on the 2n block
// operator.  Shift per harmonic sqrt(|K_k|_F / |M_k|_F) (src/cyclic_solver.cpp:985-1006, the
// square root taken at src/modal_solver.cpp:243); nev = 2n - 1 on
// the dense path (2n <= 200), else min(6 num_modes, 2n - 1) with ncv = min(max(4 nev + 1, 40),
// 2n) and 20 restarts, batched like the standard harmonics under the memory budget.  The shifted
// operator [[D - sigma M, K], [K, -sigma K]] is indefinite and factorised without pivoting, as
// in the reference, where refinement of an FP32 factor has no convergence guarantee: the QEP
// runs in FP64 at either precision setting.
void solve_qep(tmg_context* c, std::vector<Problem>& probs, int num_modes, double min_frequency) {
    Sector& S = *c->sec;
    cudaStream_t st = c->st;
    ensure_qep(c);
    auto& Q = c->qep;
    const int64_t n2 = 2 * (int64_t)S.n_free;
    const double two_omega = 2.0 * (c->rpm * 2.0 * PI / 60.0);
    const bool dense = n2 <= 200;
    const int nev = dense ? (int)n2 - 1 : (int)std::min<int64_t>(6 * (int64_t)num_modes, n2 - 1);
    const int ncv = (int)std::min<int64_t>(std::max(4 * nev + 1, 40), n2);
    if (nev <= 0 || (!dense && ncv > LZ_MAXM)) {
        for (auto& pr : probs) pr.R->status = TMG_ERR_NUMERIC;
        c->err = nev <= 0 ? "Coriolis QEP: system too small for the requested modes"
                          : "Coriolis QEP: a Lanczos subspace of " + std::to_string(ncv) + " vectors (num_modes > " +
                                std::to_string((LZ_MAXM - 1) / 24) + ") is not supported";
        return;
    }
    const UnionMaps &WK = c->W0, &WM = c->WM0, &WG = c->WG0;
    const int64_t nK = WK.U.nnz(), nM = WM.U.nnz(), nG = WG.U.nnz();
    const int64_t nA = Q.op.U.nnz(), nL = Q.l2.U.nnz();
    int bmax = (int)probs.size();
    if (!dense) {
        if (!Q.sym.valid) analyze_op(Q.sym, Q.op);
        bmax = batch_size(c, Q.sym, Q.op, nL, ncv, true, false, (int)probs.size());
    }
    for (size_t b0 = 0; b0 < probs.size(); b0 += bmax) {
        std::vector<Problem> grp(probs.begin() + b0, probs.begin() + std::min(probs.size(), b0 + bmax));
        const int B = (int)grp.size();
        std::vector<double> ph(2 * B);
        for (int p = 0; p < B; p++) { ph[2 * p] = grp[p].P.x; ph[2 * p + 1] = grp[p].P.y; }
        DVec<double> dph;
        dph.upload(ph);
        // K_k, M_k, G_k on their structural domains
        DVec<zd> Kv, Mv, Gv;
        Kv.alloc((size_t)B * std::max<int64_t>(1, nK));
        Mv.alloc((size_t)B * std::max<int64_t>(1, nM));
        Gv.alloc((size_t)B * std::max<int64_t>(1, nG));
        if (nK) TMG_LAUNCH(k_form_csum, dim3(nblk(nK), B), 256, 0, st, nK, WK.maps[0].p, WK.maps[1].p, WK.maps[2].p,
                           c->Kcf.sv.p, c->Kpf.sv.p, dph.p, Kv.p);
        if (nM) TMG_LAUNCH(k_form_csum, dim3(nblk(nM), B), 256, 0, st, nM, WM.maps[0].p, WM.maps[1].p, WM.maps[2].p,
                           c->Mcf.sv.p, c->Mpf.sv.p, dph.p, Mv.p);
        if (nG) TMG_LAUNCH(k_form_csum, dim3(nblk(nG), B), 256, 0, st, nG, WG.maps[0].p, WG.maps[1].p, WG.maps[2].p,
                           c->Gcf.sv.p, c->Gpf.sv.p, dph.p, Gv.p);
        std::vector<double> sig(B);
        {
            DVec<double> part, nk2, nm2;
            part.alloc((size_t)B * LZ_DOT_BLOCKS);
            nk2.alloc(B);
            nm2.alloc(B);
            lz_norm2<zd>(st, B, nK, Kv.p, nK, part.p, nk2.p);
            lz_norm2<zd>(st, B, nM, Mv.p, nM, part.p, nm2.p);
            const std::vector<double> hk = nk2.download(), hm = nm2.download();
            for (int p = 0; p < B; p++) {
                const double mn = std::sqrt(hm[p]);
                const double sh = mn > 0.0 ? std::sqrt(hk[p]) / mn : 1.0;
                sig[p] = sh > 0.0 ? std::sqrt(sh) : 0.1;
            }
        }
        DVec<double> dsig;
        dsig.upload(sig);
        if (dense) {   // all eigenpairs of (L1, L2) by the dense solver (src/hermitian_lanczos.cpp:68-110)
            const int64_t nn = n2 * n2;
            DVec<zd> L1v, L2v, L1d, L2d, work, X;
            DVec<double> lam, res;
            DVec<int> status;
            L1v.alloc((size_t)B * nA); L2v.alloc((size_t)B * nA);
            for (int mode : {1, 2})
                TMG_LAUNCH(k_form_lancaster, dim3(nblk(nA), B), 256, 0, st, nA, Q.sk.p, Q.sm.p, Q.sg.p, Q.blk.p, Kv.p,
                           nK, Mv.p, nM, Gv.p, nG, two_omega, dsig.p, mode, mode == 1 ? L1v.p : L2v.p);
            L1d.alloc((size_t)B * nn); L2d.alloc((size_t)B * nn); work.alloc((size_t)B * 5 * nn);
            X.alloc((size_t)B * n2 * nev); lam.alloc((size_t)B * nev); res.alloc((size_t)B * nev); status.alloc(B);
            status.zero(st);
            DVec<int64_t> cp;
            DVec<int32_t> ri;
            cp.upload(Q.op.U.p);
            ri.upload(Q.op.U.i);
            for (int p = 0; p < B; p++) {
                dense_csc_to_dense(st, (int)n2, cp.p, ri.p, L1v.p + p * nA, L1d.p + p * nn);
                dense_csc_to_dense(st, (int)n2, cp.p, ri.p, L2v.p + p * nA, L2d.p + p * nn);
            }
            auto t1 = std::chrono::steady_clock::now();
            dense_geig(st, B, (int)n2, nev, L1d.p, L2d.p, work.p, lam.p, X.p, res.p, status.p);
            const std::vector<double> hl = lam.download();
            const std::vector<int> hs = status.download();
            c->phase_ms[2] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
            for (int p = 0; p < B; p++) {
                ResultHost& R = *grp[p].R;
                if (hs[p]) { R.status = TMG_ERR_NUMERIC; c->err = "dense eigensolver: L2 is not positive definite"; continue; }
                EigOut<zd> eo;
                eo.ne = nev;
                eo.converged = true;
                eo.lam.assign(hl.begin() + (int64_t)p * nev, hl.begin() + (int64_t)(p + 1) * nev);
                eo.X.alloc((size_t)n2 * nev);
                lz_copy<zd>(st, n2 * nev, X.p + (int64_t)p * n2 * nev, eo.X.p);
                R.converged = 1;
                finish_qep(c, grp[p], eo, num_modes, min_frequency);
            }
            continue;
        }
        DVec<zd> vals, l2c, l2r;
        vals.alloc((size_t)B * nA);
        l2c.alloc((size_t)B * nL);
        l2r.alloc((size_t)B * nL);
        TMG_LAUNCH(k_form_lancaster, dim3(nblk(nA), B), 256, 0, st, nA, Q.sk.p, Q.sm.p, Q.sg.p, Q.blk.p, Kv.p, nK, Mv.p,
                   nM, Gv.p, nG, two_omega, dsig.p, 0, vals.p);
        TMG_LAUNCH(k_form_lancaster, dim3(nblk(nL), B), 256, 0, st, nL, Q.sk2.p, Q.sm2.p, Q.sg2.p, Q.blk2.p, Kv.p, nK,
                   Mv.p, nM, Gv.p, nG, two_omega, dsig.p, 2, l2c.p);
        TMG_LAUNCH(k_gather_b<zd>, dim3(nblk(nL), B), 256, 0, st, nL, Q.l2.csr2csc.p, l2c.p, nL, l2r.p, nL);
        l2c.release(); Kv.release(); Mv.release(); Gv.release();
        DevCsr<zd> L2;
        L2.nrows = n2; L2.nnz = nL; L2.rowptr = Q.l2.csr_rowptr.p; L2.col = Q.l2.csr_col.p; L2.val = l2r.p;
        L2.vstride = nL;
        try {
            run_batch<zd, zd>(c, grp, Q.sym, Q.op, vals.p, L2, nev, ncv, 0.0, 20, false, num_modes, min_frequency,
                              &sig, true);
        } catch (const numeric_error& e) {
            for (auto& pr : grp) pr.R->status = TMG_ERR_NUMERIC;
            c->err = e.what();
        }
    }
}

// Problems of a mixed batch that the mixed path could not finish: an FP32 zero pivot or a
// Lanczos breakdown (status TMG_ERR_NUMERIC), or refined solves that stalled above 100x their
// target residual.  They are solved again on the plain FP64 path, as the reference retries the
// harmonics that failed in its thread pool (src/cyclic_solver.cpp:1334-1342).
std::vector<Problem> mixed_failures(tmg_context* c, const std::vector<Problem>& grp) {
    std::vector<Problem> out;
    for (const Problem& pr : grp) {
        ResultHost& R = *pr.R;
        if (R.status == TMG_ERR_NUMERIC || (R.status == TMG_OK && R.refine_residual > 100.0 * c->refine_tol)) {
            ResultHost fresh;
            fresh.k = R.k;
            fresh.rpm = R.rpm;
            R = fresh;
            out.push_back(pr);
        }
    }
    {
        std::lock_guard<std::mutex> lk(c->mu);
        c->phase_ms[8] += (double)out.size();
    }
    if (!out.empty() && std::getenv("TMG_VERBOSE"))
        std::fprintf(stderr, "[tmg] %zu problem(s) of a mixed batch solved again in FP64\n", out.size());
    return out;
}

void solve_set(tmg_context* c, const std::vector<int>& ks, int num_modes, double min_frequency, int precision,
               std::vector<ResultHost>& results) {
    Sector& S = *c->sec;
    cudaStream_t st = c->st;
    const int N = S.ns, max_k = N / 2;
    const double alpha = 2.0 * PI / N;
    const bool mixed = precision == TMG_PREC_MIXED;
    const double shift = c->shift;
    results.assign(ks.size(), ResultHost{});
    std::vector<Problem> cplx, real0, realh, dense, qep;
    for (size_t q = 0; q < ks.size(); q++) {
        const int k = ks[q];
        ResultHost& R = results[q];
        R.k = k;
        R.rpm = c->rpm;
        Problem pr;
        pr.k = k;
        pr.P = zd{std::cos(k * alpha), std::sin(k * alpha)};
        pr.R = &R;
        if (S.n_free <= 1) { R.status = TMG_ERR_ARG; continue; }
        pr.degenerate = (k > 0) && !(N % 2 == 0 && k == max_k);
        if (c->coriolis && k > 0) {   // QEP: the full mode count, no degenerate duplication
            pr.nev_target = num_modes;
            qep.push_back(pr);
            continue;
        }
        pr.nev_target = pr.degenerate ? (num_modes + 1) / 2 : num_modes;
        const bool is_real = (k == 0) || (N % 2 == 0 && k == max_k);
        if (S.n_free <= 200) { dense.push_back(pr); continue; }
        if (!is_real) cplx.push_back(pr);
        else if (k == 0) real0.push_back(pr);
        else realh.push_back(pr);
    }
    const int n_extra = min_frequency > 0.0 ? 6 : 0;
    // small sectors (n <= 200): dense generalized eigensolver, all harmonics in one launch
    // (src/hermitian_lanczos.cpp:68-110, :283)
    if (!dense.empty()) {
        const int n = S.n_free;
        const int B = (int)dense.size();
        int nev = 1;                                           // computed for every problem
        for (const Problem& pr : dense) nev = std::max(nev, std::min(pr.nev_target + n_extra, n - 1));
        const int64_t nn = (int64_t)n * n;
        DVec<zd> Kd, Md, work, X;
        DVec<double> lam, res;
        DVec<int> status;
        Kd.alloc((size_t)B * nn); Md.alloc((size_t)B * nn); work.alloc((size_t)B * 5 * nn);
        X.alloc((size_t)B * n * nev); lam.alloc((size_t)B * nev); res.alloc((size_t)B * nev); status.alloc(B);
        status.zero(st);
        for (int p = 0; p < B; p++) {
            const Problem& pr = dense[p];
            const bool is_real = (pr.k == 0) || (N % 2 == 0 && pr.k == max_k);
            for (int which = 0; which < 2; which++) {      // 0: K_k, 1: M_k
                DVec<int64_t> cp;
                DVec<int32_t> ri;
                DVec<zd> v;
                if (is_real) {
                    const auto& R = c->real[pr.k == 0 ? 0 : 1];
                    if (!R.valid) throw numeric_error("real harmonic operator missing");
                    const FreeMat& fm = which == 0 ? R.Kr : R.Mr;
                    cp.upload(fm.pat.p); ri.upload(fm.pat.i);
                    v.alloc(std::max<size_t>(1, fm.v.n));
                    if (fm.v.n) TMG_LAUNCH(k_real_to_complex, nblk(fm.v.n), 256, 0, st, (int64_t)fm.v.n, fm.v.p, v.p);
                } else {
                    const UnionMaps& w = which == 0 ? c->W0 : c->WM0;
                    const FreeMat& cc = which == 0 ? c->Kcf : c->Mcf;
                    const FreeMat& pp = which == 0 ? c->Kpf : c->Mpf;
                    cp.upload(w.U.p); ri.upload(w.U.i);
                    DVec<double> ph;
                    ph.upload(std::vector<double>{pr.P.x, pr.P.y});
                    v.alloc(std::max<int64_t>(1, w.U.nnz()));
                    if (w.U.nnz())
                        TMG_LAUNCH(k_form_csum, dim3(nblk(w.U.nnz()), 1), 256, 0, st, w.U.nnz(), w.maps[0].p,
                                   w.maps[1].p, w.maps[2].p, cc.sv.p, pp.sv.p, ph.p, v.p);
                    TMG_CUDA(cudaStreamSynchronize(st));
                }
                dense_csc_to_dense(st, n, cp.p, ri.p, v.p, (which == 0 ? Kd.p : Md.p) + p * nn);
                TMG_CUDA(cudaStreamSynchronize(st));
            }
        }
        auto t1 = std::chrono::steady_clock::now();
        dense_geig(st, B, n, nev, Kd.p, Md.p, work.p, lam.p, X.p, res.p, status.p);
        const std::vector<double> hl = lam.download(), hr = res.download();
        const std::vector<int> hs = status.download();
        auto t2 = std::chrono::steady_clock::now();
        c->phase_ms[2] += std::chrono::duration<double, std::milli>(t2 - t1).count();
        DevCsr<zd> none;
        for (int p = 0; p < B; p++) {
            ResultHost& R = *dense[p].R;
            if (hs[p]) { R.status = TMG_ERR_NUMERIC; c->err = "dense eigensolver: M is not positive definite"; continue; }
            const int nev_p = std::max(1, std::min(dense[p].nev_target + n_extra, n - 1));
            EigOut<zd> eo;
            eo.ne = nev_p;
            eo.converged = true;
            eo.lam.assign(hl.begin() + (int64_t)p * nev, hl.begin() + (int64_t)p * nev + nev_p);
            eo.X.alloc((size_t)n * nev_p);
            lz_copy<zd>(st, (int64_t)n * nev_p, X.p + (int64_t)p * n * nev, eo.X.p);
            R.converged = 1;
            finish_result<zd>(c, dense[p], eo, none, none, shift, num_modes, min_frequency, hr.data() + (int64_t)p * nev);
        }
        c->phase_ms[3] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t2).count();
    }
    // real harmonics k = 0 and N/2: one batch (of one or two problems) on the structural
    // domains W (operator) and W_M (mass), whose analysis is shared by both and by every speed
    {
        std::vector<Problem> grp;
        for (auto* g : {&real0, &realh})
            for (auto& pr : *g) {
                if (!c->real[pr.k == 0 ? 0 : 1].valid) { pr.R->status = TMG_ERR_STATE; continue; }
                grp.push_back(pr);
            }
        if (!grp.empty()) {
            if (!c->pairSym.valid) analyze_op(c->pairSym, c->pairOp);
            const int nev = std::min(grp[0].nev_target + n_extra, S.n_free - 1);
            const int ncv = std::min(std::max(4 * nev + 1, 40), S.n_free);
            UnionMaps& um = c->pairOp;
            UnionMaps& mu = c->pairM;
            const int B = (int)grp.size();
            const int64_t nU = um.U.nnz(), nMU = mu.U.nnz();
            DVec<double> vals, mcsc, mcsr;
            vals.alloc((size_t)B * nU);
            mcsc.alloc((size_t)B * nMU);
            mcsr.alloc((size_t)B * nMU);
            for (int q = 0; q < B; q++) {
                const auto& R = c->real[grp[q].k == 0 ? 0 : 1];
                if (nU)
                    TMG_LAUNCH(k_form_real_op, nblk(nU), 256, 0, st, nU, um.maps[0].p, um.maps[1].p, R.Ks.p, R.Ms.p,
                               shift, 1.0, vals.p + q * nU);
                if (nMU)
                    TMG_LAUNCH(k_form_real_op, nblk(nMU), 256, 0, st, nMU, mu.maps[0].p, mu.maps[0].p, R.Ms.p, R.Ms.p,
                               0.0, 1.0, mcsc.p + q * nMU);
            }
            if (nMU)
                TMG_LAUNCH(k_gather_b<double>, dim3(nblk(nMU), B), 256, 0, st, nMU, mu.csr2csc.p, mcsc.p, nMU, mcsr.p,
                           nMU);
            mcsc.release();
            DevCsr<double> M;
            M.nrows = S.n_free; M.nnz = nMU; M.rowptr = mu.csr_rowptr.p; M.col = mu.csr_col.p; M.val = mcsr.p;
            M.vstride = nMU;
            try {
                if (mixed)
                    run_batch<double, float>(c, grp, c->pairSym, um, vals.p, M, nev, ncv, shift, 1000, true, num_modes,
                                             min_frequency);
                else
                    run_batch<double, double>(c, grp, c->pairSym, um, vals.p, M, nev, ncv, shift, 1000, false,
                                              num_modes, min_frequency);
            } catch (const numeric_error& e) {
                for (auto& pr : grp) pr.R->status = TMG_ERR_NUMERIC;
                c->err = e.what();
            }
            if (mixed) {
                std::vector<Problem> again = mixed_failures(c, grp);
                if (!again.empty()) {
                    // the retried problems' operator and mass values, compacted to the batch's front
                    DVec<double> v2, m2;
                    v2.alloc((size_t)again.size() * nU);
                    m2.alloc((size_t)again.size() * nMU);
                    for (size_t q = 0; q < again.size(); q++) {
                        size_t src = 0;
                        while (grp[src].R != again[q].R) src++;
                        if (nU) lz_copy<double>(st, nU, vals.p + src * nU, v2.p + q * nU);
                        if (nMU) lz_copy<double>(st, nMU, mcsr.p + src * nMU, m2.p + q * nMU);
                    }
                    DevCsr<double> M2 = M;
                    M2.val = m2.p;
                    try {
                        run_batch<double, double>(c, again, c->pairSym, um, v2.p, M2, nev, ncv, shift, 1000, false,
                                                  num_modes, min_frequency);
                    } catch (const numeric_error& e) {
                        for (auto& pr : again) pr.R->status = TMG_ERR_NUMERIC;
                        c->err = e.what();
                    } catch (const cuda_error& e) {   // the FP64 factor does not fit: these problems fail alone
                        if (!std::strstr(e.what(), "out of memory")) throw;
                        for (auto& pr : again) pr.R->status = TMG_ERR_NOMEM;
                        c->err = std::string("FP64 retry of a mixed-path failure: ") + e.what();
                    }
                }
            }
        }
    }
    // complex harmonics: one shared symbolic analysis, batched under the memory budget
    if (!cplx.empty()) {
        if (!c->symC.valid) { analyze_op(c->symC, c->opC); c->tune_choice = TuneCand{}; }
        UnionMaps& um = c->opC;
        UnionMaps& mu = c->opMC;
        int nev = std::min(cplx[0].nev_target + n_extra, S.n_free - 1);
        const int ncv = std::min(std::max(4 * nev + 1, 40), S.n_free);
        const int bmax = batch_size(c, c->symC, um, mu.U.nnz(), ncv, true, mixed, (int)cplx.size());
        for (size_t b0 = 0; b0 < cplx.size(); b0 += bmax) {
            std::vector<Problem> grp(cplx.begin() + b0, cplx.begin() + std::min(cplx.size(), b0 + bmax));
            const int B = (int)grp.size();
            std::vector<double> ph(2 * B);
            for (int p = 0; p < B; p++) { ph[2 * p] = grp[p].P.x; ph[2 * p + 1] = grp[p].P.y; }
            DVec<double> dph;
            dph.upload(ph);
            DVec<zd> vals, mvals, mcsr;
            vals.alloc((size_t)B * um.U.nnz());
            mvals.alloc((size_t)B * mu.U.nnz());
            mcsr.alloc((size_t)B * mu.U.nnz());
            if (um.U.nnz())
                TMG_LAUNCH(k_form_complex, dim3(nblk(um.U.nnz()), B), 256, 0, st, um.U.nnz(), um.maps[0].p, um.maps[1].p,
                           um.maps[2].p, um.maps[3].p, um.maps[4].p, um.maps[5].p, c->Kcf.sv.p, c->Kpf.sv.p, c->Mcf.sv.p,
                           c->Mpf.sv.p, dph.p, shift, vals.p);
            if (mu.U.nnz()) {
                TMG_LAUNCH(k_form_csum, dim3(nblk(mu.U.nnz()), B), 256, 0, st, mu.U.nnz(), mu.maps[0].p, mu.maps[1].p,
                           mu.maps[2].p, c->Mcf.sv.p, c->Mpf.sv.p, dph.p, mvals.p);
                TMG_LAUNCH(k_gather_b<zd>, dim3(nblk(mu.U.nnz()), B), 256, 0, st, mu.U.nnz(), mu.csr2csc.p, mvals.p,
                           mu.U.nnz(), mcsr.p, mu.U.nnz());
            }
            mvals.release();
            if (c->autotune && c->tuned_key != c->symC_key) tune_complex(c, um, vals.p, B, mixed);
            DevCsr<zd> M;
            M.nrows = S.n_free; M.nnz = mu.U.nnz(); M.rowptr = mu.csr_rowptr.p; M.col = mu.csr_col.p; M.val = mcsr.p;
            M.vstride = mu.U.nnz();
            // previous speed's eigenvectors of every harmonic of the batch, when all are kept
            DVec<zd> Wd;
            int md = 0;
            if (mixed && c->deflate && c->recycle_key == c->symC_key) {
                bool all = true;
                for (const Problem& pr : grp) {
                    auto it = c->recycle.find(pr.k);
                    all = all && it != c->recycle.end() && it->second.n == (size_t)S.n_free * DEFL_M;
                }
                if (all) {
                    const size_t nm = (size_t)S.n_free * DEFL_M;
                    Wd.alloc((size_t)B * nm);
                    for (int p = 0; p < B; p++)
                        TMG_CUDA(cudaMemcpyAsync(Wd.p + p * nm, c->recycle[grp[p].k].p, nm * sizeof(zd),
                                                 cudaMemcpyDeviceToDevice, st));
                    md = DEFL_M;
                }
            }
            try {
                if (mixed)
                    run_batch<zd, zf>(c, grp, c->symC, um, vals.p, M, nev, ncv, shift, 1000, true, num_modes,
                                      min_frequency, nullptr, false, md ? Wd.p : nullptr, md);
                else
                    run_batch<zd, zd>(c, grp, c->symC, um, vals.p, M, nev, ncv, shift, 1000, false, num_modes,
                                      min_frequency);
            } catch (const numeric_error& e) {
                for (auto& pr : grp) pr.R->status = TMG_ERR_NUMERIC;
                c->err = e.what();
            }
            if (mixed) {
                std::vector<Problem> again = mixed_failures(c, grp);
                if (!again.empty()) {
                    const int64_t nU = um.U.nnz(), nMU = mu.U.nnz();
                    DVec<zd> v2, m2;
                    v2.alloc((size_t)again.size() * nU);
                    m2.alloc((size_t)again.size() * nMU);
                    for (size_t q = 0; q < again.size(); q++) {
                        size_t src = 0;
                        while (grp[src].R != again[q].R) src++;
                        if (nU) lz_copy<zd>(st, nU, vals.p + src * nU, v2.p + q * nU);
                        if (nMU) lz_copy<zd>(st, nMU, mcsr.p + src * nMU, m2.p + q * nMU);
                    }
                    DevCsr<zd> M2 = M;
                    M2.val = m2.p;
                    try {
                        run_batch<zd, zd>(c, again, c->symC, um, v2.p, M2, nev, ncv, shift, 1000, false, num_modes,
                                          min_frequency);
                    } catch (const numeric_error& e) {
                        for (auto& pr : again) pr.R->status = TMG_ERR_NUMERIC;
                        c->err = e.what();
                    } catch (const cuda_error& e) {   // the FP64 factor does not fit: these problems fail alone
                        if (!std::strstr(e.what(), "out of memory")) throw;
                        for (auto& pr : again) pr.R->status = TMG_ERR_NOMEM;
                        c->err = std::string("FP64 retry of a mixed-path failure: ") + e.what();
                    }
                }
            }
        }
    }
    if (!qep.empty()) solve_qep(c, qep, num_modes, min_frequency);
    TMG_CUDA(cudaStreamSynchronize(st));
}

// Several speeds of a sweep in one pass (src/cyclic_solver.cpp:1359-1373 solves them one after
// another).  The speeds are taken in groups that share the operator pattern (rest and speed
// differ) and fit the device-memory budget; each speed of a group is prepared in turn and the
// operator and mass values of its harmonics are formed into one multi-speed batch, so every
// factorisation and Lanczos launch covers the harmonics of all speeds of the group.  Dense
// (n <= 200) and Coriolis problems keep the per-speed path.  results: speed-major, harmonics in
// the order of ks.
void solve_sweep(tmg_context* c, const std::vector<double>& rpms, const std::vector<int>& ks, int num_modes,
                 double min_frequency, int precision, std::vector<ResultHost>& results) {
    Sector& S = *c->sec;
    cudaStream_t st = c->st;
    const int N = S.ns, max_k = N / 2;
    const double alpha = 2.0 * PI / N;
    const bool mixed = precision == TMG_PREC_MIXED;
    const double shift = c->shift;
    const size_t nk = ks.size();
    results.assign(rpms.size() * nk, ResultHost{});
    if (S.n_free <= 200) {   // dense path: per speed
        for (size_t g = 0; g < rpms.size(); g++) {
            prepare(c, rpms[g], false);
            std::vector<ResultHost> r;
            solve_set(c, ks, num_modes, min_frequency, precision, r);
            std::copy(r.begin(), r.end(), results.begin() + g * nk);
        }
        return;
    }
    const int n_extra = min_frequency > 0.0 ? 6 : 0;
    size_t g0 = 0;
    while (g0 < rpms.size()) {
        // the group: speeds after g0 with the pattern of g0 whose problems fit one batch
        prepare(c, rpms[g0], false);
        if (!c->symC.valid) { analyze_op(c->symC, c->opC); c->tune_choice = TuneCand{}; }
        if (!c->pairSym.valid) analyze_op(c->pairSym, c->pairOp);
        const std::string key = c->symC_key;
        std::vector<int> cks, rks;
        for (int k : ks) {
            const bool is_real = (k == 0) || (N % 2 == 0 && k == max_k);
            (is_real ? rks : cks).push_back(k);
        }
        if (c->autotune && c->tuned_key != c->symC_key && !cks.empty()) {
            // tune on this speed's complex harmonics before the group is sized
            const int Bt = (int)cks.size();
            std::vector<double> ph(2 * Bt);
            for (int p = 0; p < Bt; p++) { ph[2 * p] = std::cos(cks[p] * alpha); ph[2 * p + 1] = std::sin(cks[p] * alpha); }
            DVec<double> dph;
            dph.upload(ph);
            DVec<zd> tv;
            const int64_t nUt = c->opC.U.nnz();
            tv.alloc((size_t)Bt * std::max<int64_t>(1, nUt));
            if (nUt)
                TMG_LAUNCH(k_form_complex, dim3(nblk(nUt), Bt), 256, 0, st, nUt, c->opC.maps[0].p, c->opC.maps[1].p,
                           c->opC.maps[2].p, c->opC.maps[3].p, c->opC.maps[4].p, c->opC.maps[5].p, c->Kcf.sv.p,
                           c->Kpf.sv.p, c->Mcf.sv.p, c->Mpf.sv.p, dph.p, shift, tv.p);
            tune_complex(c, c->opC, tv.p, Bt, mixed);
        }
        int nev_c = 1, nev_r = 1;
        for (int k : cks) nev_c = std::max(nev_c, std::min((num_modes + 1) / 2 + n_extra, S.n_free - 1));
        for (int k : rks) nev_r = std::max(nev_r, std::min(num_modes + n_extra, S.n_free - 1));
        (void)nev_r;
        const int ncv_c = std::min(std::max(4 * nev_c + 1, 40), S.n_free);
        UnionMaps& um = c->opC;
        UnionMaps& mu = c->opMC;
        const int64_t nU = um.U.nnz(), nMU = mu.U.nnz();
        int per_speed = (int)cks.size();
        int bmax = per_speed ? batch_size(c, c->symC, um, mu.U.nnz(), ncv_c, true, mixed, 1 << 20) : 1 << 20;
        // value buffers of the group count against the same budget: one speed at least
        const int gmax = std::max(1, per_speed ? bmax / std::max(1, per_speed) : (int)rpms.size());
        std::vector<size_t> group{g0};
        for (size_t g = g0 + 1; g < rpms.size() && (int)group.size() < gmax; g++) {
            if ((rpms[g] == 0.0) != (rpms[g0] == 0.0)) break;   // rest and speed have different patterns
            group.push_back(g);
        }
        const int G = (int)group.size();
        const int Bc = G * per_speed, Br = G * (int)rks.size();
        DVec<zd> cvals, cm;
        DVec<double> rvals, rm;
        cvals.alloc((size_t)std::max(1, Bc) * std::max<int64_t>(nU, 1));
        cm.alloc((size_t)std::max(1, Bc) * std::max<int64_t>(nMU, 1));
        const int64_t rnU = c->pairOp.U.nnz(), rnM = c->pairM.U.nnz();
        rvals.alloc((size_t)std::max(1, Br) * std::max<int64_t>(rnU, 1));
        rm.alloc((size_t)std::max(1, Br) * std::max<int64_t>(rnM, 1));
        std::vector<Problem> cplx, real;
        for (int gi = 0; gi < G; gi++) {
            const size_t g = group[gi];
            if (gi > 0) prepare(c, rpms[g], false);
            if (c->symC_key != key) throw numeric_error("operator pattern changed inside a speed group");
            for (size_t q = 0; q < nk; q++) {
                const int k = ks[q];
                ResultHost& R = results[g * nk + q];
                R.k = k;
                R.rpm = rpms[g];
                Problem pr;
                pr.k = k;
                pr.P = zd{std::cos(k * alpha), std::sin(k * alpha)};
                pr.R = &R;
                pr.degenerate = (k > 0) && !(N % 2 == 0 && k == max_k);
                pr.nev_target = pr.degenerate ? (num_modes + 1) / 2 : num_modes;
                const bool is_real = (k == 0) || (N % 2 == 0 && k == max_k);
                if (!is_real) {
                    const int slot = (int)cplx.size();
                    DVec<double> dph;
                    dph.upload(std::vector<double>{pr.P.x, pr.P.y});
                    if (nU)
                        TMG_LAUNCH(k_form_complex, dim3(nblk(nU), 1), 256, 0, st, nU, um.maps[0].p, um.maps[1].p,
                                   um.maps[2].p, um.maps[3].p, um.maps[4].p, um.maps[5].p, c->Kcf.sv.p, c->Kpf.sv.p,
                                   c->Mcf.sv.p, c->Mpf.sv.p, dph.p, shift, cvals.p + (int64_t)slot * nU);
                    if (nMU) {
                        DVec<zd> mv;
                        mv.alloc(nMU);
                        TMG_LAUNCH(k_form_csum, dim3(nblk(nMU), 1), 256, 0, st, nMU, mu.maps[0].p, mu.maps[1].p,
                                   mu.maps[2].p, c->Mcf.sv.p, c->Mpf.sv.p, dph.p, mv.p);
                        TMG_LAUNCH(k_gather_b<zd>, dim3(nblk(nMU), 1), 256, 0, st, nMU, mu.csr2csc.p, mv.p, nMU,
                                   cm.p + (int64_t)slot * nMU, nMU);
                    }
                    TMG_CUDA(cudaStreamSynchronize(st));   // dph, mv are freed at scope end
                    cplx.push_back(pr);
                } else {
                    const auto& Rr = c->real[k == 0 ? 0 : 1];
                    if (!Rr.valid) { R.status = TMG_ERR_STATE; continue; }
                    const int slot = (int)real.size();
                    if (rnU)
                        TMG_LAUNCH(k_form_real_op, nblk(rnU), 256, 0, st, rnU, c->pairOp.maps[0].p, c->pairOp.maps[1].p,
                                   Rr.Ks.p, Rr.Ms.p, shift, 1.0, rvals.p + (int64_t)slot * rnU);
                    if (rnM) {
                        DVec<double> mc;
                        mc.alloc(rnM);
                        TMG_LAUNCH(k_form_real_op, nblk(rnM), 256, 0, st, rnM, c->pairM.maps[0].p, c->pairM.maps[0].p,
                                   Rr.Ms.p, Rr.Ms.p, 0.0, 1.0, mc.p);
                        TMG_LAUNCH(k_gather_b<double>, dim3(nblk(rnM), 1), 256, 0, st, rnM, c->pairM.csr2csc.p, mc.p,
                                   rnM, rm.p + (int64_t)slot * rnM, rnM);
                        TMG_CUDA(cudaStreamSynchronize(st));
                    }
                    real.push_back(pr);
                }
            }
        }
        // real harmonics of the group: one batch (problem stride rnU / rnM), run by a helper
        // thread on the context's second stream while this thread runs the complex batches
        // (both are latency-bound at these batch sizes, so their launches overlap on the device)
        auto real_batch = [&]() {
            const int nev = std::min(real[0].nev_target + n_extra, S.n_free - 1);
            const int ncv = std::min(std::max(4 * nev + 1, 40), S.n_free);
            DevCsr<double> M;
            M.nrows = S.n_free; M.nnz = rnM; M.rowptr = c->pairM.csr_rowptr.p; M.col = c->pairM.csr_col.p;
            M.val = rm.p; M.vstride = rnM;
            try {
                if (mixed)
                    run_batch<double, float>(c, real, c->pairSym, c->pairOp, rvals.p, M, nev, ncv, shift, 1000, true,
                                             num_modes, min_frequency);
                else
                    run_batch<double, double>(c, real, c->pairSym, c->pairOp, rvals.p, M, nev, ncv, shift, 1000, false,
                                              num_modes, min_frequency);
            } catch (const numeric_error& e) {
                for (auto& pr : real) pr.R->status = TMG_ERR_NUMERIC;
                note_err(c, e.what());
            }
            if (mixed) {
                std::vector<Problem> again = mixed_failures(c, real);
                if (!again.empty()) {
                    DVec<double> v2, m2;
                    v2.alloc((size_t)again.size() * rnU);
                    m2.alloc((size_t)again.size() * rnM);
                    for (size_t q = 0; q < again.size(); q++) {
                        size_t src = 0;
                        while (real[src].R != again[q].R) src++;
                        if (rnU) lz_copy<double>(g_stream, rnU, rvals.p + src * rnU, v2.p + q * rnU);
                        if (rnM) lz_copy<double>(g_stream, rnM, rm.p + src * rnM, m2.p + q * rnM);
                    }
                    DevCsr<double> M2 = M;
                    M2.val = m2.p;
                    try {
                        run_batch<double, double>(c, again, c->pairSym, c->pairOp, v2.p, M2, nev, ncv, shift, 1000,
                                                  false, num_modes, min_frequency);
                    } catch (const numeric_error& e) {
                        for (auto& pr : again) pr.R->status = TMG_ERR_NUMERIC;
                        note_err(c, e.what());
                    } catch (const cuda_error& e) {   // the FP64 factor does not fit: these problems fail alone
                        if (!std::strstr(e.what(), "out of memory")) throw;
                        for (auto& pr : again) pr.R->status = TMG_ERR_NOMEM;
                        note_err(c, std::string("FP64 retry of a mixed-path failure: ") + e.what());
                    }
                }
            }
        };
        std::thread helper;
        std::exception_ptr helper_err;
        int64_t helper_launches = 0;
        cudaEvent_t formed = nullptr;
        struct Join {   // the helper thread ends before anything it reads goes out of scope
            std::thread& t;
            cudaEvent_t& ev;
            ~Join() {
                if (t.joinable()) t.join();
                if (ev) cudaEventDestroy(ev);   // only after the helper waited on it
                ev = nullptr;
            }
        } join_helper{helper, formed};
        if (!real.empty()) {
            if (c->profile) {
                real_batch();
            } else {
                if (!c->st2) TMG_CUDA(cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking));
                if (!S.dcand_i.p) S.dcand_i.upload(S.cand.i);   // shared, read-only from here on
                TMG_CUDA(cudaEventCreateWithFlags(&formed, cudaEventDisableTiming));
                TMG_CUDA(cudaEventRecord(formed, st));
                const int dev = c->device;
                cudaStream_t st2 = c->st2;
                cudaEvent_t ready = formed;
                helper = std::thread([&, ready, dev, st2]() {
                    try {
                        TMG_CUDA(cudaSetDevice(dev));
                        g_stream = st2;
                        g_bytes = &c->bytes;
                        TMG_CUDA(cudaStreamWaitEvent(st2, ready, 0));
                        const int64_t l0 = g_kernel_launches;
                        real_batch();
                        helper_launches = g_kernel_launches - l0;
                        TMG_CUDA(cudaStreamSynchronize(st2));
                    } catch (...) {
                        helper_err = std::current_exception();
                    }
                    g_stream = nullptr;
                    g_bytes = nullptr;
                });
            }
        }

        // complex harmonics of the group, in batches of at most bmax problems
        for (size_t b0 = 0; b0 < cplx.size(); b0 += bmax) {
            std::vector<Problem> grp(cplx.begin() + b0, cplx.begin() + std::min(cplx.size(), b0 + (size_t)bmax));
            const int B = (int)grp.size();
            const int nev = std::min(grp[0].nev_target + n_extra, S.n_free - 1);
            const int ncv = std::min(std::max(4 * nev + 1, 40), S.n_free);
            DevCsr<zd> M;
            M.nrows = S.n_free; M.nnz = nMU; M.rowptr = mu.csr_rowptr.p; M.col = mu.csr_col.p;
            M.val = cm.p + (int64_t)b0 * nMU; M.vstride = nMU;
            const zd* vals = cvals.p + (int64_t)b0 * nU;
            DVec<zd> Wd;
            int md = 0;
            if (mixed && c->deflate && c->recycle_key == c->symC_key) {
                bool all = true;
                for (const Problem& pr : grp) {
                    auto it = c->recycle.find(pr.k);
                    all = all && it != c->recycle.end() && it->second.n == (size_t)S.n_free * DEFL_M;
                }
                if (all) {
                    const size_t nm = (size_t)S.n_free * DEFL_M;
                    Wd.alloc((size_t)B * nm);
                    for (int p = 0; p < B; p++)
                        TMG_CUDA(cudaMemcpyAsync(Wd.p + p * nm, c->recycle[grp[p].k].p, nm * sizeof(zd),
                                                 cudaMemcpyDeviceToDevice, st));
                    md = DEFL_M;
                }
            }
            try {
                if (mixed)
                    run_batch<zd, zf>(c, grp, c->symC, um, vals, M, nev, ncv, shift, 1000, true, num_modes,
                                      min_frequency, nullptr, false, md ? Wd.p : nullptr, md);
                else
                    run_batch<zd, zd>(c, grp, c->symC, um, vals, M, nev, ncv, shift, 1000, false, num_modes,
                                      min_frequency);
            } catch (const numeric_error& e) {
                for (auto& pr : grp) pr.R->status = TMG_ERR_NUMERIC;
                note_err(c, e.what());
            }
            if (mixed) {
                std::vector<Problem> again = mixed_failures(c, grp);
                if (!again.empty()) {
                    DVec<zd> v2, m2;
                    v2.alloc((size_t)again.size() * nU);
                    m2.alloc((size_t)again.size() * nMU);
                    for (size_t q = 0; q < again.size(); q++) {
                        size_t src = 0;
                        while (grp[src].R != again[q].R) src++;
                        if (nU) lz_copy<zd>(st, nU, vals + src * nU, v2.p + q * nU);
                        if (nMU) lz_copy<zd>(st, nMU, M.val + src * nMU, m2.p + q * nMU);
                    }
                    DevCsr<zd> M2 = M;
                    M2.val = m2.p;
                    try {
                        run_batch<zd, zd>(c, again, c->symC, um, v2.p, M2, nev, ncv, shift, 1000, false, num_modes,
                                          min_frequency);
                    } catch (const numeric_error& e) {
                        for (auto& pr : again) pr.R->status = TMG_ERR_NUMERIC;
                        note_err(c, e.what());
                    } catch (const cuda_error& e) {   // the FP64 factor does not fit: these problems fail alone
                        if (!std::strstr(e.what(), "out of memory")) throw;
                        for (auto& pr : again) pr.R->status = TMG_ERR_NOMEM;
                        note_err(c, std::string("FP64 retry of a mixed-path failure: ") + e.what());
                    }
                }
            }
        }
        if (helper.joinable()) helper.join();
        if (formed) { cudaEventDestroy(formed); formed = nullptr; }
        g_kernel_launches += helper_launches;
        if (helper_err) std::rethrow_exception(helper_err);
        g0 = group.back() + 1;
    }
    TMG_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

namespace {

int copy_csc(const Pattern& P, const double* dvals_or_null, const std::vector<double>* hvals, int64_t* nnz,
             int32_t* colptr, int32_t* rowidx, double* values, bool complex_out) {
    *nnz = P.nnz();
    if (!colptr) return TMG_OK;
    for (int32_t j = 0; j <= P.ncols; j++) colptr[j] = (int32_t)P.p[j];
    if (rowidx) std::copy(P.i.begin(), P.i.end(), rowidx);
    if (values) {
        std::vector<double> v;
        if (hvals) v = *hvals;
        else {
            v.resize(P.nnz());
            if (P.nnz()) {
                TMG_CUDA(cudaMemcpyAsync(v.data(), dvals_or_null, v.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                         g_stream));
                TMG_CUDA(cudaStreamSynchronize(g_stream));
            }
        }
        if (complex_out)
            for (int64_t q = 0; q < P.nnz(); q++) { values[2 * q] = v[q]; values[2 * q + 1] = 0.0; }
        else
            std::copy(v.begin(), v.end(), values);
    }
    return TMG_OK;
}

}  // namespace

// =====================================================================================
// C ABI
// =====================================================================================
extern "C" {

int tmg_create(int device, size_t mem_budget_bytes, tmg_context** out) {
    if (!out) return TMG_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return TMG_ERR_CUDA;
    auto* c = new tmg_context();
    c->device = device;
    // non-blocking stream: contexts driven from different host threads overlap on the device
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return TMG_ERR_CUDA;
    }
    {   // keep freed stream-ordered allocations in this process's pool instead of returning them
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    c->budget = mem_budget_bytes ? mem_budget_bytes : (size_t)(0.9 * (double)device_free_bytes(device));
    *out = c;
    return TMG_OK;
}

int tmg_set_memory_budget(tmg_context* c, size_t mem_budget_bytes) {
    if (!c) return TMG_ERR_ARG;
    return guarded(c, [&]() {
        c->budget = mem_budget_bytes ? mem_budget_bytes : (size_t)(0.9 * (double)device_free_bytes(c->device));
        return TMG_OK;
    });
}

int tmg_set_option(tmg_context* c, int option, double value) {
    if (!c) return TMG_ERR_ARG;
    switch (option) {
        case TMG_OPT_SHIFT:
            if (!std::isfinite(value)) return set_err(c, TMG_ERR_ARG, "shift must be finite");
            c->shift = value;
            return TMG_OK;
        case TMG_OPT_DEFLATE:
            c->deflate = value != 0.0;
            if (!c->deflate) c->recycle.clear();
            return TMG_OK;
        case TMG_OPT_TENSOR_CORES:
            c->tensor_cores = value != 0.0;
            return TMG_OK;
        case TMG_OPT_AUTOTUNE:
            c->autotune = value != 0.0;
            return TMG_OK;
        case TMG_OPT_REFINE_TOL:
            if (!(value >= 1e-14 && value <= 1e-6)) return set_err(c, TMG_ERR_ARG, "refinement target outside [1e-14, 1e-6]");
            c->refine_tol = value;
            return TMG_OK;
        default:
            return set_err(c, TMG_ERR_ARG, "unknown option " + std::to_string(option));
    }
}

int tmg_get_option(tmg_context* c, int option, double* value) {
    if (!c || !value) return TMG_ERR_ARG;
    switch (option) {
        case TMG_OPT_SHIFT: *value = c->shift; return TMG_OK;
        case TMG_OPT_DEFLATE: *value = c->deflate ? 1.0 : 0.0; return TMG_OK;
        case TMG_OPT_TENSOR_CORES: *value = c->tensor_cores ? 1.0 : 0.0; return TMG_OK;
        case TMG_OPT_AUTOTUNE: *value = c->autotune ? 1.0 : 0.0; return TMG_OK;
        case TMG_OPT_REFINE_TOL: *value = c->refine_tol; return TMG_OK;
        default: return set_err(c, TMG_ERR_ARG, "unknown option " + std::to_string(option));
    }
}

int tmg_destroy(tmg_context* c) {
    if (!c) return TMG_ERR_ARG;
    cudaSetDevice(c->device);
    cudaStream_t st = c->st, st2 = c->st2;
    g_stream = st;                     // the context's buffers are freed in its stream's order
    delete c;
    g_stream = nullptr;
    if (st2) {
        cudaStreamSynchronize(st2);
        cudaStreamDestroy(st2);
    }
    if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    return TMG_OK;
}

const char* tmg_last_error(const tmg_context* c) { return c ? c->err.c_str() : "null context"; }

int tmg_upload_sector(tmg_context* c, const tmg_sector_desc* d) {
    if (!c || !d) return TMG_ERR_ARG;
    return guarded(c, [&]() { setup_sector(c, d); return TMG_OK; });
}

int tmg_assemble(tmg_context* c, int which, double rpm, int64_t* nnz, int32_t* colptr, int32_t* rowidx, double* values) {
    if (!c || !nnz) return TMG_ERR_ARG;
    if (!c->sec) return set_err(c, TMG_ERR_STATE, "no sector uploaded");
    return guarded(c, [&]() {
        Sector& S = *c->sec;
        const double omega = rpm * 2.0 * PI / 60.0;
        const CandMat* m = nullptr;
        switch (which) {
            case TMG_MAT_K: assemble_KM(c); m = &c->K; break;
            case TMG_MAT_M: assemble_KM(c); m = &c->M; break;
            case TMG_MAT_KOMEGA: assemble_rot(c, omega); m = &c->Kw; break;
            case TMG_MAT_G: assemble_rot(c, omega); m = &c->G; break;
            case TMG_MAT_KSIGMA:
                if (!c->prepared || c->rpm != rpm) prepare(c, rpm, false);
                if (std::fabs(omega) == 0.0 || S.hub.empty()) return set_err(c, TMG_ERR_STATE, "no stress stiffening at this speed");
                m = &c->Ks; break;
            case TMG_MAT_KEFF:
                if (!c->prepared || c->rpm != rpm) prepare(c, rpm, false);
                m = &c->Keff; break;
            default: return set_err(c, TMG_ERR_ARG, "unknown matrix selector");
        }
        TMG_CUDA(cudaStreamSynchronize(c->st));
        Flagged f = flagged(S.cand, m->f.download());
        *nnz = f.pat.nnz();
        if (!colptr) return TMG_OK;
        std::vector<double> cv = m->v.download(), v(f.cand.size());
        for (size_t q = 0; q < f.cand.size(); q++) v[q] = cv[f.cand[q]];
        return copy_csc(f.pat, nullptr, &v, nnz, colptr, rowidx, values, false);
    });
}

int tmg_prepare(tmg_context* c, double rpm, int coriolis) {
    if (!c) return TMG_ERR_ARG;
    if (!c->sec) return set_err(c, TMG_ERR_STATE, "no sector uploaded");
    return guarded(c, [&]() { prepare(c, rpm, coriolis != 0); return TMG_OK; });
}

int tmg_projection(tmg_context* c, int which, int k, int64_t* nnz, int32_t* n, int32_t* colptr, int32_t* rowidx,
                   double* values) {
    if (!c || !nnz) return TMG_ERR_ARG;
    if (!c->prepared) return set_err(c, TMG_ERR_STATE, "call tmg_prepare first");
    return guarded(c, [&]() {
        Sector& S = *c->sec;
        if (n) *n = S.n_free;
        const FreeMat* fm = nullptr;
        bool cplx = true;
        switch (which) {
            case TMG_MAT_KCF: fm = &c->Kcf; break;
            case TMG_MAT_KPF: fm = &c->Kpf; break;
            case TMG_MAT_MCF: fm = &c->Mcf; break;
            case TMG_MAT_MPF: fm = &c->Mpf; break;
            case TMG_MAT_GCF: fm = &c->Gcf; break;
            case TMG_MAT_GPF: fm = &c->Gpf; break;
            case TMG_MAT_K0R: fm = &c->real[0].Kr; cplx = false; break;
            case TMG_MAT_M0R: fm = &c->real[0].Mr; cplx = false; break;
            case TMG_MAT_KHR: fm = &c->real[1].Kr; cplx = false; break;
            case TMG_MAT_MHR: fm = &c->real[1].Mr; cplx = false; break;
            case TMG_MAT_KK:
            case TMG_MAT_MK: {
                UnionMaps& w = which == TMG_MAT_KK ? c->W0 : c->WM0;
                const FreeMat& cc = which == TMG_MAT_KK ? c->Kcf : c->Mcf;
                const FreeMat& pp = which == TMG_MAT_KK ? c->Kpf : c->Mpf;
                const double alpha = 2.0 * PI / S.ns;
                DVec<zd> v;
                v.alloc(w.U.nnz());
                DVec<double> ph;
                ph.upload(std::vector<double>{std::cos(k * alpha), std::sin(k * alpha)});
                if (v.n)
                    TMG_LAUNCH(k_form_csum, dim3(nblk(v.n), 1), 256, 0, c->st, (int64_t)v.n, w.maps[0].p, w.maps[1].p,
                               w.maps[2].p, cc.sv.p, pp.sv.p, ph.p, v.p);
                TMG_CUDA(cudaStreamSynchronize(c->st));
                *nnz = w.U.nnz();
                if (!colptr) return TMG_OK;
                for (int32_t j = 0; j <= w.U.ncols; j++) colptr[j] = (int32_t)w.U.p[j];
                if (rowidx) std::copy(w.U.i.begin(), w.U.i.end(), rowidx);
                if (values && v.n) {
                    TMG_CUDA(cudaMemcpyAsync(values, v.p, v.n * sizeof(zd), cudaMemcpyDeviceToHost, c->st));
                    TMG_CUDA(cudaStreamSynchronize(c->st));
                }
                return TMG_OK;
            }
            case TMG_MAT_L1:
            case TMG_MAT_L2: {
                if (!c->coriolis) return set_err(c, TMG_ERR_STATE, "prepare with coriolis at a nonzero speed first");
                if (k <= 0 || k > S.ns / 2) return set_err(c, TMG_ERR_ARG, "the Coriolis QEP is solved for 0 < k <= N/2");
                ensure_qep(c);
                const auto& Q = c->qep;
                const UnionMaps *WK = &c->W0, *WM = &c->WM0, *WG = &c->WG0;
                const int64_t nK = WK->U.nnz(), nM = WM->U.nnz(), nG = WG->U.nnz(), nA = Q.op.U.nnz();
                const double alpha = 2.0 * PI / S.ns;
                DVec<double> ph, sig;
                ph.upload(std::vector<double>{std::cos(k * alpha), std::sin(k * alpha)});
                sig.upload(std::vector<double>{0.0});
                DVec<zd> Kv, Mv, Gv, v;
                Kv.alloc(std::max<int64_t>(1, nK)); Mv.alloc(std::max<int64_t>(1, nM)); Gv.alloc(std::max<int64_t>(1, nG));
                v.alloc(std::max<int64_t>(1, nA));
                if (nK) TMG_LAUNCH(k_form_csum, dim3(nblk(nK), 1), 256, 0, c->st, nK, WK->maps[0].p, WK->maps[1].p,
                                   WK->maps[2].p, c->Kcf.sv.p, c->Kpf.sv.p, ph.p, Kv.p);
                if (nM) TMG_LAUNCH(k_form_csum, dim3(nblk(nM), 1), 256, 0, c->st, nM, WM->maps[0].p, WM->maps[1].p,
                                   WM->maps[2].p, c->Mcf.sv.p, c->Mpf.sv.p, ph.p, Mv.p);
                if (nG) TMG_LAUNCH(k_form_csum, dim3(nblk(nG), 1), 256, 0, c->st, nG, WG->maps[0].p, WG->maps[1].p,
                                   WG->maps[2].p, c->Gcf.sv.p, c->Gpf.sv.p, ph.p, Gv.p);
                if (nA) TMG_LAUNCH(k_form_lancaster, dim3(nblk(nA), 1), 256, 0, c->st, nA, Q.sk.p, Q.sm.p, Q.sg.p,
                                   Q.blk.p, Kv.p, nK, Mv.p, nM, Gv.p, nG, 2.0 * (c->rpm * 2.0 * PI / 60.0), sig.p,
                                   which == TMG_MAT_L1 ? 1 : 2, v.p);
                TMG_CUDA(cudaStreamSynchronize(c->st));
                if (n) *n = Q.op.U.ncols;
                *nnz = nA;
                if (!colptr) return TMG_OK;
                for (int32_t j = 0; j <= Q.op.U.ncols; j++) colptr[j] = (int32_t)Q.op.U.p[j];
                if (rowidx) std::copy(Q.op.U.i.begin(), Q.op.U.i.end(), rowidx);
                if (values && nA) {
                    TMG_CUDA(cudaMemcpyAsync(values, v.p, nA * sizeof(zd), cudaMemcpyDeviceToHost, c->st));
                    TMG_CUDA(cudaStreamSynchronize(c->st));
                }
                return TMG_OK;
            }
            default: return set_err(c, TMG_ERR_ARG, "unknown projection selector");
        }
        TMG_CUDA(cudaStreamSynchronize(c->st));
        return copy_csc(fm->pat, fm->v.p, nullptr, nnz, colptr, rowidx, values, cplx);
    });
}

int tmg_symbolic(tmg_context* c, int kind, int32_t* n, int32_t* perm, int32_t* parent, int32_t* colcount) {
    if (!c || !n) return TMG_ERR_ARG;
    if (!c->prepared) return set_err(c, TMG_ERR_STATE, "call tmg_prepare first");
    return guarded(c, [&]() {
        // the analysis of the reference's operator pattern (pruned / filtered matrices)
        const Symbolic* sp = nullptr;
        if (kind == 0) {
            std::vector<int64_t> t1, t2;
            const Pattern kh = transpose_map(c->Kpf.pat, t1), mh = transpose_map(c->Mpf.pat, t2);
            const Pattern U = pattern_union({&c->Kcf.pat, &c->Kpf.pat, &kh, &c->Mcf.pat, &c->Mpf.pat, &mh});
            const std::string key = pattern_key(U);
            if (key != c->symRef_key[0]) {
                c->symRef[0] = analyze(lower_triangle(U), 0.0, 0);
                c->symRef_key[0] = key;
            }
            sp = &c->symRef[0];
        } else if (kind == 1 || kind == 2) {
            auto& RO = c->real[kind - 1];
            if (!RO.valid) return set_err(c, TMG_ERR_STATE, "no such real harmonic");
            const Pattern U = pattern_union({&RO.Kr.pat, &RO.Mr.pat});
            const std::string key = pattern_key(U);
            if (key != c->symRef_key[kind]) {
                c->symRef[kind] = analyze(lower_triangle(U), 0.0, 0);
                c->symRef_key[kind] = key;
            }
            sp = &c->symRef[kind];
        } else {
            return set_err(c, TMG_ERR_ARG, "unknown symbolic kind");
        }
        *n = sp->n;
        if (perm) std::copy(sp->amd.begin(), sp->amd.end(), perm);
        if (parent) std::copy(sp->etree.begin(), sp->etree.end(), parent);
        if (colcount) std::copy(sp->colcount.begin(), sp->colcount.end(), colcount);
        return TMG_OK;
    });
}

int tmg_symbolic_stats(tmg_context* c, int kind, double* out) {
    if (!c || !out) return TMG_ERR_ARG;
    if (!c->prepared) return set_err(c, TMG_ERR_STATE, "call tmg_prepare first");
    return guarded(c, [&]() {
        // the factorisation the solver runs (structural operator pattern)
        OpSymbolic* os = nullptr;
        if (kind == 0) {
            if (!c->symC.valid) analyze_op(c->symC, c->opC);
            os = &c->symC;
        } else if (kind == 1 || kind == 2) {
            if (!c->real[kind - 1].valid) return set_err(c, TMG_ERR_STATE, "no such real harmonic");
            if (!c->pairSym.valid) analyze_op(c->pairSym, c->pairOp);
            os = &c->pairSym;
        } else if (kind == 3) {
            if (!c->coriolis) return set_err(c, TMG_ERR_STATE, "prepare with coriolis at a nonzero speed first");
            ensure_qep(c);
            if (!c->qep.sym.valid) analyze_op(c->qep.sym, c->qep.op);
            os = &c->qep.sym;
        } else {
            return set_err(c, TMG_ERR_ARG, "unknown symbolic kind");
        }
        const Symbolic& S = os->S;
        out[0] = S.n; out[1] = (double)S.nnz_l; out[2] = S.ns; out[3] = (double)S.level_ptr.size() - 1;
        out[4] = S.max_front; out[5] = (double)os->D.l_entries; out[6] = 4.0 * S.flops_real;
        out[7] = (double)os->D.nlower; out[8] = (double)os->D.u_entries; out[9] = (double)os->D.l_stored;
        return TMG_OK;
    });
}

int tmg_solve_at_rpm(tmg_context* c, double rpm, int num_modes, const int32_t* harmonics, int nh, int coriolis,
                     double min_frequency, int precision, int32_t* num_results) {
    if (!c || !num_results) return TMG_ERR_ARG;
    if (!c->sec) return set_err(c, TMG_ERR_STATE, "no sector uploaded");
    if (num_modes <= 0) return set_err(c, TMG_ERR_ARG, "num_modes must be positive");
    return guarded(c, [&]() {
        for (double& p : c->phase_ms) p = 0.0;
        const int64_t l0 = g_kernel_launches;
        cudaEvent_t ev0, ev1;
        TMG_CUDA(cudaEventCreate(&ev0));
        TMG_CUDA(cudaEventCreate(&ev1));
        TMG_CUDA(cudaEventRecord(ev0, c->st));
        const bool cor = coriolis != 0;
        if (!c->prepared || c->rpm != rpm || c->coriolis != (cor && rpm != 0.0)) prepare(c, rpm, cor);
        Sector& S = *c->sec;
        const int max_k = S.ns / 2;
        std::vector<int> hs;
        if (!harmonics || nh == 0) for (int k = 0; k <= max_k; k++) hs.push_back(k);
        else for (int q = 0; q < nh; q++) if (harmonics[q] >= 0 && harmonics[q] <= max_k) hs.push_back(harmonics[q]);
        c->results.clear();
        c->err.clear();
        solve_set(c, hs, num_modes, min_frequency, precision, c->results);
        std::sort(c->results.begin(), c->results.end(), [](const ResultHost& a, const ResultHost& b) { return a.k < b.k; });
        *num_results = (int32_t)c->results.size();
        c->launches = g_kernel_launches - l0;
        TMG_CUDA(cudaEventRecord(ev1, c->st));
        TMG_CUDA(cudaEventSynchronize(ev1));
        float ms = 0.f;
        TMG_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        c->phase_ms[4] = ms;
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        return TMG_OK;
    });
}

int tmg_solve_sweep(tmg_context* c, const double* rpms, int nrpm, int num_modes, const int32_t* harmonics, int nh,
                    int coriolis, double min_frequency, int precision, int32_t* num_results) {
    if (!c || !num_results || (nrpm > 0 && !rpms) || nrpm < 0) return TMG_ERR_ARG;
    if (!c->sec) return set_err(c, TMG_ERR_STATE, "no sector uploaded");
    if (num_modes <= 0) return set_err(c, TMG_ERR_ARG, "num_modes must be positive");
    return guarded(c, [&]() {
        for (double& p : c->phase_ms) p = 0.0;
        const int64_t l0 = g_kernel_launches;
        cudaEvent_t ev0, ev1;
        TMG_CUDA(cudaEventCreate(&ev0));
        TMG_CUDA(cudaEventCreate(&ev1));
        TMG_CUDA(cudaEventRecord(ev0, c->st));
        Sector& S = *c->sec;
        const int max_k = S.ns / 2;
        std::vector<int> hs;
        if (!harmonics || nh == 0) for (int k = 0; k <= max_k; k++) hs.push_back(k);
        else for (int q = 0; q < nh; q++) if (harmonics[q] >= 0 && harmonics[q] <= max_k) hs.push_back(harmonics[q]);
        std::sort(hs.begin(), hs.end());
        hs.erase(std::unique(hs.begin(), hs.end()), hs.end());
        std::vector<double> rs(rpms, rpms + nrpm);
        c->results.clear();
        c->err.clear();
        if (coriolis) {   // the QEP keeps the per-speed path
            for (double rpm : rs) {
                prepare(c, rpm, true);
                std::vector<ResultHost> r;
                solve_set(c, hs, num_modes, min_frequency, precision, r);
                std::sort(r.begin(), r.end(), [](const ResultHost& a, const ResultHost& b) { return a.k < b.k; });
                c->results.insert(c->results.end(), r.begin(), r.end());
            }
        } else {
            solve_sweep(c, rs, hs, num_modes, min_frequency, precision, c->results);
        }
        *num_results = (int32_t)c->results.size();
        c->launches = g_kernel_launches - l0;
        TMG_CUDA(cudaEventRecord(ev1, c->st));
        TMG_CUDA(cudaEventSynchronize(ev1));
        float ms = 0.f;
        TMG_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        c->phase_ms[4] = ms;
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        return TMG_OK;
    });
}

int tmg_result_info(tmg_context* c, int idx, tmg_result_meta* info) {
    if (!c || !info || idx < 0 || idx >= (int)c->results.size()) return TMG_ERR_ARG;
    const ResultHost& R = c->results[idx];
    info->harmonic_index = R.k;
    info->num_modes = (int32_t)R.freqs.size();
    info->converged = R.converged;
    info->iterations = R.iterations;
    info->status = R.status;
    info->rpm = R.rpm;
    info->max_residual = R.max_residual;
    info->refine_residual = R.refine_residual;
    return TMG_OK;
}

int tmg_device_bytes(tmg_context* c, int64_t* current, int64_t* peak) {
    if (!c) return TMG_ERR_ARG;
    if (current) *current = c->bytes.cur.load();
    if (peak) *peak = c->bytes.peak.load();
    return TMG_OK;
}

int tmg_reset_peak_bytes(tmg_context* c) {
    if (!c) return TMG_ERR_ARG;
    c->bytes.peak.store(c->bytes.cur.load());
    return TMG_OK;
}

int tmg_tuning_report(tmg_context* c, double* out, int max_rows, int* rows) {
    if (!c || !rows) return TMG_ERR_ARG;
    *rows = (int)c->tune_rows.size();
    if (!out) return TMG_OK;
    for (int r = 0; r < std::min(max_rows, *rows); r++) {
        const TuneRow& t = c->tune_rows[r];
        const bool chosen = t.cand.relax == c->tune_choice.relax && t.cand.maxw == c->tune_choice.maxw &&
                            t.cand.tc_min == c->tune_choice.tc_min;
        double* o = out + (size_t)r * 9;
        o[0] = t.cand.relax; o[1] = t.cand.maxw; o[2] = t.cand.tc_min; o[3] = t.factor_ms; o[4] = t.solve_ms;
        o[5] = t.score_ms; o[6] = (double)t.stored; o[7] = t.supernodes; o[8] = chosen ? 1.0 : 0.0;
    }
    return TMG_OK;
}

int tmg_result_modal_mass(tmg_context* c, int idx, double* mass) {
    if (!c || !mass) return TMG_ERR_ARG;
    if (idx < 0 || idx >= (int)c->results.size()) return set_err(c, TMG_ERR_ARG, "result index out of range");
    const ResultHost& R = c->results[idx];
    if (R.modal_mass.size() != R.freqs.size()) return set_err(c, TMG_ERR_STATE, "no modal masses for this result");
    std::copy(R.modal_mass.begin(), R.modal_mass.end(), mass);
    return TMG_OK;
}

int tmg_result_copy(tmg_context* c, int idx, double* freqs, double* shapes, int32_t* whirl) {
    if (!c || idx < 0 || idx >= (int)c->results.size()) return TMG_ERR_ARG;
    const ResultHost& R = c->results[idx];
    if (freqs) std::copy(R.freqs.begin(), R.freqs.end(), freqs);
    if (whirl) std::copy(R.whirl.begin(), R.whirl.end(), whirl);
    if (shapes && !R.shapes.empty()) std::memcpy(shapes, R.shapes.data(), R.shapes.size() * sizeof(zd));
    return TMG_OK;
}

int tmg_set_profiling(tmg_context* c, int on) {
    if (!c) return TMG_ERR_ARG;
    c->profile = on != 0;
    c->solve_ms = 0.0;
    c->solve_bytes = 0.0;
    c->solve_count = 0;
    return TMG_OK;
}

int tmg_profile_solve(tmg_context* c, double* out) {
    if (!c || !out) return TMG_ERR_ARG;
    out[0] = (double)c->solve_count;
    out[1] = c->solve_ms;
    out[2] = c->solve_bytes;
    return TMG_OK;
}

int tmg_last_timing(tmg_context* c, double* phase_ms, int nphase, int64_t* kernel_launches) {
    if (!c) return TMG_ERR_ARG;
    for (int q = 0; q < nphase && q < 9; q++) phase_ms[q] = c->phase_ms[q];
    if (kernel_launches) *kernel_launches = c->launches;
    return TMG_OK;
}

}  // extern "C"

// ---- per-harmonic K_k / M_k without device allocation ---------------------------------
// tmg_projection forms K_k (or M_k) on the union pattern into a device buffer it allocates
// per call, then copies it to the caller.  This variant forms it into one file-scope device
// array instead, so the call performs no cudaMalloc / cudaFree and uploads nothing: the phase
// e^{ik alpha} travels as kernel arguments.  The arithmetic is the same as k_form_csum.
namespace {

__device__ __align__(256) double g_harmonic_scratch[2 * TMG_STATIC_SCRATCH_ENTRIES];

constexpr int kMaxScratchDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxScratchDevices] = {};

// Address of this device's copy of the scratch array, with the device current (the caller
// made it current).  It is looked up again on every call made outside a stream capture, so a
// primary context that was reset and re-created gets its new address; a call made while the
// stream is being captured uses the address recorded by the last call outside a capture.
zd* static_scratch(int device, cudaStream_t st) {
    if (device < 0 || device >= kMaxScratchDevices)
        throw std::invalid_argument("device ordinal beyond the static-scratch table");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) cs = cudaStreamCaptureStatusNone;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[device] || cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_harmonic_scratch);
        if (e != cudaSuccess)
            throw cuda_error(std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[device] = p;
    }
    return reinterpret_cast<zd*>(g_scratch_addr[device]);
}

__global__ void k_form_csum_static(int64_t n, const int64_t* __restrict__ ic, const int64_t* __restrict__ ip,
                                   const int64_t* __restrict__ ih, const double* __restrict__ c,
                                   const double* __restrict__ pv, double pre, double pim, zd* __restrict__ out) {
    const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const double a = ic[e] >= 0 ? c[ic[e]] : 0.0;
    const double b = ip[e] >= 0 ? pv[ip[e]] : 0.0;
    const double h = ih[e] >= 0 ? pv[ih[e]] : 0.0;
    const zd P{pre, pim}, Pc{pre, -pim};
    out[e] = (zd{a, 0.0} + P * zd{b, 0.0}) + Pc * zd{h, 0.0};
}

}  // namespace

extern "C" int tmg_projection_harmonic_static(tmg_context* c, int which, int k, int64_t* nnz, int32_t* n,
                                              int32_t* colptr, int32_t* rowidx, double* values) {
    if (!c || !nnz) return TMG_ERR_ARG;
    if (which != TMG_MAT_KK && which != TMG_MAT_MK)
        return set_err(c, TMG_ERR_ARG, "tmg_projection_harmonic_static forms TMG_MAT_KK or TMG_MAT_MK only");
    if (!c->prepared) return set_err(c, TMG_ERR_STATE, "call tmg_prepare first");
    return guarded(c, [&]() {
        Sector& S = *c->sec;
        const UnionMaps& w = which == TMG_MAT_KK ? c->W0 : c->WM0;
        const FreeMat& cc = which == TMG_MAT_KK ? c->Kcf : c->Mcf;
        const FreeMat& pp = which == TMG_MAT_KK ? c->Kpf : c->Mpf;
        const int64_t ne = w.U.nnz();
        if (n) *n = S.n_free;
        *nnz = ne;
        if (ne > (int64_t)TMG_STATIC_SCRATCH_ENTRIES)
            return set_err(c, TMG_ERR_ARG, "the harmonic matrix has " + std::to_string(ne) +
                                               " entries; the static scratch holds at most " +
                                               std::to_string((long long)TMG_STATIC_SCRATCH_ENTRIES) +
                                               " (use tmg_projection)");
        if (!colptr) return TMG_OK;
        zd* out = static_scratch(c->device, c->st);
        const double alpha = 2.0 * PI / S.ns;
        if (ne)
            TMG_LAUNCH(k_form_csum_static, nblk(ne), 256, 0, c->st, ne, w.maps[0].p, w.maps[1].p, w.maps[2].p, cc.sv.p,
                       pp.sv.p, std::cos(k * alpha), std::sin(k * alpha), out);
        TMG_CHECK_LAUNCH();
        for (int32_t j = 0; j <= w.U.ncols; j++) colptr[j] = (int32_t)w.U.p[j];
        if (rowidx) std::copy(w.U.i.begin(), w.U.i.end(), rowidx);
        if (values && ne)
            TMG_CUDA(cudaMemcpyAsync(values, out, (size_t)ne * sizeof(zd), cudaMemcpyDeviceToHost, c->st));
        TMG_CUDA(cudaStreamSynchronize(c->st));
        return TMG_OK;
    });
}
