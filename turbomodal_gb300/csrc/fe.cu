// TET10 element kernels and sector assembly (FP64).
//
// One 128-thread CTA per element.  Per Gauss point the CTA builds J, det J, J^-1, the
// physical shape-function gradients and B^T D in shared memory; each thread then owns
// up to 8 of the 900 entries of the element matrix and accumulates them in registers.
// The arithmetic is the reference's (src/element.cpp:292-371, src/rotating_effects.cpp:5-226,
// src/assembler.cpp:102-110) written as explicit sums in a fixed order.  This file is
// compiled with --fmad=false, so every product and sum is a separate IEEE operation and
// the element matrices are reproducible bit for bit; that keeps the reference's
// value-dependent drop rule (|v| <= 1e-15 max|Ke|, src/assembler.cpp:274-289) exact.
//
// Assembly gathers element entries into the candidate sector pattern (node adjacency x
// 3x3 blocks) in element order, which is the order the reference's setFromTriplets sums
// duplicates in, and flags the candidates the reference pattern contains.
#include "common.cuh"
#include "fe.cuh"

namespace tmg {

__constant__ double c_gp14[14][3] = {
    {0.5, 0.5, 0.0}, {0.5, 0.0, 0.5}, {0.5, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.0, 0.5, 0.0}, {0.0, 0.0, 0.5},
    {0.100526765225204467, 0.100526765225204467, 0.100526765225204467},
    {0.698419704324386603, 0.100526765225204467, 0.100526765225204467},
    {0.100526765225204467, 0.698419704324386603, 0.100526765225204467},
    {0.100526765225204467, 0.100526765225204467, 0.698419704324386603},
    {0.314372873493192195, 0.314372873493192195, 0.314372873493192195},
    {0.0568813795204234229, 0.314372873493192195, 0.314372873493192195},
    {0.314372873493192195, 0.0568813795204234229, 0.314372873493192195},
    {0.314372873493192195, 0.314372873493192195, 0.0568813795204234229}};
__constant__ double c_gw14[14] = {
    0.00317460317460317503, 0.00317460317460317503, 0.00317460317460317503,
    0.00317460317460317503, 0.00317460317460317503, 0.00317460317460317503,
    0.01476497079049678, 0.01476497079049678, 0.01476497079049678, 0.01476497079049678,
    0.02213979111426512, 0.02213979111426512, 0.02213979111426512, 0.02213979111426512};
__constant__ double c_gp4[4][3] = {
    {0.1381966011250105, 0.1381966011250105, 0.1381966011250105},
    {0.5854101966249685, 0.1381966011250105, 0.1381966011250105},
    {0.1381966011250105, 0.5854101966249685, 0.1381966011250105},
    {0.1381966011250105, 0.1381966011250105, 0.5854101966249685}};

constexpr int EB = 128;                 // threads per element CTA
constexpr int EPT = (900 + EB - 1) / EB; // entries per thread

__device__ void d_shape_N(double xi, double eta, double zeta, double* N) {
    const double L1 = 1.0 - xi - eta - zeta, L2 = xi, L3 = eta, L4 = zeta;
    N[0] = L1 * (2.0 * L1 - 1.0); N[1] = L2 * (2.0 * L2 - 1.0);
    N[2] = L3 * (2.0 * L3 - 1.0); N[3] = L4 * (2.0 * L4 - 1.0);
    N[4] = 4.0 * L1 * L2; N[5] = 4.0 * L2 * L3; N[6] = 4.0 * L1 * L3;
    N[7] = 4.0 * L1 * L4; N[8] = 4.0 * L2 * L4; N[9] = 4.0 * L3 * L4;
}

__device__ void d_shape_dN(double xi, double eta, double zeta, double (*dN)[3]) {
    const double L1 = 1.0 - xi - eta - zeta, L2 = xi, L3 = eta, L4 = zeta;
    dN[0][0] = 1.0 - 4.0 * L1; dN[0][1] = 1.0 - 4.0 * L1; dN[0][2] = 1.0 - 4.0 * L1;
    dN[1][0] = 4.0 * L2 - 1.0; dN[1][1] = 0.0; dN[1][2] = 0.0;
    dN[2][0] = 0.0; dN[2][1] = 4.0 * L3 - 1.0; dN[2][2] = 0.0;
    dN[3][0] = 0.0; dN[3][1] = 0.0; dN[3][2] = 4.0 * L4 - 1.0;
    dN[4][0] = 4.0 * (L1 - L2); dN[4][1] = -4.0 * L2; dN[4][2] = -4.0 * L2;
    dN[5][0] = 4.0 * L3; dN[5][1] = 4.0 * L2; dN[5][2] = 0.0;
    dN[6][0] = -4.0 * L3; dN[6][1] = 4.0 * (L1 - L3); dN[6][2] = -4.0 * L3;
    dN[7][0] = -4.0 * L4; dN[7][1] = -4.0 * L4; dN[7][2] = 4.0 * (L1 - L4);
    dN[8][0] = 4.0 * L4; dN[8][1] = 0.0; dN[8][2] = 4.0 * L2;
    dN[9][0] = 0.0; dN[9][1] = 4.0 * L4; dN[9][2] = 4.0 * L3;
}

__device__ __forceinline__ double d_det3(const double (*J)[3]) {
    return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1])
         - J[1][0] * (J[0][1] * J[2][2] - J[0][2] * J[2][1])
         + J[2][0] * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
}

__device__ void d_inv3(const double (*J)[3], double det, double (*Ji)[3]) {
    const double inv = 1.0 / det;
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * inv;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * inv;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * inv;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * inv;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * inv;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * inv;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * inv;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * inv;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * inv;
}

struct ElemShared {
    double X[10][3];
    double N[10];
    double dN[10][3];
    double J[3][3];
    double Ji[3][3];
    double detJ, detJs, sc;
    double dNdx[10][3];
    double B[6][30];
    double T[30][6];
    double D[6][6];
    double ue[30];
    double sig[6];
    double eps[6];
    double red[EB];
    int bad;
};

__device__ void load_element(ElemShared& S, const double* __restrict__ X, const int32_t* __restrict__ conn,
                             int e) {
    const int t = threadIdx.x;
    if (t < 30) {
        const int a = t / 3, c = t % 3;
        const int nid = conn[(int64_t)e * 10 + a];
        S.X[a][c] = X[(int64_t)nid * 3 + c];
    }
}

// Per-point geometry shared by every kind: N, dN, J, signed det J, J^-1, dN/dx.
__device__ void point_geometry(ElemShared& S, const double* xi, bool need_inverse) {
    const int t = threadIdx.x;
    if (t == 0) {
        d_shape_N(xi[0], xi[1], xi[2], S.N);
        d_shape_dN(xi[0], xi[1], xi[2], S.dN);
    }
    __syncthreads();
    if (t < 9) {
        const int a = t / 3, b = t % 3;
        double s = 0.0;
        for (int i = 0; i < 10; i++) s += S.dN[i][a] * S.X[i][b];
        S.J[a][b] = s;
    }
    __syncthreads();
    if (t == 0) {
        S.detJs = d_det3(S.J);
        if (need_inverse) d_inv3(S.J, S.detJs, S.Ji);
    }
    __syncthreads();
    if (need_inverse && t < 30) {
        const int i = t / 3, a = t % 3;
        S.dNdx[i][a] = S.dN[i][0] * S.Ji[a][0] + S.dN[i][1] * S.Ji[a][1] + S.dN[i][2] * S.Ji[a][2];
    }
    __syncthreads();
}

// B matrix (6x30) from dN/dx, element.cpp:213-258
__device__ void build_B(ElemShared& S) {
    const int t = threadIdx.x;
    for (int q = t; q < 180; q += EB) S.B[q / 30][q % 30] = 0.0;
    __syncthreads();
    if (t < 10) {
        const int i = t, c = 3 * i;
        const double dx = S.dNdx[i][0], dy = S.dNdx[i][1], dz = S.dNdx[i][2];
        S.B[0][c] = dx; S.B[1][c + 1] = dy; S.B[2][c + 2] = dz;
        S.B[3][c] = dy; S.B[3][c + 1] = dx;
        S.B[4][c + 1] = dz; S.B[4][c + 2] = dy;
        S.B[5][c] = dz; S.B[5][c + 2] = dx;
    }
    __syncthreads();
}

__device__ double block_max(ElemShared& S, double v) {
    S.red[threadIdx.x] = v;
    __syncthreads();
    for (int s = EB / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) S.red[threadIdx.x] = fmax(S.red[threadIdx.x], S.red[threadIdx.x + s]);
        __syncthreads();
    }
    const double r = S.red[0];
    __syncthreads();
    return r;
}

// Apply the drop rule and store the element matrix (row-major 30x30).
__device__ void store_dropped(ElemShared& S, const double (&acc)[EPT], double* __restrict__ out, int e) {
    double mx = 0.0;
#pragma unroll
    for (int k = 0; k < EPT; k++) {
        const int idx = threadIdx.x + k * EB;
        if (idx < 900) mx = fmax(mx, fabs(acc[k]));
    }
    const double nrm = block_max(S, mx);
    const double tol = 1e-15 * nrm;
#pragma unroll
    for (int k = 0; k < EPT; k++) {
        const int idx = threadIdx.x + k * EB;
        if (idx < 900) out[(int64_t)e * 900 + idx] = fabs(acc[k]) > tol ? acc[k] : 0.0;
    }
}

// K and M: element.cpp:292-371
__global__ void __launch_bounds__(EB) k_elem_KM(int ne, const double* __restrict__ X,
                                                const int32_t* __restrict__ conn, double E, double nu,
                                                double rho, double* __restrict__ Ke, double* __restrict__ Me,
                                                int* __restrict__ neg_jac) {
    __shared__ ElemShared S;
    const int e = blockIdx.x;
    const int t = threadIdx.x;
    if (e >= ne) return;
    if (t == 0) {
        const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++) S.D[i][j] = 0.0;
        S.D[0][0] = S.D[1][1] = S.D[2][2] = c * (1.0 - nu);
        S.D[0][1] = S.D[0][2] = S.D[1][0] = S.D[1][2] = S.D[2][0] = S.D[2][1] = c * nu;
        S.D[3][3] = S.D[4][4] = S.D[5][5] = c * (1.0 - 2.0 * nu) / 2.0;
    }
    load_element(S, X, conn, e);
    __syncthreads();
    double ak[EPT], am[EPT];
#pragma unroll
    for (int k = 0; k < EPT; k++) { ak[k] = 0.0; am[k] = 0.0; }
    int neg = 0;
    for (int gp = 0; gp < 14; gp++) {
        point_geometry(S, c_gp14[gp], true);
        if (t == 0) {
            double detJ = S.detJs;
            if (detJ <= 0.0) { neg++; detJ = fabs(detJ); }
            S.detJ = detJ;
            S.sc = detJ * c_gw14[gp];
        }
        build_B(S);
        for (int q = t; q < 180; q += EB) {
            const int a = q / 6, qq = q % 6;
            double s = 0.0;
            for (int p = 0; p < 6; p++) s += S.B[p][a] * S.D[p][qq];
            S.T[a][qq] = s;
        }
        __syncthreads();
        const double sc = S.sc;
        const double scm = S.detJ * c_gw14[gp];
#pragma unroll
        for (int k = 0; k < EPT; k++) {
            const int idx = t + k * EB;
            if (idx < 900) {
                const int a = idx / 30, b = idx % 30;
                double s = 0.0;
                for (int q = 0; q < 6; q++) s += S.T[a][q] * S.B[q][b];
                ak[k] += s * sc;
                if (a % 3 == b % 3) am[k] += (rho * (S.N[a / 3] * S.N[b / 3])) * scm;
            }
        }
        __syncthreads();
    }
    if (t == 0 && neg) atomicAdd(neg_jac, neg);
    store_dropped(S, ak, Ke, e);
    store_dropped(S, am, Me, e);
}

// K_omega(omega) and G: rotating_effects.cpp:140-226 (signed det J)
__global__ void __launch_bounds__(EB) k_elem_rot(int ne, const double* __restrict__ X,
                                                 const int32_t* __restrict__ conn, double rho, double omega,
                                                 int axis, double* __restrict__ Kw, double* __restrict__ Ge) {
    __shared__ ElemShared S;
    const int e = blockIdx.x;
    const int t = threadIdx.x;
    if (e >= ne) return;
    load_element(S, X, conn, e);
    __syncthreads();
    double a3[3] = {0.0, 0.0, 0.0};
    a3[axis] = 1.0;
    const double o2 = omega * omega;
    double Om[3][3], Sk[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Om[r][c] = o2 * ((r == c ? 1.0 : 0.0) - a3[r] * a3[c]);
    Sk[0][0] = 0; Sk[0][1] = -a3[2]; Sk[0][2] = a3[1];
    Sk[1][0] = a3[2]; Sk[1][1] = 0; Sk[1][2] = -a3[0];
    Sk[2][0] = -a3[1]; Sk[2][1] = a3[0]; Sk[2][2] = 0;
    double aw[EPT], ag[EPT];
#pragma unroll
    for (int k = 0; k < EPT; k++) { aw[k] = 0.0; ag[k] = 0.0; }
    for (int gp = 0; gp < 14; gp++) {
        point_geometry(S, c_gp14[gp], false);
        const double sc = S.detJs * c_gw14[gp];
#pragma unroll
        for (int k = 0; k < EPT; k++) {
            const int idx = t + k * EB;
            if (idx < 900) {
                const int a = idx / 30, b = idx % 30;
                const double nn = rho * (S.N[a / 3] * S.N[b / 3]);
                aw[k] += (nn * Om[a % 3][b % 3]) * sc;
                ag[k] += (nn * Sk[a % 3][b % 3]) * sc;
            }
        }
        __syncthreads();
    }
    store_dropped(S, aw, Kw, e);
    store_dropped(S, ag, Ge, e);
}

// K_sigma from the static displacement: prestress at the 14 points (assembler.cpp:102-110)
// then sum B_NL^T S B_NL det J w (rotating_effects.cpp:53-138).
__global__ void __launch_bounds__(EB) k_elem_ksig(int ne, const double* __restrict__ X,
                                                  const int32_t* __restrict__ conn, double E, double nu,
                                                  const double* __restrict__ u, double* __restrict__ Ks,
                                                  int* __restrict__ bad) {
    __shared__ ElemShared S;
    __shared__ double sig14[14][6];
    const int e = blockIdx.x;
    const int t = threadIdx.x;
    if (e >= ne) return;
    if (t == 0) {
        const double c = E / ((1.0 + nu) * (1.0 - 2.0 * nu));
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < 6; j++) S.D[i][j] = 0.0;
        S.D[0][0] = S.D[1][1] = S.D[2][2] = c * (1.0 - nu);
        S.D[0][1] = S.D[0][2] = S.D[1][0] = S.D[1][2] = S.D[2][0] = S.D[2][1] = c * nu;
        S.D[3][3] = S.D[4][4] = S.D[5][5] = c * (1.0 - 2.0 * nu) / 2.0;
        S.bad = 0;
    }
    load_element(S, X, conn, e);
    if (t < 30) {
        const int a = t / 3, c = t % 3;
        S.ue[t] = u[(int64_t)conn[(int64_t)e * 10 + a] * 3 + c];
    }
    __syncthreads();
    for (int gp = 0; gp < 14; gp++) {
        point_geometry(S, c_gp14[gp], true);
        if (t == 0 && fabs(S.detJs) < 1e-30) S.bad = 1;
        build_B(S);
        if (t < 6) {
            double s = 0.0;
            for (int c = 0; c < 30; c++) s += S.B[t][c] * S.ue[c];
            S.eps[t] = s;
        }
        __syncthreads();
        if (t < 6) {
            double s = 0.0;
            for (int c = 0; c < 6; c++) s += S.D[t][c] * S.eps[c];
            sig14[gp][t] = s;
        }
        __syncthreads();
    }
    double acc[EPT];
#pragma unroll
    for (int k = 0; k < EPT; k++) acc[k] = 0.0;
    for (int gp = 0; gp < 14; gp++) {
        point_geometry(S, c_gp14[gp], true);
        const double sc = S.detJs * c_gw14[gp];
        const double* s = sig14[gp];
        const double sm[3][3] = {{s[0], s[3], s[5]}, {s[3], s[1], s[4]}, {s[5], s[4], s[2]}};
#pragma unroll
        for (int k = 0; k < EPT; k++) {
            const int idx = t + k * EB;
            if (idx < 900) {
                const int a = idx / 30, b = idx % 30;
                if (a % 3 == b % 3) {
                    const int i = a / 3, j = b / 3;
                    double tv[3];
                    for (int q = 0; q < 3; q++)
                        tv[q] = S.dNdx[i][0] * sm[0][q] + S.dNdx[i][1] * sm[1][q] + S.dNdx[i][2] * sm[2][q];
                    const double v = (tv[0] * S.dNdx[j][0] + tv[1] * S.dNdx[j][1] + tv[2] * S.dNdx[j][2]) * sc;
                    acc[k] += v;
                }
            }
        }
        __syncthreads();
    }
    if (t == 0 && S.bad) atomicExch(bad, 1);
    store_dropped(S, acc, Ks, e);
}

// Centrifugal element load, 4-point rule (rotating_effects.cpp:5-51)
__global__ void __launch_bounds__(EB) k_elem_fc(int ne, const double* __restrict__ X,
                                                const int32_t* __restrict__ conn, double rho, double omega,
                                                int axis, double* __restrict__ Fe) {
    __shared__ ElemShared S;
    const int e = blockIdx.x;
    const int t = threadIdx.x;
    if (e >= ne) return;
    load_element(S, X, conn, e);
    __syncthreads();
    double acc = 0.0;
    for (int gp = 0; gp < 4; gp++) {
        point_geometry(S, c_gp4[gp], false);
        const double sc = S.detJs * (1.0 / 24.0);
        if (t < 30) {
            const int i = t / 3, c = t % 3;
            double pos[3];
            for (int cc = 0; cc < 3; cc++) {
                double s = 0.0;
                for (int q = 0; q < 10; q++) s += S.X[q][cc] * S.N[q];
                pos[cc] = s;
            }
            double rp = pos[c];
            if (c == axis) rp = pos[c] - pos[c];
            const double f = rho * omega * omega;
            acc += (f * S.N[i] * rp) * sc;
        }
        __syncthreads();
    }
    if (t < 30) Fe[(int64_t)e * 30 + t] = acc;
}

// One thread per node pair: sums the 3x3 block of every contributing element in element
// order and flags the candidates the reference keeps (any kept contribution).
__global__ void k_gather_blocks(int64_t npairs, const int32_t* __restrict__ pair_col,
                                const int32_t* __restrict__ pair_pos, const int64_t* __restrict__ nadj_p,
                                const int64_t* __restrict__ cptr, const int32_t* __restrict__ clist,
                                const int64_t* __restrict__ cand_p, const double* __restrict__ Kel,
                                double* __restrict__ vals, uint8_t* __restrict__ flags) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= npairs) return;
    const int32_t nb = pair_col[q];
    const int32_t t = pair_pos[q];
    const int64_t deg = nadj_p[nb + 1] - nadj_p[nb];
    double acc[9];
    bool any[9];
#pragma unroll
    for (int k = 0; k < 9; k++) { acc[k] = 0.0; any[k] = false; }
    for (int64_t r = cptr[q]; r < cptr[q + 1]; r++) {
        const int32_t code = clist[r];
        const int32_t e = code / 100, la = (code / 10) % 10, lb = code % 10;
        const double* base = Kel + (int64_t)e * 900;
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const double v = base[(3 * la + c) * 30 + 3 * lb + d];
                acc[c * 3 + d] += v;
                any[c * 3 + d] |= (v != 0.0);
            }
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int64_t col0 = cand_p[3 * (int64_t)nb + d];
        (void)deg;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const int64_t s = col0 + 3 * (int64_t)t + c;
            vals[s] = acc[c * 3 + d];
            flags[s] = any[c * 3 + d] ? 1 : 0;
        }
    }
}

// F[3n+c] = sum over elements containing node n (element order) of Fe
__global__ void k_gather_load(int nn, const int64_t* __restrict__ nptr, const int32_t* __restrict__ nlist,
                              const double* __restrict__ Fe, double* __restrict__ F) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= 3 * (int64_t)nn) return;
    const int64_t node = q / 3;
    const int c = (int)(q % 3);
    double acc = 0.0;
    for (int64_t r = nptr[node]; r < nptr[node + 1]; r++) {
        const int32_t code = nlist[r];
        acc += Fe[(int64_t)(code / 10) * 30 + 3 * (code % 10) + c];
    }
    F[q] = acc;
}

// out = a*A + b*B + c*C on the candidate pattern (missing operands are exact zeros, as in
// the reference's sparse sums); flags OR-ed (union pattern).
__global__ void k_cand_axpy3(int64_t n, double a, const double* A, const uint8_t* fa, double b, const double* B,
                             const uint8_t* fb, double c, const double* Cv, const uint8_t* fc, double* out,
                             uint8_t* fout) {
    const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (q >= n) return;
    double v = a * A[q];
    uint8_t f = fa[q];
    if (B) { v = v + b * B[q]; f |= fb[q]; }
    if (Cv) { v = v + c * Cv[q]; f |= fc[q]; }
    out[q] = v;
    fout[q] = f;
}

void launch_elem_KM(cudaStream_t st, int ne, const double* X, const int32_t* conn, double E, double nu,
                    double rho, double* Ke, double* Me, int* neg) {
    if (ne == 0) return;
    TMG_LAUNCH(k_elem_KM, ne, EB, 0, st, ne, X, conn, E, nu, rho, Ke, Me, neg);
    TMG_CHECK_LAUNCH();
}
void launch_elem_rot(cudaStream_t st, int ne, const double* X, const int32_t* conn, double rho, double omega,
                     int axis, double* Kw, double* Ge) {
    if (ne == 0) return;
    TMG_LAUNCH(k_elem_rot, ne, EB, 0, st, ne, X, conn, rho, omega, axis, Kw, Ge);
    TMG_CHECK_LAUNCH();
}
void launch_elem_ksig(cudaStream_t st, int ne, const double* X, const int32_t* conn, double E, double nu,
                      const double* u, double* Ks, int* bad) {
    if (ne == 0) return;
    TMG_LAUNCH(k_elem_ksig, ne, EB, 0, st, ne, X, conn, E, nu, u, Ks, bad);
    TMG_CHECK_LAUNCH();
}
void launch_elem_fc(cudaStream_t st, int ne, const double* X, const int32_t* conn, double rho, double omega,
                    int axis, double* Fe) {
    if (ne == 0) return;
    TMG_LAUNCH(k_elem_fc, ne, EB, 0, st, ne, X, conn, rho, omega, axis, Fe);
    TMG_CHECK_LAUNCH();
}
void launch_gather_blocks(cudaStream_t st, int64_t npairs, const int32_t* pair_col, const int32_t* pair_pos,
                          const int64_t* nadj_p, const int64_t* cptr, const int32_t* clist, const int64_t* cand_p,
                          const double* Kel, double* vals, uint8_t* flags) {
    if (npairs == 0) return;
    TMG_LAUNCH(k_gather_blocks, (unsigned)ceil_div(npairs, 128), 128, 0, st, npairs, pair_col, pair_pos, nadj_p,
               cptr, clist, cand_p, Kel, vals, flags);
    TMG_CHECK_LAUNCH();
}
void launch_gather_load(cudaStream_t st, int nn, const int64_t* nptr, const int32_t* nlist, const double* Fe,
                        double* F) {
    if (nn == 0) return;
    TMG_LAUNCH(k_gather_load, (unsigned)ceil_div(3 * (int64_t)nn, 128), 128, 0, st, nn, nptr, nlist, Fe, F);
    TMG_CHECK_LAUNCH();
}
void launch_cand_axpy3(cudaStream_t st, int64_t n, double a, const double* A, const uint8_t* fa, double b,
                       const double* B, const uint8_t* fb, double c, const double* C, const uint8_t* fc,
                       double* out, uint8_t* fout) {
    if (n == 0) return;
    TMG_LAUNCH(k_cand_axpy3, (unsigned)ceil_div(n, 256), 256, 0, st, n, a, A, fa, b, B, fb, c, C, fc, out, fout);
    TMG_CHECK_LAUNCH();
}

}  // namespace tmg
