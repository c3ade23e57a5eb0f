// Oracle (test infrastructure only): CPU restatement of the reference's TET10 element
// kernels.  Only tests, the smoke check and the bench's CPU-baseline leg use this code.
//
// Follows src/element.cpp:13-371, src/rotating_effects.cpp:5-226, src/material.cpp:24-31.
// Every product is written as explicit loops in a fixed order; the library is built with
// -ffp-contract=off so each sum is a plain sequence of IEEE multiplies and adds.
#pragma once
#include <array>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace orc {

struct Mat { double E, nu, rho; };

// material.cpp:24-31
inline void constitutive(const Mat& m, double D[6][6]) {
    const double c = m.E / ((1.0 + m.nu) * (1.0 - 2.0 * m.nu));
    for (int i = 0; i < 6; i++) for (int j = 0; j < 6; j++) D[i][j] = 0.0;
    D[0][0] = D[1][1] = D[2][2] = c * (1.0 - m.nu);
    D[0][1] = D[0][2] = D[1][0] = D[1][2] = D[2][0] = D[2][1] = c * m.nu;
    D[3][3] = D[4][4] = D[5][5] = c * (1.0 - 2.0 * m.nu) / 2.0;
}

// element.cpp:13-21 (4-point rule) and :36-69 (Keast 14-point rule, weights include 1/6)
static const double GP4[4][3] = {
    {0.1381966011250105, 0.1381966011250105, 0.1381966011250105},
    {0.5854101966249685, 0.1381966011250105, 0.1381966011250105},
    {0.1381966011250105, 0.5854101966249685, 0.1381966011250105},
    {0.1381966011250105, 0.1381966011250105, 0.5854101966249685}};
static const double GW4 = 1.0 / 24.0;
static const double GP14[14][3] = {
    {0.5, 0.5, 0.0}, {0.5, 0.0, 0.5}, {0.5, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.0, 0.5, 0.0}, {0.0, 0.0, 0.5},
    {0.100526765225204467, 0.100526765225204467, 0.100526765225204467},
    {0.698419704324386603, 0.100526765225204467, 0.100526765225204467},
    {0.100526765225204467, 0.698419704324386603, 0.100526765225204467},
    {0.100526765225204467, 0.100526765225204467, 0.698419704324386603},
    {0.314372873493192195, 0.314372873493192195, 0.314372873493192195},
    {0.0568813795204234229, 0.314372873493192195, 0.314372873493192195},
    {0.314372873493192195, 0.0568813795204234229, 0.314372873493192195},
    {0.314372873493192195, 0.314372873493192195, 0.0568813795204234229}};
static const double GW14[14] = {
    0.00317460317460317503, 0.00317460317460317503, 0.00317460317460317503,
    0.00317460317460317503, 0.00317460317460317503, 0.00317460317460317503,
    0.01476497079049678, 0.01476497079049678, 0.01476497079049678, 0.01476497079049678,
    0.02213979111426512, 0.02213979111426512, 0.02213979111426512, 0.02213979111426512};

// element.cpp:90-112
inline void shape_N(double xi, double eta, double zeta, double N[10]) {
    const double L1 = 1.0 - xi - eta - zeta, L2 = xi, L3 = eta, L4 = zeta;
    N[0] = L1 * (2.0 * L1 - 1.0); N[1] = L2 * (2.0 * L2 - 1.0);
    N[2] = L3 * (2.0 * L3 - 1.0); N[3] = L4 * (2.0 * L4 - 1.0);
    N[4] = 4.0 * L1 * L2; N[5] = 4.0 * L2 * L3; N[6] = 4.0 * L1 * L3;
    N[7] = 4.0 * L1 * L4; N[8] = 4.0 * L2 * L4; N[9] = 4.0 * L3 * L4;
}

// element.cpp:114-201
inline void shape_dN(double xi, double eta, double zeta, double dN[10][3]) {
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

// J = dN^T X (element.cpp:203-211); J[a][b] = sum_i dN[i][a] * X[i][b]
inline void jacobian(const double dN[10][3], const double X[10][3], double J[3][3]) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            double s = 0.0;
            for (int i = 0; i < 10; i++) s += dN[i][a] * X[i][b];
            J[a][b] = s;
        }
}

// 3x3 determinant by first-column cofactor expansion (Eigen's 3x3 determinant form)
inline double det3(const double J[3][3]) {
    return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1])
         - J[1][0] * (J[0][1] * J[2][2] - J[0][2] * J[2][1])
         + J[2][0] * (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
}

// inverse = adjugate * (1/det); adjugate entry (i,j) = cofactor (j,i)
inline void inv3(const double J[3][3], double det, double Ji[3][3]) {
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

// dNdx = dNdxi * Jinv^T : dNdx[i][a] = sum_b dN[i][b] * Ji[a][b]
inline void phys_derivs(const double dN[10][3], const double Ji[3][3], double dNdx[10][3]) {
    for (int i = 0; i < 10; i++)
        for (int a = 0; a < 3; a++)
            dNdx[i][a] = dN[i][0] * Ji[a][0] + dN[i][1] * Ji[a][1] + dN[i][2] * Ji[a][2];
}

// B (6x30) per element.cpp:213-258 / :318-329
inline void bmat(const double dNdx[10][3], double B[6][30]) {
    for (int r = 0; r < 6; r++) for (int c = 0; c < 30; c++) B[r][c] = 0.0;
    for (int i = 0; i < 10; i++) {
        const double dx = dNdx[i][0], dy = dNdx[i][1], dz = dNdx[i][2];
        const int c = 3 * i;
        B[0][c] = dx; B[1][c + 1] = dy; B[2][c + 2] = dz;
        B[3][c] = dy; B[3][c + 1] = dx;
        B[4][c + 1] = dz; B[4][c + 2] = dy;
        B[5][c] = dz; B[5][c + 2] = dx;
    }
}

// Ke = sum_gp B^T D B (|detJ| w), element.cpp:292-335.  (B^T D) is formed first, then
// multiplied by B, then scaled: Ke[a][b] += (sum_q T[a][q] B[q][b]) * (detJ*w).
inline void stiffness(const double X[10][3], const Mat& m, double Ke[30][30], int* neg_jac = nullptr) {
    double D[6][6];
    constitutive(m, D);
    for (int a = 0; a < 30; a++) for (int b = 0; b < 30; b++) Ke[a][b] = 0.0;
    for (int gp = 0; gp < 14; gp++) {
        const double w = GW14[gp];
        double dN[10][3], J[3][3], Ji[3][3], dNdx[10][3], B[6][30];
        shape_dN(GP14[gp][0], GP14[gp][1], GP14[gp][2], dN);
        jacobian(dN, X, J);
        double detJ = det3(J);
        if (detJ <= 0.0) { if (neg_jac) (*neg_jac)++; detJ = std::fabs(detJ); }
        inv3(J, det3(J), Ji);
        phys_derivs(dN, Ji, dNdx);
        bmat(dNdx, B);
        double T[30][6];
        for (int a = 0; a < 30; a++)
            for (int q = 0; q < 6; q++) {
                double s = 0.0;
                for (int p = 0; p < 6; p++) s += B[p][a] * D[p][q];
                T[a][q] = s;
            }
        const double sc = detJ * w;
        for (int a = 0; a < 30; a++)
            for (int b = 0; b < 30; b++) {
                double s = 0.0;
                for (int q = 0; q < 6; q++) s += T[a][q] * B[q][b];
                Ke[a][b] += s * sc;
            }
    }
}

// Me = sum_gp rho N^T N (|detJ| w), element.cpp:337-371: only same-component entries are
// nonzero; Me[3i+c][3j+c] += (rho * (N_i * N_j)) * (detJ * w).
inline void mass(const double X[10][3], const Mat& m, double Me[30][30]) {
    for (int a = 0; a < 30; a++) for (int b = 0; b < 30; b++) Me[a][b] = 0.0;
    for (int gp = 0; gp < 14; gp++) {
        const double w = GW14[gp];
        double N[10], dN[10][3], J[3][3];
        shape_N(GP14[gp][0], GP14[gp][1], GP14[gp][2], N);
        shape_dN(GP14[gp][0], GP14[gp][1], GP14[gp][2], dN);
        jacobian(dN, X, J);
        double detJ = det3(J);
        if (detJ <= 0.0) detJ = std::fabs(detJ);
        const double sc = detJ * w;
        for (int i = 0; i < 10; i++)
            for (int j = 0; j < 10; j++) {
                const double v = (m.rho * (N[i] * N[j])) * sc;
                for (int c = 0; c < 3; c++) Me[3 * i + c][3 * j + c] += v;
            }
    }
}

// Kw = sum_gp rho N^T [omega^2 (I - a a^T)] N detJ w  (signed detJ), rotating_effects.cpp:140-179
inline void spin_softening(const double X[10][3], const Mat& m, double omega, int axis, double Kw[30][30]) {
    double a[3] = {0, 0, 0};
    a[axis] = 1.0;
    const double o2 = omega * omega;
    double Om[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Om[r][c] = o2 * ((r == c ? 1.0 : 0.0) - a[r] * a[c]);
    for (int p = 0; p < 30; p++) for (int q = 0; q < 30; q++) Kw[p][q] = 0.0;
    for (int gp = 0; gp < 14; gp++) {
        const double w = GW14[gp];
        double N[10], dN[10][3], J[3][3];
        shape_N(GP14[gp][0], GP14[gp][1], GP14[gp][2], N);
        shape_dN(GP14[gp][0], GP14[gp][1], GP14[gp][2], dN);
        jacobian(dN, X, J);
        const double sc = det3(J) * w;
        for (int i = 0; i < 10; i++)
            for (int j = 0; j < 10; j++) {
                const double nn = m.rho * (N[i] * N[j]);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) Kw[3 * i + r][3 * j + c] += (nn * Om[r][c]) * sc;
            }
    }
}

// G = sum_gp rho N^T [a x] N detJ w (skew, no 2*omega), rotating_effects.cpp:181-226
inline void gyroscopic(const double X[10][3], const Mat& m, int axis, double Ge[30][30]) {
    double a[3] = {0, 0, 0};
    a[axis] = 1.0;
    const double S[3][3] = {{0, -a[2], a[1]}, {a[2], 0, -a[0]}, {-a[1], a[0], 0}};
    for (int p = 0; p < 30; p++) for (int q = 0; q < 30; q++) Ge[p][q] = 0.0;
    for (int gp = 0; gp < 14; gp++) {
        const double w = GW14[gp];
        double N[10], dN[10][3], J[3][3];
        shape_N(GP14[gp][0], GP14[gp][1], GP14[gp][2], N);
        shape_dN(GP14[gp][0], GP14[gp][1], GP14[gp][2], dN);
        jacobian(dN, X, J);
        const double sc = det3(J) * w;
        for (int i = 0; i < 10; i++)
            for (int j = 0; j < 10; j++) {
                const double nn = m.rho * (N[i] * N[j]);
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) Ge[3 * i + r][3 * j + c] += (nn * S[r][c]) * sc;
            }
    }
}

// Fe = sum_{4 gp} rho omega^2 N^T r_perp detJ w (signed detJ), rotating_effects.cpp:5-51
inline void centrifugal(const double X[10][3], const Mat& m, double omega, int axis, double Fe[30]) {
    for (int p = 0; p < 30; p++) Fe[p] = 0.0;
    for (int gp = 0; gp < 4; gp++) {
        double N[10], dN[10][3], J[3][3];
        shape_N(GP4[gp][0], GP4[gp][1], GP4[gp][2], N);
        shape_dN(GP4[gp][0], GP4[gp][1], GP4[gp][2], dN);
        jacobian(dN, X, J);
        const double sc = det3(J) * GW4;
        double pos[3];
        for (int c = 0; c < 3; c++) {
            double s = 0.0;
            for (int i = 0; i < 10; i++) s += X[i][c] * N[i];
            pos[c] = s;
        }
        double rp[3] = {pos[0], pos[1], pos[2]};
        rp[axis] = pos[axis] - pos[axis];      // r_perp = pos - (pos.a) a with a a unit axis
        const double f = m.rho * omega * omega;
        for (int i = 0; i < 10; i++)
            for (int c = 0; c < 3; c++) Fe[3 * i + c] += (f * N[i] * rp[c]) * sc;
    }
}

// Prestress at the 14 points: sigma = D (B u_e), B recomputed per point and throwing on
// |detJ| < 1e-30 (assembler.cpp:102-110, element.cpp:213-222).
inline void prestress14(const double X[10][3], const Mat& m, const double ue[30], double sig[14][6]) {
    double D[6][6];
    constitutive(m, D);
    for (int gp = 0; gp < 14; gp++) {
        double dN[10][3], J[3][3], Ji[3][3], dNdx[10][3], B[6][30];
        shape_dN(GP14[gp][0], GP14[gp][1], GP14[gp][2], dN);
        jacobian(dN, X, J);
        const double detJ = det3(J);
        if (std::fabs(detJ) < 1e-30) throw std::runtime_error("TET10::B_matrix: singular Jacobian");
        inv3(J, detJ, Ji);
        phys_derivs(dN, Ji, dNdx);
        bmat(dNdx, B);
        double eps[6];
        for (int r = 0; r < 6; r++) {
            double s = 0.0;
            for (int c = 0; c < 30; c++) s += B[r][c] * ue[c];
            eps[r] = s;
        }
        for (int r = 0; r < 6; r++) {
            double s = 0.0;
            for (int c = 0; c < 6; c++) s += D[r][c] * eps[c];
            sig[gp][r] = s;
        }
    }
}

// Ks = sum_gp B_NL^T S B_NL detJ w (signed detJ), rotating_effects.cpp:53-138.  Only
// same-component blocks are nonzero: Ks[3i+c][3j+c] += (g_i^T sigma g_j) * (detJ w),
// g_i = grad N_i.
inline void stress_stiffening(const double X[10][3], const double sig[14][6], double Ks[30][30]) {
    for (int p = 0; p < 30; p++) for (int q = 0; q < 30; q++) Ks[p][q] = 0.0;
    for (int gp = 0; gp < 14; gp++) {
        const double w = GW14[gp];
        double dN[10][3], J[3][3], Ji[3][3], dNdx[10][3];
        shape_dN(GP14[gp][0], GP14[gp][1], GP14[gp][2], dN);
        jacobian(dN, X, J);
        const double detJ = det3(J);
        inv3(J, detJ, Ji);
        phys_derivs(dN, Ji, dNdx);
        const double* s = sig[gp];
        const double sm[3][3] = {{s[0], s[3], s[5]}, {s[3], s[1], s[4]}, {s[5], s[4], s[2]}};
        const double sc = detJ * w;
        for (int i = 0; i < 10; i++) {
            double t[3];
            for (int b = 0; b < 3; b++)
                t[b] = dNdx[i][0] * sm[0][b] + dNdx[i][1] * sm[1][b] + dNdx[i][2] * sm[2][b];
            for (int j = 0; j < 10; j++) {
                const double v = (t[0] * dNdx[j][0] + t[1] * dNdx[j][1] + t[2] * dNdx[j][2]) * sc;
                for (int c = 0; c < 3; c++) Ks[3 * i + c][3 * j + c] += v;
            }
        }
    }
}

}  // namespace orc
