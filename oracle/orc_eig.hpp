// Oracle (test infrastructure only): eigensolvers of the reference's modal path.
//   * Hermitian shift-invert Lanczos with full M-reorthogonalisation and implicit QR
//     restarts: src/hermitian_lanczos.cpp:114-460 (restated step by step);
//   * dense generalized Hermitian solve for n <= 200: src/hermitian_lanczos.cpp:68-110.
//     Eigen's GeneralizedSelfAdjointEigenSolver is restated as Cholesky reduction
//     C = L^-1 K L^-H, eigen-decomposition of C (real 2n x 2n embedding, Householder
//     tridiagonalisation + implicit QL, the public EISPACK tred2/tql2 algorithms), x = L^-H y;
//   * the small symmetric tridiagonal eigenproblem (Eigen SelfAdjointEigenSolver at
//     src/hermitian_lanczos.cpp:128,390): implicit QL (tql2), eigenvalues ascending.
//   * k = 0 and k = N/2 use Spectra::SymGEigsShiftSolver in the reference
//     (src/modal_solver.cpp:39-50).  Spectra is an un-vendored submodule; its published
//     algorithm (implicitly restarted Lanczos in shift-invert mode, B-inner product,
//     LargestMagn selection) is restated by running the same Lanczos as the complex path
//     on the real matrices.
#pragma once
#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "orc_amd.hpp"

namespace orc {

// JAMA/EISPACK tred2 + tql2 on a dense real symmetric matrix (row-major V in/out).
inline void sym_eig(int n, std::vector<double>& V, std::vector<double>& d) {
    std::vector<double> e(n, 0.0);
    d.assign(n, 0.0);
    auto A = [&](int i, int j) -> double& { return V[(size_t)i * n + j]; };
    for (int j = 0; j < n; j++) d[j] = A(n - 1, j);
    for (int i = n - 1; i > 0; i--) {
        double scale = 0.0, h = 0.0;
        for (int k = 0; k < i; k++) scale += std::fabs(d[k]);
        if (scale == 0.0) {
            e[i] = d[i - 1];
            for (int j = 0; j < i; j++) { d[j] = A(i - 1, j); A(i, j) = 0.0; A(j, i) = 0.0; }
        } else {
            for (int k = 0; k < i; k++) { d[k] /= scale; h += d[k] * d[k]; }
            double f = d[i - 1];
            double g = std::sqrt(h);
            if (f > 0) g = -g;
            e[i] = scale * g;
            h = h - f * g;
            d[i - 1] = f - g;
            for (int j = 0; j < i; j++) e[j] = 0.0;
            for (int j = 0; j < i; j++) {
                f = d[j];
                A(j, i) = f;
                g = e[j] + A(j, j) * f;
                for (int k = j + 1; k <= i - 1; k++) { g += A(k, j) * d[k]; e[k] += A(k, j) * f; }
                e[j] = g;
            }
            f = 0.0;
            for (int j = 0; j < i; j++) { e[j] /= h; f += e[j] * d[j]; }
            const double hh = f / (h + h);
            for (int j = 0; j < i; j++) e[j] -= hh * d[j];
            for (int j = 0; j < i; j++) {
                f = d[j]; g = e[j];
                for (int k = j; k <= i - 1; k++) A(k, j) -= (f * e[k] + g * d[k]);
                d[j] = A(i - 1, j);
                A(i, j) = 0.0;
            }
        }
        d[i] = h;
    }
    for (int i = 0; i < n - 1; i++) {
        A(n - 1, i) = A(i, i);
        A(i, i) = 1.0;
        const double h = d[i + 1];
        if (h != 0.0) {
            for (int k = 0; k <= i; k++) d[k] = A(k, i + 1) / h;
            for (int j = 0; j <= i; j++) {
                double g = 0.0;
                for (int k = 0; k <= i; k++) g += A(k, i + 1) * A(k, j);
                for (int k = 0; k <= i; k++) A(k, j) -= g * d[k];
            }
        }
        for (int k = 0; k <= i; k++) A(k, i + 1) = 0.0;
    }
    for (int j = 0; j < n; j++) { d[j] = A(n - 1, j); A(n - 1, j) = 0.0; }
    A(n - 1, n - 1) = 1.0;
    e[0] = 0.0;
    // tql2
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    double f = 0.0, tst1 = 0.0;
    const double eps = std::ldexp(1.0, -52);
    for (int l = 0; l < n; l++) {
        tst1 = std::max(tst1, std::fabs(d[l]) + std::fabs(e[l]));
        int m = l;
        while (m < n) {
            if (std::fabs(e[m]) <= eps * tst1) break;
            m++;
        }
        if (m > l) {
            int iter = 0;
            do {
                iter++;
                double g = d[l];
                double p = (d[l + 1] - g) / (2.0 * e[l]);
                double r = std::hypot(p, 1.0);
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < n; i++) d[i] -= h;
                f = f + h;
                p = d[m];
                double c = 1.0, c2 = c, c3 = c;
                const double el1 = e[l + 1];
                double s = 0.0, s2 = 0.0;
                for (int i = m - 1; i >= l; i--) {
                    c3 = c2; c2 = c; s2 = s;
                    g = c * e[i];
                    h = c * p;
                    r = std::hypot(p, e[i]);
                    e[i + 1] = s * r;
                    s = e[i] / r;
                    c = p / r;
                    p = c * d[i] - s * g;
                    d[i + 1] = h + s * (c * g + s * d[i]);
                    for (int k = 0; k < n; k++) {
                        h = A(k, i + 1);
                        A(k, i + 1) = s * A(k, i) + c * h;
                        A(k, i) = c * A(k, i) - s * h;
                    }
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (std::fabs(e[l]) > eps * tst1 && iter < 200);
        }
        d[l] = d[l] + f;
        e[l] = 0.0;
    }
    for (int i = 0; i < n - 1; i++) {
        int k = i;
        double p = d[i];
        for (int j = i + 1; j < n; j++)
            if (d[j] < p) { k = j; p = d[j]; }
        if (k != i) {
            d[k] = d[i];
            d[i] = p;
            for (int j = 0; j < n; j++) std::swap(A(j, i), A(j, k));
        }
    }
}

// Symmetric tridiagonal eigenproblem (alpha diagonal, beta[i] couples i and i+1):
// eigenvalues ascending in theta, eigenvectors column-major S[col*m + row].
inline void tridiag_eig(int m, const double* alpha, const double* beta, std::vector<double>& theta,
                        std::vector<double>& S) {
    std::vector<double> V((size_t)m * m, 0.0);
    for (int i = 0; i < m; i++) {
        V[(size_t)i * m + i] = alpha[i];
        if (i + 1 < m) { V[(size_t)i * m + i + 1] = beta[i]; V[(size_t)(i + 1) * m + i] = beta[i]; }
    }
    sym_eig(m, V, theta);
    S.assign((size_t)m * m, 0.0);
    for (int r = 0; r < m; r++)
        for (int c = 0; c < m; c++) S[(size_t)c * m + r] = V[(size_t)r * m + c];
}

template <typename T>
struct EigResult {
    std::vector<double> eigenvalues;
    std::vector<T> vectors;      // n x nconv column-major
    int nconv = 0;
    bool converged = false;
    std::string message;
    int restarts = 0, steps = 0;
};

template <typename T>
inline T dotc(int n, const T* a, const T* b) {  // a^H b
    T s = T(0);
    for (int i = 0; i < n; i++) s += conjv(a[i]) * b[i];
    return s;
}

// Dense generalized Hermitian eigenproblem K x = lambda M x (n <= 200 path).
template <typename T>
EigResult<T> solve_dense(const Csc<T>& K, const Csc<T>& M, int nev) {
    EigResult<T> res;
    const int n = K.rows;
    nev = std::min(nev, n);
    std::vector<cd> Kd((size_t)n * n, 0.0), Md((size_t)n * n, 0.0);  // row-major
    for (int j = 0; j < n; j++) {
        for (int q = K.p[j]; q < K.p[j + 1]; q++) Kd[(size_t)K.i[q] * n + j] += cd(K.x[q]);
        for (int q = M.p[j]; q < M.p[j + 1]; q++) Md[(size_t)M.i[q] * n + j] += cd(M.x[q]);
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= i; j++) {
            const cd kk = (Kd[(size_t)i * n + j] + std::conj(Kd[(size_t)j * n + i])) * 0.5;
            Kd[(size_t)i * n + j] = kk; Kd[(size_t)j * n + i] = std::conj(kk);
            const cd mm = (Md[(size_t)i * n + j] + std::conj(Md[(size_t)j * n + i])) * 0.5;
            Md[(size_t)i * n + j] = mm; Md[(size_t)j * n + i] = std::conj(mm);
        }
    // Cholesky M = L L^H (lower, row-major)
    std::vector<cd> L((size_t)n * n, 0.0);
    for (int j = 0; j < n; j++) {
        double s = std::real(Md[(size_t)j * n + j]);
        for (int k = 0; k < j; k++) s -= std::norm(L[(size_t)j * n + k]);
        if (!(s > 0.0)) { res.message = "Dense generalized eigensolver failed"; return res; }
        const double ljj = std::sqrt(s);
        L[(size_t)j * n + j] = ljj;
        for (int i = j + 1; i < n; i++) {
            cd t = Md[(size_t)i * n + j];
            for (int k = 0; k < j; k++) t -= L[(size_t)i * n + k] * std::conj(L[(size_t)j * n + k]);
            L[(size_t)i * n + j] = t / ljj;
        }
    }
    // C = L^-1 K L^-H : Y = L^-1 K (forward on columns), C = (L^-1 Y^H)^H
    std::vector<cd> Y(Kd);
    for (int c = 0; c < n; c++)
        for (int i = 0; i < n; i++) {
            cd t = Y[(size_t)i * n + c];
            for (int k = 0; k < i; k++) t -= L[(size_t)i * n + k] * Y[(size_t)k * n + c];
            Y[(size_t)i * n + c] = t / L[(size_t)i * n + i];
        }
    std::vector<cd> Z((size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) Z[(size_t)i * n + j] = std::conj(Y[(size_t)j * n + i]);
    for (int c = 0; c < n; c++)
        for (int i = 0; i < n; i++) {
            cd t = Z[(size_t)i * n + c];
            for (int k = 0; k < i; k++) t -= L[(size_t)i * n + k] * Z[(size_t)k * n + c];
            Z[(size_t)i * n + c] = t / L[(size_t)i * n + i];
        }
    // real embedding [[A, -B], [B, A]] of C = Z^H = A + iB
    const int n2 = 2 * n;
    std::vector<double> R((size_t)n2 * n2);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const cd cij = std::conj(Z[(size_t)j * n + i]);
            R[(size_t)i * n2 + j] = cij.real();
            R[(size_t)(i + n) * n2 + j + n] = cij.real();
            R[(size_t)i * n2 + j + n] = -cij.imag();
            R[(size_t)(i + n) * n2 + j] = cij.imag();
        }
    std::vector<double> ev;
    sym_eig(n2, R, ev);
    res.eigenvalues.resize(nev);
    res.vectors.assign((size_t)n * nev, T(0));
    std::vector<cd> y(n), x(n);
    for (int t = 0; t < nev; t++) {
        const int col = 2 * t;
        res.eigenvalues[t] = ev[col];
        for (int i = 0; i < n; i++) y[i] = cd(R[(size_t)i * n2 + col], R[(size_t)(i + n) * n2 + col]);
        double nrm = 0.0;
        for (int i = 0; i < n; i++) nrm += std::norm(y[i]);
        nrm = std::sqrt(nrm);
        for (int i = n - 1; i >= 0; i--) {  // x = L^-H y
            cd s = y[i] / nrm;
            for (int k = i + 1; k < n; k++) s -= std::conj(L[(size_t)k * n + i]) * x[k];
            x[i] = s / L[(size_t)i * n + i];
        }
        if constexpr (std::is_same<T, double>::value) {
            // a real problem's eigenvector comes out of the complex embedding with an arbitrary
            // phase (possibly purely imaginary): rotate its largest entry onto the real axis
            int im = 0;
            for (int i = 1; i < n; i++) if (std::abs(x[i]) > std::abs(x[im])) im = i;
            const cd ph = std::abs(x[im]) > 0.0 ? std::conj(x[im]) / std::abs(x[im]) : cd(1.0);
            for (int i = 0; i < n; i++) res.vectors[(size_t)t * n + i] = (x[i] * ph).real();
        } else {
            for (int i = 0; i < n; i++) res.vectors[(size_t)t * n + i] = x[i];
        }
    }
    res.nconv = nev;
    res.converged = true;
    res.message = "Dense solver";
    return res;
}

struct LanczosConfig {
    int nev = 20, ncv = 0;
    double shift = 0.0, tolerance = 1e-8;
    int max_iterations = 10;
};

template <typename T>
inline T rnd_entry(std::mt19937& gen, std::normal_distribution<double>& dist) {
    if constexpr (std::is_same<T, double>::value) {
        return dist(gen);
    } else {
        const double re = dist(gen);
        const double im = dist(gen);
        return cd(re, im);
    }
}

// src/hermitian_lanczos.cpp:114-260
template <typename T>
void implicit_restart(int n, std::vector<T>& V, std::vector<T>& MV, std::vector<double>& alpha,
                      std::vector<double>& beta, int nev, int ncv, const Csc<T>& M) {
    std::vector<double> ritz, S;
    tridiag_eig(ncv, alpha.data(), beta.data(), ritz, S);
    std::vector<int> ridx(ncv);
    std::iota(ridx.begin(), ridx.end(), 0);
    std::sort(ridx.begin(), ridx.end(), [&](int a, int b) { return ritz[a] < ritz[b]; });
    const int n_shifts = ncv - nev;
    std::vector<double> Q((size_t)ncv * ncv, 0.0);  // column-major
    for (int i = 0; i < ncv; i++) Q[(size_t)i * ncv + i] = 1.0;
    for (int s = 0; s < n_shifts; s++) {
        const double mu = ritz[ridx[s]];
        double x = alpha[0] - mu, z = beta[0];
        for (int i = 0; i < ncv - 1; i++) {
            const double r = std::hypot(x, z);
            double c, sn;
            if (r < 1e-300) { c = 1.0; sn = 0.0; } else { c = x / r; sn = z / r; }
            if (i > 0) beta[i - 1] = r;
            const double a0 = alpha[i], a1 = alpha[i + 1], b0 = beta[i];
            alpha[i] = c * c * a0 + 2.0 * c * sn * b0 + sn * sn * a1;
            alpha[i + 1] = sn * sn * a0 - 2.0 * c * sn * b0 + c * c * a1;
            beta[i] = c * sn * (a1 - a0) + (c * c - sn * sn) * b0;
            if (i + 2 < ncv) {
                const double bulge = sn * beta[i + 1];
                beta[i + 1] = c * beta[i + 1];
                x = beta[i];
                z = bulge;
            }
            for (int row = 0; row < ncv; row++) {
                const double q0 = Q[(size_t)i * ncv + row], q1 = Q[(size_t)(i + 1) * ncv + row];
                Q[(size_t)i * ncv + row] = c * q0 + sn * q1;
                Q[(size_t)(i + 1) * ncv + row] = -sn * q0 + c * q1;
            }
        }
    }
    const double beta_tridiag = beta[nev - 1];
    const double beta_dangling = beta[ncv - 1];
    std::vector<T> f(n, T(0));
    if (nev < ncv) {
        for (int i = 0; i < n; i++) {
            T s = T(0);
            for (int c = 0; c < ncv; c++) s += V[(size_t)c * n + i] * Q[(size_t)nev * ncv + c];
            f[i] = beta_tridiag * s + beta_dangling * Q[(size_t)(nev - 1) * ncv + ncv - 1] * V[(size_t)ncv * n + i];
        }
    }
    std::vector<T> Vn((size_t)n * nev);
    for (int c = 0; c < nev; c++)
        for (int i = 0; i < n; i++) {
            T s = T(0);
            for (int k = 0; k < ncv; k++) s += V[(size_t)k * n + i] * Q[(size_t)c * ncv + k];
            Vn[(size_t)c * n + i] = s;
        }
    std::copy(Vn.begin(), Vn.end(), V.begin());
    if (nev < ncv) {
        std::vector<T> Mf(n);
        spmv(M, f.data(), Mf.data());
        const double bnew = std::sqrt(std::fabs(std::real(cd(dotc(n, f.data(), Mf.data())))));
        if (bnew > 1e-14) {
            for (int i = 0; i < n; i++) {
                V[(size_t)nev * n + i] = f[i] / bnew;
                MV[(size_t)nev * n + i] = Mf[i] / bnew;
            }
            beta[nev - 1] = bnew;
        } else {
            beta[nev - 1] = 0.0;
        }
    }
    for (int j = 0; j < nev; j++) spmv(M, &V[(size_t)j * n], &MV[(size_t)j * n]);
}

// src/hermitian_lanczos.cpp:264-460 (factorisation by SimplicialLDL on the lower triangle of
// K - sigma M; the SparseLU fallback of :27-34 is not restated: a zero pivot is reported).
template <typename T>
EigResult<T> lanczos_solve(const Csc<T>& K, const Csc<T>& M, const LanczosConfig& cfg) {
    EigResult<T> result;
    const int n = K.rows;
    if (n == 0) { result.message = "Empty matrices"; return result; }
    const int nev = std::min(cfg.nev, n - 1);
    if (nev <= 0) { result.message = "System too small for requested number of eigenvalues"; return result; }
    if (n <= 200) return solve_dense(K, M, nev);
    int ncv = cfg.ncv;
    if (ncv <= 0) ncv = std::min(std::max(4 * nev + 1, 40), n);
    ncv = std::min(ncv, n);
    Csc<T> A = add<T>(K, T(1.0), M, T(-cfg.shift));
    SimplicialLDL<T> ldl;
    ldl.analyze(A);
    if (!ldl.factorize(A)) { result.message = "Factorization failed for shift-invert operator"; return result; }
    std::vector<T> V((size_t)n * (ncv + 1), T(0)), MV((size_t)n * (ncv + 1), T(0));
    std::vector<double> alpha(ncv, 0.0), beta(ncv, 0.0);
    {
        std::mt19937 gen(42);
        std::normal_distribution<double> dist(0.0, 1.0);
        for (int i = 0; i < n; i++) V[i] = rnd_entry<T>(gen, dist);
        std::vector<T> Mv0(n);
        spmv(M, V.data(), Mv0.data());
        const double mn = std::sqrt(std::real(cd(dotc(n, V.data(), Mv0.data()))));
        for (int i = 0; i < n; i++) { V[i] = V[i] / mn; MV[i] = Mv0[i] / mn; }
    }
    std::vector<T> w(n), Mw(n);
    const int max_restarts = cfg.max_iterations;
    for (int restart = 0; restart <= max_restarts; restart++) {
        const int j_start = (restart == 0) ? 0 : nev;
        for (int j = j_start; j < ncv; j++) {
            result.steps++;
            ldl.solve(&MV[(size_t)j * n], w.data());
            alpha[j] = std::real(cd(dotc(n, &MV[(size_t)j * n], w.data())));
            for (int i = 0; i < n; i++) w[i] -= alpha[j] * V[(size_t)j * n + i];
            if (j > 0)
                for (int i = 0; i < n; i++) w[i] -= beta[j - 1] * V[(size_t)(j - 1) * n + i];
            for (int k = 0; k <= j; k++) {
                const T h = dotc(n, &MV[(size_t)k * n], w.data());
                for (int i = 0; i < n; i++) w[i] -= h * V[(size_t)k * n + i];
            }
            spmv(M, w.data(), Mw.data());
            double bj = std::sqrt(std::fabs(std::real(cd(dotc(n, w.data(), Mw.data())))));
            if (bj < 1e-14) {
                std::mt19937 gen(42 + restart * 100 + j);
                std::normal_distribution<double> dist(0.0, 1.0);
                for (int i = 0; i < n; i++) w[i] = rnd_entry<T>(gen, dist);
                for (int k = 0; k <= j; k++) {
                    const T h = dotc(n, &MV[(size_t)k * n], w.data());
                    for (int i = 0; i < n; i++) w[i] -= h * V[(size_t)k * n + i];
                }
                spmv(M, w.data(), Mw.data());
                bj = std::sqrt(std::fabs(std::real(cd(dotc(n, w.data(), Mw.data())))));
                if (bj < 1e-14) { ncv = j + 1; break; }
            }
            beta[j] = bj;
            for (int i = 0; i < n; i++) {
                V[(size_t)(j + 1) * n + i] = w[i] / bj;
                MV[(size_t)(j + 1) * n + i] = Mw[i] / bj;
            }
        }
        const int m = std::min(ncv, n);
        std::vector<double> theta, S;
        tridiag_eig(m, alpha.data(), beta.data(), theta, S);
        std::vector<int> idx(m);
        std::iota(idx.begin(), idx.end(), 0);
        std::vector<double> lam(m);
        for (int i = 0; i < m; i++) lam[i] = std::fabs(theta[i]) > 1e-15 ? cfg.shift + 1.0 / theta[i] : 1e30;
        std::sort(idx.begin(), idx.end(), [&](int a, int b) { return lam[a] < lam[b]; });
        const double beta_last = (m > 0 && m - 1 < ncv) ? beta[m - 1] : 0.0;
        int nconv = 0;
        for (int i = 0; i < std::min(nev, m); i++) {
            const int ii = idx[i];
            const double resid = std::fabs(beta_last * S[(size_t)ii * m + m - 1]);
            if (resid < cfg.tolerance * std::max(1.0, std::fabs(theta[ii]))) nconv++;
        }
        if (nconv >= nev || restart == max_restarts) {
            int ne = std::min(nconv > 0 ? nconv : nev, m);
            ne = std::min(ne, nev);
            result.eigenvalues.resize(ne);
            result.vectors.assign((size_t)n * ne, T(0));
            for (int t = 0; t < ne; t++) {
                const int ii = idx[t];
                result.eigenvalues[t] = lam[ii];
                for (int c = 0; c < m; c++) {
                    const double s = S[(size_t)ii * m + c];
                    for (int i = 0; i < n; i++) result.vectors[(size_t)t * n + i] += V[(size_t)c * n + i] * s;
                }
            }
            result.nconv = ne;
            result.converged = nconv >= nev;
            result.restarts = restart;
            result.message = result.converged ? "Converged"
                : "Not all eigenvalues converged (" + std::to_string(nconv) + "/" + std::to_string(nev) +
                  ") after " + std::to_string(restart + 1) + " restarts";
            return result;
        }
        implicit_restart(n, V, MV, alpha, beta, nev, m, M);
    }
    result.message = "Unexpected exit from Lanczos loop";
    return result;
}

}  // namespace orc
