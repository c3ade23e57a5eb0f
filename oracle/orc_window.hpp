// Oracle (test infrastructure only): timing samples of the reference's shift-invert
// factorisation on a full-size operator, for the bench's CPU baseline and reference arm.
//
// The reference factorises K_k - sigma M_k with Eigen's SimplicialLDLT<..., Lower>
// (src/hermitian_lanczos.cpp:12-56), an up-looking LDL^H that computes row k of L from the
// columns of L finished so far (SimplicialLDL::factorize in orc_amd.hpp restates it).  On the
// config-1 operator one factorisation takes tens of minutes on one core, so the bench cannot
// run it whole.  What the loop does at row k (which columns it visits, how many entries of
// each it updates) depends only on the sparsity structure of L, which the symbolic analysis
// gives in full.  LdlWindows therefore:
//   1. analyses the operator as SimplicialLDL does (Eigen's AMD order, etree, column counts)
//      and writes the complete row structure of L (the row indices the numeric loop would
//      append), with the loop's work per row;
//   2. times the numeric loop of factorize() on a window of rows [a, b) with the columns of
//      L already holding their entries of rows < a (their values are zero and D = 1 there:
//      the arithmetic done per entry is the same for any finite values);
//   3. times one solve (forward and backward sweep over all of L) as SimplicialLDL::solve.
// Each slot holds its own L values and work vectors, so several slots run concurrently on
// separate threads the way the reference's thread pool runs one harmonic per thread
// (src/cyclic_solver.cpp:1226-1332).
#pragma once
#include <algorithm>
#include <chrono>
#include <thread>

#include "orc_amd.hpp"

namespace orc {

struct LdlWindows {
    using T = cd;
    int n = 0;
    SimplicialLDL<T> S;                // order, etree, column pointers (slot 0's analysis)
    std::vector<int> Li;               // complete row structure of L (rows ascending per column)
    std::vector<int64_t> cum;          // cum[k] = inner-loop updates of rows < k
    struct Slot {
        std::vector<T> Lx, y;
        std::vector<double> D;
        std::vector<int> pattern, tags, nzc;
    };
    std::vector<Slot> slots;

    void analyze(const Csc<T>& A) {
        S.analyze(A);
        n = S.n;
        std::vector<T>().swap(S.Lx);   // values live in the slots
        Li.assign((size_t)S.Lp[n], 0);
        cum.assign((size_t)n + 1, 0);
        std::vector<int> nzc(n, 0), tags(n, -1), pattern(n);
        const Csc<T>& ap = S.ap;
        for (int k = 0; k < n; k++) {
            int top = n;
            tags[k] = k;
            for (int q = ap.p[k]; q < ap.p[k + 1]; q++) {
                int i = ap.i[q];
                if (i <= k) {
                    int len;
                    for (len = 0; tags[i] != k; i = S.parent[i]) {
                        pattern[len++] = i;
                        tags[i] = k;
                    }
                    while (len > 0) pattern[--top] = pattern[--len];
                }
            }
            int64_t w = 0;
            for (; top < n; ++top) {
                const int i = pattern[top];
                w += nzc[i] + 1;
                Li[(size_t)S.Lp[i] + nzc[i]] = k;
                ++nzc[i];
            }
            cum[k + 1] = cum[k] + w;
        }
        add_slot();
    }

    // One more slot: its own L values and work vectors over the analysed operator.  The
    // reference's threads hold one harmonic each, all with this pattern; the loop's work does
    // not depend on the values, so the slots share the operator (read only).
    void add_slot() {
        Slot s;
        s.Lx.assign((size_t)S.Lp[n], T(0));
        s.y.assign(n, T(0));
        s.D.assign(n, 1.0);
        s.pattern.assign(n, 0);
        s.tags.assign(n, -1);
        s.nzc.assign(n, 0);
        slots.push_back(std::move(s));
    }

    int64_t nnz_l() const { return S.Lp[n]; }

    // entries of column i with row < r
    int below(int i, int r) const {
        const int* b = Li.data() + S.Lp[i];
        const int* e = Li.data() + S.Lp[i + 1];
        return (int)(std::lower_bound(b, e, r) - b);
    }

    // Seconds of the numeric loop of SimplicialLDL::factorize over rows [a, b) on slot sl.
    double time_window(int sl, int a, int b) {
        Slot& s = slots[sl];
        for (int i = 0; i < n; i++) {
            s.nzc[i] = i < a ? below(i, a) : 0;
            s.tags[i] = -1;
            s.D[i] = 1.0;
        }
        const Csc<T>& ap = S.ap;
        std::vector<T>& y = s.y;
        std::vector<int>& pattern = s.pattern;
        std::vector<int>& tags = s.tags;
        std::vector<int>& nzc = s.nzc;
        std::vector<T>& Lx = s.Lx;
        std::vector<double>& D = s.D;
        const std::vector<int>& Lp = S.Lp;
        const std::vector<int>& parent = S.parent;
        const auto t0 = std::chrono::steady_clock::now();
        for (int k = a; k < b; k++) {
            y[k] = T(0);
            int top = n;
            tags[k] = k;
            nzc[k] = 0;
            for (int q = ap.p[k]; q < ap.p[k + 1]; q++) {
                int i = ap.i[q];
                if (i <= k) {
                    y[i] += conjv(ap.x[q]);
                    int len;
                    for (len = 0; tags[i] != k; i = parent[i]) {
                        pattern[len++] = i;
                        tags[i] = k;
                    }
                    while (len > 0) pattern[--top] = pattern[--len];
                }
            }
            double d = std::real(cd(y[k]));
            y[k] = T(0);
            for (; top < n; ++top) {
                const int i = pattern[top];
                const T yi = y[i];
                y[i] = T(0);
                const T l_ki = yi / D[i];
                const int p2 = Lp[i] + nzc[i];
                int p;
                for (p = Lp[i]; p < p2; ++p) y[Li[p]] -= conjv(Lx[p]) * yi;
                d -= std::real(cd(l_ki * conjv(yi)));
                Lx[p] = l_ki;          // Li[p] == k already (complete structure)
                ++nzc[i];
            }
            D[k] = d != 0.0 ? d : 1.0;
        }
        const auto t1 = std::chrono::steady_clock::now();
        for (int i = 0; i < std::min(b, n); i++) {   // back to zero values for the next sample
            const int lo = i < a ? below(i, a) : 0, hi = below(i, b);
            std::fill(Lx.begin() + Lp[i] + lo, Lx.begin() + Lp[i] + hi, T(0));
        }
        return std::chrono::duration<double>(t1 - t0).count();
    }

    // Seconds of one solve over all of L (the sweeps of SimplicialLDL::solve) on slot sl.
    double time_solve(int sl) {
        Slot& s = slots[sl];
        std::vector<T> b(n, T(1)), x(n);
        std::vector<T> z(n);
        const auto t0 = std::chrono::steady_clock::now();
        for (int i = 0; i < n; i++) z[S.P[i]] = b[i];
        for (int j = 0; j < n; j++) {
            const T zj = z[j];
            for (int q = S.Lp[j]; q < S.Lp[j + 1]; q++) z[Li[q]] -= s.Lx[q] * zj;
        }
        for (int j = 0; j < n; j++) z[j] = z[j] / s.D[j];
        for (int j = n - 1; j >= 0; j--) {
            T acc = z[j];
            for (int q = S.Lp[j]; q < S.Lp[j + 1]; q++) acc -= conjv(s.Lx[q]) * z[Li[q]];
            z[j] = acc;
        }
        for (int k = 0; k < n; k++) x[S.Pinv[k]] = z[k];
        const auto t1 = std::chrono::steady_clock::now();
        volatile double sink = std::real(x[0]);
        (void)sink;
        return std::chrono::duration<double>(t1 - t0).count();
    }

    // Run nt samples concurrently, one thread per slot: window [a[t], b[t]) then one solve.
    void run(int nt, const int* sl, const int* a, const int* b, double* t_fact, double* t_solve) {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++)
            th.emplace_back([=]() {
                t_fact[t] = time_window(sl[t], a[t], b[t]);
                if (t_solve) t_solve[t] = time_solve(sl[t]);
            });
        for (auto& x : th) x.join();
    }
};

}  // namespace orc
