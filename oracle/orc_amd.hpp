// Oracle (test infrastructure only): approximate minimum degree ordering and the
// simplicial LDL^H (up-looking) factorisation that the reference gets from Eigen 3.4.0's
// SimplicialLDLT<SparseMatrix, Lower> with its default AMDOrdering
// (include/turbomodal/hermitian_lanczos.hpp:56, include/turbomodal/sym_shift_invert_ldlt.hpp:36;
// called at src/hermitian_lanczos.cpp:20-21,38).  Eigen is not in the reference tree; the
// published algorithms it implements are restated:
//   * AMD: Amestoy, Davis & Duff's approximate minimum degree as given in T. A. Davis,
//     "Direct Methods for Sparse Linear Systems" (SIAM 2006), routine cs_amd, in the
//     variant Eigen uses: the pattern of A + A^T keeps its diagonal, a node whose only
//     entry is its diagonal is eliminated first, and a node with no diagonal entry (or of
//     degree above max(16, 10 sqrt(n))) is ordered last;
//   * elimination tree and column counts: Liu's path-compression-free row-subtree walk of
//     Davis's LDL package (ldl_symbolic); numeric factorisation: ldl_numeric (up-looking,
//     D real = real part of the pivot, failure only on an exactly zero pivot).
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "orc_sparse.hpp"

namespace orc {

static inline int amd_flip(int i) { return -i - 2; }

static inline int amd_wclear(int mark, int lemax, int* w, int n) {
    if (mark < 2 || (mark + lemax < 0)) {
        for (int k = 0; k < n; k++)
            if (w[k] != 0) w[k] = 1;
        mark = 2;
    }
    return mark;
}

static inline int amd_tdfs(int j, int k, int* head, const int* next, int* post, int* stack) {
    int top = 0;
    stack[0] = j;
    while (top >= 0) {
        const int p = stack[top];
        const int i = head[p];
        if (i == -1) {
            top--;
            post[k++] = p;
        } else {
            head[p] = next[i];
            stack[++top] = i;
        }
    }
    return k;
}

// Cp/Ci: full symmetric pattern (both triangles and the diagonal), n columns.
// Returns perm with perm[k] = original index of the k-th pivot.
inline std::vector<int> amd_order(int n, const std::vector<int>& Cp_in, const std::vector<int>& Ci_in) {
    std::vector<int> perm(n + 1);
    if (n == 0) { perm.resize(0); return perm; }
    int dense = std::max(16, (int)(10 * std::sqrt((double)n)));
    dense = std::min(n - 2, dense);
    int cnz = Cp_in[n];
    const int t = cnz + cnz / 5 + 2 * n;
    std::vector<int> Cpv(Cp_in.begin(), Cp_in.end());
    std::vector<int> Civ(t);
    std::copy(Ci_in.begin(), Ci_in.begin() + cnz, Civ.begin());
    int* Cp = Cpv.data();
    int* Ci = Civ.data();
    std::vector<int> W(8 * (n + 1));
    int* len = W.data();
    int* nv = len + (n + 1);
    int* next = len + 2 * (n + 1);
    int* head = len + 3 * (n + 1);
    int* elen = len + 4 * (n + 1);
    int* degree = len + 5 * (n + 1);
    int* w = len + 6 * (n + 1);
    int* hhead = len + 7 * (n + 1);
    int* last = perm.data();

    int d, dk, dext, lemax = 0, e, elenk, eln, i, j, k, k1, k2, k3, jlast, ln, nzmax, mindeg = 0,
        nvi, nvj, nvk, mark, wnvi, ok, nel = 0, p, p1, p2, p3, p4, pj, pk, pk1, pk2, pn, q, h;

    for (k = 0; k < n; k++) len[k] = Cp[k + 1] - Cp[k];
    len[n] = 0;
    nzmax = t;
    for (i = 0; i <= n; i++) {
        head[i] = -1; last[i] = -1; next[i] = -1; hhead[i] = -1;
        nv[i] = 1; w[i] = 1; elen[i] = 0; degree[i] = len[i];
    }
    mark = amd_wclear(0, 0, w, n);
    for (i = 0; i < n; i++) {
        bool has_diag = false;
        for (p = Cp[i]; p < Cp[i + 1]; ++p)
            if (Ci[p] == i) { has_diag = true; break; }
        d = degree[i];
        if (d == 1 && has_diag) {
            elen[i] = -2; nel++; Cp[i] = -1; w[i] = 0;
        } else if (d > dense || !has_diag) {
            nv[i] = 0; elen[i] = -1; nel++; Cp[i] = amd_flip(n); nv[n]++;
        } else {
            if (head[d] != -1) last[head[d]] = i;
            next[i] = head[d];
            head[d] = i;
        }
    }
    elen[n] = -2; Cp[n] = -1; w[n] = 0;

    while (nel < n) {
        for (k = -1; mindeg < n && (k = head[mindeg]) == -1; mindeg++) {}
        if (next[k] != -1) last[next[k]] = -1;
        head[mindeg] = next[k];
        elenk = elen[k];
        nvk = nv[k];
        nel += nvk;
        // garbage collection
        if (elenk > 0 && cnz + mindeg >= nzmax) {
            for (j = 0; j < n; j++) {
                if ((p = Cp[j]) >= 0) { Cp[j] = Ci[p]; Ci[p] = amd_flip(j); }
            }
            for (q = 0, p = 0; p < cnz;) {
                if ((j = amd_flip(Ci[p++])) >= 0) {
                    Ci[q] = Cp[j];
                    Cp[j] = q++;
                    for (k3 = 0; k3 < len[j] - 1; k3++) Ci[q++] = Ci[p++];
                }
            }
            cnz = q;
        }
        // construct new element
        dk = 0;
        nv[k] = -nvk;
        p = Cp[k];
        pk1 = (elenk == 0) ? p : cnz;
        pk2 = pk1;
        for (k1 = 1; k1 <= elenk + 1; k1++) {
            if (k1 > elenk) { e = k; pj = p; ln = len[k] - elenk; }
            else { e = Ci[p++]; pj = Cp[e]; ln = len[e]; }
            for (k2 = 1; k2 <= ln; k2++) {
                i = Ci[pj++];
                if ((nvi = nv[i]) <= 0) continue;
                dk += nvi;
                nv[i] = -nvi;
                Ci[pk2++] = i;
                if (next[i] != -1) last[next[i]] = last[i];
                if (last[i] != -1) next[last[i]] = next[i];
                else head[degree[i]] = next[i];
            }
            if (e != k) { Cp[e] = amd_flip(k); w[e] = 0; }
        }
        if (elenk != 0) cnz = pk2;
        degree[k] = dk;
        Cp[k] = pk1;
        len[k] = pk2 - pk1;
        elen[k] = -2;
        // find set differences
        mark = amd_wclear(mark, lemax, w, n);
        for (pk = pk1; pk < pk2; pk++) {
            i = Ci[pk];
            if ((eln = elen[i]) <= 0) continue;
            nvi = -nv[i];
            wnvi = mark - nvi;
            for (p = Cp[i]; p <= Cp[i] + eln - 1; p++) {
                e = Ci[p];
                if (w[e] >= mark) w[e] -= nvi;
                else if (w[e] != 0) w[e] = degree[e] + wnvi;
            }
        }
        // degree update
        for (pk = pk1; pk < pk2; pk++) {
            i = Ci[pk];
            p1 = Cp[i];
            p2 = p1 + elen[i] - 1;
            pn = p1;
            for (h = 0, d = 0, p = p1; p <= p2; p++) {
                e = Ci[p];
                if (w[e] != 0) {
                    dext = w[e] - mark;
                    if (dext > 0) { d += dext; Ci[pn++] = e; h += e; }
                    else { Cp[e] = amd_flip(k); w[e] = 0; }
                }
            }
            elen[i] = pn - p1 + 1;
            p3 = pn;
            p4 = p1 + len[i];
            for (p = p2 + 1; p < p4; p++) {
                j = Ci[p];
                if ((nvj = nv[j]) <= 0) continue;
                d += nvj;
                Ci[pn++] = j;
                h += j;
            }
            if (d == 0) {
                Cp[i] = amd_flip(k);
                nvi = -nv[i];
                dk -= nvi;
                nvk += nvi;
                nel += nvi;
                nv[i] = 0;
                elen[i] = -1;
            } else {
                degree[i] = std::min(degree[i], d);
                Ci[pn] = Ci[p3];
                Ci[p3] = Ci[p1];
                Ci[p1] = k;
                len[i] = pn - p1 + 1;
                h %= n;
                next[i] = hhead[h];
                hhead[h] = i;
                last[i] = h;
            }
        }
        degree[k] = dk;
        lemax = std::max(lemax, dk);
        mark = amd_wclear(mark + lemax, lemax, w, n);
        // supernode detection
        for (pk = pk1; pk < pk2; pk++) {
            i = Ci[pk];
            if (nv[i] >= 0) continue;
            h = last[i];
            i = hhead[h];
            hhead[h] = -1;
            for (; i != -1 && next[i] != -1; i = next[i], mark++) {
                ln = len[i];
                eln = elen[i];
                for (p = Cp[i] + 1; p <= Cp[i] + ln - 1; p++) w[Ci[p]] = mark;
                jlast = i;
                for (j = next[i]; j != -1;) {
                    ok = (len[j] == ln) && (elen[j] == eln);
                    for (p = Cp[j] + 1; ok && p <= Cp[j] + ln - 1; p++)
                        if (w[Ci[p]] != mark) ok = 0;
                    if (ok) {
                        Cp[j] = amd_flip(i);
                        nv[i] += nv[j];
                        nv[j] = 0;
                        elen[j] = -1;
                        j = next[j];
                        next[jlast] = j;
                    } else {
                        jlast = j;
                        j = next[j];
                    }
                }
            }
        }
        // finalize new element
        for (p = pk1, pk = pk1; pk < pk2; pk++) {
            i = Ci[pk];
            if ((nvi = -nv[i]) <= 0) continue;
            nv[i] = nvi;
            d = degree[i] + dk - nvi;
            d = std::min(d, n - nel - nvi);
            if (head[d] != -1) last[head[d]] = i;
            next[i] = head[d];
            last[i] = -1;
            head[d] = i;
            mindeg = std::min(mindeg, d);
            degree[i] = d;
            Ci[p++] = i;
        }
        nv[k] = nvk;
        if ((len[k] = p - pk1) == 0) { Cp[k] = -1; w[k] = 0; }
        if (elenk != 0) cnz = p;
    }
    // postorder the assembly tree
    for (i = 0; i < n; i++) Cp[i] = amd_flip(Cp[i]);
    for (j = 0; j <= n; j++) head[j] = -1;
    for (j = n; j >= 0; j--) {
        if (nv[j] > 0) continue;
        next[j] = head[Cp[j]];
        head[Cp[j]] = j;
    }
    for (e = n; e >= 0; e--) {
        if (nv[e] <= 0) continue;
        if (Cp[e] != -1) {
            next[e] = head[Cp[e]];
            head[Cp[e]] = e;
        }
    }
    for (k = 0, i = 0; i <= n; i++)
        if (Cp[i] == -1) k = amd_tdfs(i, k, head, next, perm.data(), w);
    perm.resize(n);
    return perm;
}

// Symbolic + numeric simplicial LDL^H of a Hermitian matrix given by its LOWER triangle.
template <typename T>
struct SimplicialLDL {
    int n = 0;
    std::vector<int> P, Pinv;        // P[old] = new, Pinv[new] = old (Pinv = AMD order)
    std::vector<int> parent, colcount;
    std::vector<int> Lp, Li;
    std::vector<T> Lx;
    std::vector<double> D;
    Csc<T> ap;                        // upper triangle of the permuted matrix
    bool ok = false;

    // Eigen SimplicialCholeskyBase::ordering: full Hermitian pattern from the lower
    // triangle, AMD on A+A^T (with diagonal), then the permuted upper triangle.
    void analyze(const Csc<T>& A) {
        n = A.cols;
        std::vector<Trip<T>> full;
        full.reserve(2 * A.i.size());
        for (int j = 0; j < n; j++)
            for (int q = A.p[j]; q < A.p[j + 1]; q++) {
                const int i = A.i[q];
                if (i < j) continue;
                full.push_back({i, j, A.x[q]});
                if (i != j) full.push_back({j, i, conjv(A.x[q])});
            }
        Csc<T> C = from_triplets<T>(n, n, full);
        Pinv = amd_order(n, C.p, C.i);
        P.assign(n, 0);
        for (int k = 0; k < n; k++) P[Pinv[k]] = k;
        permute_upper(A);
        // etree and column counts (ldl_symbolic)
        parent.assign(n, -1);
        colcount.assign(n, 0);
        std::vector<int> tags(n);
        for (int k = 0; k < n; k++) {
            parent[k] = -1;
            tags[k] = k;
            colcount[k] = 0;
            for (int q = ap.p[k]; q < ap.p[k + 1]; q++) {
                int i = ap.i[q];
                if (i < k) {
                    for (; tags[i] != k; i = parent[i]) {
                        if (parent[i] == -1) parent[i] = k;
                        colcount[i]++;
                        tags[i] = k;
                    }
                }
            }
        }
        Lp.assign(n + 1, 0);
        for (int k = 0; k < n; k++) Lp[k + 1] = Lp[k] + colcount[k];
        Li.assign(Lp[n], 0);
        Lx.assign(Lp[n], T(0));
    }

    void permute_upper(const Csc<T>& A) {
        std::vector<Trip<T>> up;
        up.reserve(A.i.size());
        for (int j = 0; j < n; j++)
            for (int q = A.p[j]; q < A.p[j + 1]; q++) {
                const int i = A.i[q];
                if (i < j) continue;
                const int pi = P[i], pj = P[j];
                if (pi <= pj) up.push_back({pi, pj, A.x[q]});
                else up.push_back({pj, pi, conjv(A.x[q])});
            }
        ap = from_triplets<T>(n, n, up);
    }

    // ldl_numeric (up-looking): returns false on an exactly zero pivot.
    bool factorize(const Csc<T>& A) {
        permute_upper(A);
        std::vector<T> y(n, T(0));
        std::vector<int> pattern(n), tags(n), nzc(n);
        D.assign(n, 0.0);
        ok = true;
        for (int k = 0; k < n; k++) {
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
                Li[p] = k;
                Lx[p] = l_ki;
                ++nzc[i];
            }
            D[k] = d;
            if (d == 0.0) { ok = false; break; }
        }
        return ok;
    }

    // x = P^T L^-H D^-1 L^-1 P b
    void solve(const T* b, T* x) const {
        std::vector<T> z(n);
        for (int i = 0; i < n; i++) z[P[i]] = b[i];
        for (int j = 0; j < n; j++) {
            const T zj = z[j];
            for (int q = Lp[j]; q < Lp[j + 1]; q++) z[Li[q]] -= Lx[q] * zj;
        }
        for (int j = 0; j < n; j++) z[j] = z[j] / D[j];
        for (int j = n - 1; j >= 0; j--) {
            T s = z[j];
            for (int q = Lp[j]; q < Lp[j + 1]; q++) s -= conjv(Lx[q]) * z[Li[q]];
            z[j] = s;
        }
        for (int k = 0; k < n; k++) x[Pinv[k]] = z[k];
    }
};

}  // namespace orc
