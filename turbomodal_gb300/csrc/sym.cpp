// Host symbolic analysis: AMD, elimination tree, postorder, supernodes, fronts, levels.
#include "sym.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <numeric>
#include <stdexcept>

namespace tmg {

// ---------------------------------------------------------------------------------
// Approximate minimum degree on the quotient graph.  State arrays follow the cs_amd
// formulation: for every index i, len (list length), nv (supervariable size, negated
// while in the current element), next/last (degree or hash lists), head (degree list
// heads), elen (element count of i, -1 dead node, -2 element), degree, w (set-difference
// workspace) and hhead (hash heads).
// ---------------------------------------------------------------------------------
namespace {

inline int32_t flip(int32_t i) { return -i - 2; }

struct QuotientGraph {
    int32_t n;
    std::vector<int32_t> cp, ci;    // object pointers and list memory
    std::vector<int32_t> len, nv, next, head, elen, degree, w, hhead, last;
    int32_t dense = 0, nzmax = 0, cnz = 0, mark = 0, mindeg = 0, lemax = 0, nel = 0;

    int32_t wclear(int32_t m, int32_t lmax) {
        if (m < 2 || m + lmax < 0) {
            for (int32_t k = 0; k < n; k++)
                if (w[k] != 0) w[k] = 1;
            m = 2;
        }
        return m;
    }

    void init(const std::vector<int64_t>& colptr, const std::vector<int32_t>& rowind) {
        dense = std::max<int32_t>(16, (int32_t)(10 * std::sqrt((double)n)));
        dense = std::min<int32_t>(n - 2, dense);
        cnz = (int32_t)colptr[n];
        nzmax = cnz + cnz / 5 + 2 * n;
        cp.assign(n + 1, 0);
        for (int32_t k = 0; k <= n; k++) cp[k] = (int32_t)colptr[k];
        ci.assign(nzmax, 0);
        std::copy(rowind.begin(), rowind.begin() + cnz, ci.begin());
        len.assign(n + 1, 0); nv.assign(n + 1, 1); next.assign(n + 1, -1); head.assign(n + 1, -1);
        elen.assign(n + 1, 0); degree.assign(n + 1, 0); w.assign(n + 1, 1); hhead.assign(n + 1, -1);
        last.assign(n + 1, -1);
        for (int32_t k = 0; k < n; k++) len[k] = cp[k + 1] - cp[k];
        len[n] = 0;
        for (int32_t i = 0; i <= n; i++) degree[i] = len[i];
        mark = wclear(0, 0);
        for (int32_t i = 0; i < n; i++) {
            bool has_diag = false;
            for (int32_t p = cp[i]; p < cp[i + 1]; ++p)
                if (ci[p] == i) { has_diag = true; break; }
            const int32_t d = degree[i];
            if (d == 1 && has_diag) {          // only the diagonal: eliminated at once
                elen[i] = -2; nel++; cp[i] = -1; w[i] = 0;
            } else if (d > dense || !has_diag) {   // ordered last, absorbed into element n
                nv[i] = 0; elen[i] = -1; nel++; cp[i] = flip(n); nv[n]++;
            } else {
                if (head[d] != -1) last[head[d]] = i;
                next[i] = head[d];
                head[d] = i;
            }
        }
        elen[n] = -2; cp[n] = -1; w[n] = 0;
    }

    void compact() {
        for (int32_t j = 0; j < n; j++) {
            int32_t p = cp[j];
            if (p >= 0) { cp[j] = ci[p]; ci[p] = flip(j); }
        }
        int32_t q = 0;
        for (int32_t p = 0; p < cnz;) {
            const int32_t j = flip(ci[p++]);
            if (j >= 0) {
                ci[q] = cp[j];
                cp[j] = q++;
                for (int32_t k3 = 0; k3 < len[j] - 1; k3++) ci[q++] = ci[p++];
            }
        }
        cnz = q;
    }

    void eliminate() {
        while (nel < n) {
            int32_t k = -1;
            for (; mindeg < n && (k = head[mindeg]) == -1; mindeg++) {}
            if (next[k] != -1) last[next[k]] = -1;
            head[mindeg] = next[k];
            const int32_t elenk = elen[k];
            int32_t nvk = nv[k];
            nel += nvk;
            if (elenk > 0 && cnz + mindeg >= nzmax) compact();

            // new element Lk = union of the pivot's elements and variables
            int32_t dk = 0;
            nv[k] = -nvk;
            int32_t p = cp[k];
            const int32_t pk1 = (elenk == 0) ? p : cnz;
            int32_t pk2 = pk1;
            for (int32_t k1 = 1; k1 <= elenk + 1; k1++) {
                int32_t e, pj, ln;
                if (k1 > elenk) { e = k; pj = p; ln = len[k] - elenk; }
                else { e = ci[p++]; pj = cp[e]; ln = len[e]; }
                for (int32_t k2 = 1; k2 <= ln; k2++) {
                    const int32_t i = ci[pj++];
                    const int32_t nvi = nv[i];
                    if (nvi <= 0) continue;
                    dk += nvi;
                    nv[i] = -nvi;
                    ci[pk2++] = i;
                    if (next[i] != -1) last[next[i]] = last[i];
                    if (last[i] != -1) next[last[i]] = next[i];
                    else head[degree[i]] = next[i];
                }
                if (e != k) { cp[e] = flip(k); w[e] = 0; }
            }
            if (elenk != 0) cnz = pk2;
            degree[k] = dk;
            cp[k] = pk1;
            len[k] = pk2 - pk1;
            elen[k] = -2;

            // |Le \ Lk| for every element e adjacent to Lk
            mark = wclear(mark, lemax);
            for (int32_t pk = pk1; pk < pk2; pk++) {
                const int32_t i = ci[pk];
                const int32_t eln = elen[i];
                if (eln <= 0) continue;
                const int32_t nvi = -nv[i];
                const int32_t wnvi = mark - nvi;
                for (int32_t q = cp[i]; q <= cp[i] + eln - 1; q++) {
                    const int32_t e = ci[q];
                    if (w[e] >= mark) w[e] -= nvi;
                    else if (w[e] != 0) w[e] = degree[e] + wnvi;
                }
            }

            // approximate degrees, aggressive absorption, hashing
            for (int32_t pk = pk1; pk < pk2; pk++) {
                const int32_t i = ci[pk];
                const int32_t p1 = cp[i];
                const int32_t p2 = p1 + elen[i] - 1;
                int32_t pn = p1, h = 0, d = 0;
                for (int32_t q = p1; q <= p2; q++) {
                    const int32_t e = ci[q];
                    if (w[e] != 0) {
                        const int32_t dext = w[e] - mark;
                        if (dext > 0) { d += dext; ci[pn++] = e; h += e; }
                        else { cp[e] = flip(k); w[e] = 0; }
                    }
                }
                elen[i] = pn - p1 + 1;
                const int32_t p3 = pn;
                const int32_t p4 = p1 + len[i];
                for (int32_t q = p2 + 1; q < p4; q++) {
                    const int32_t j = ci[q];
                    const int32_t nvj = nv[j];
                    if (nvj <= 0) continue;
                    d += nvj;
                    ci[pn++] = j;
                    h += j;
                }
                if (d == 0) {                      // mass elimination
                    cp[i] = flip(k);
                    const int32_t nvi = -nv[i];
                    dk -= nvi;
                    nvk += nvi;
                    nel += nvi;
                    nv[i] = 0;
                    elen[i] = -1;
                } else {
                    degree[i] = std::min(degree[i], d);
                    ci[pn] = ci[p3];
                    ci[p3] = ci[p1];
                    ci[p1] = k;
                    len[i] = pn - p1 + 1;
                    h %= n;
                    next[i] = hhead[h];
                    hhead[h] = i;
                    last[i] = h;
                }
            }
            degree[k] = dk;
            lemax = std::max(lemax, dk);
            mark = wclear(mark + lemax, lemax);

            // indistinguishable variables -> supervariables
            for (int32_t pk = pk1; pk < pk2; pk++) {
                int32_t i = ci[pk];
                if (nv[i] >= 0) continue;
                const int32_t h = last[i];
                i = hhead[h];
                hhead[h] = -1;
                for (; i != -1 && next[i] != -1; i = next[i], mark++) {
                    const int32_t ln = len[i], eln = elen[i];
                    for (int32_t q = cp[i] + 1; q <= cp[i] + ln - 1; q++) w[ci[q]] = mark;
                    int32_t jlast = i;
                    for (int32_t j = next[i]; j != -1;) {
                        bool ok = (len[j] == ln) && (elen[j] == eln);
                        for (int32_t q = cp[j] + 1; ok && q <= cp[j] + ln - 1; q++)
                            if (w[ci[q]] != mark) ok = false;
                        if (ok) {
                            cp[j] = flip(i);
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

            // finalize Lk and put its variables back in the degree lists
            int32_t pw = pk1;
            for (int32_t pk = pk1; pk < pk2; pk++) {
                const int32_t i = ci[pk];
                const int32_t nvi = -nv[i];
                if (nvi <= 0) continue;
                nv[i] = nvi;
                int32_t d = degree[i] + dk - nvi;
                d = std::min(d, n - nel - nvi);
                if (head[d] != -1) last[head[d]] = i;
                next[i] = head[d];
                last[i] = -1;
                head[d] = i;
                mindeg = std::min(mindeg, d);
                degree[i] = d;
                ci[pw++] = i;
            }
            nv[k] = nvk;
            if ((len[k] = pw - pk1) == 0) { cp[k] = -1; w[k] = 0; }
            if (elenk != 0) cnz = pw;
        }
    }

    std::vector<int32_t> postorder() {
        std::vector<int32_t> order(n + 1);
        for (int32_t i = 0; i < n; i++) cp[i] = flip(cp[i]);
        for (int32_t j = 0; j <= n; j++) head[j] = -1;
        for (int32_t j = n; j >= 0; j--) {
            if (nv[j] > 0) continue;
            next[j] = head[cp[j]];
            head[cp[j]] = j;
        }
        for (int32_t e = n; e >= 0; e--) {
            if (nv[e] <= 0) continue;
            if (cp[e] != -1) { next[e] = head[cp[e]]; head[cp[e]] = e; }
        }
        int32_t k = 0;
        std::vector<int32_t>& stack = w;
        for (int32_t i = 0; i <= n; i++) {
            if (cp[i] != -1) continue;
            int32_t top = 0;
            stack[0] = i;
            while (top >= 0) {
                const int32_t pnode = stack[top];
                const int32_t c = head[pnode];
                if (c == -1) { top--; order[k++] = pnode; }
                else { head[pnode] = next[c]; stack[++top] = c; }
            }
        }
        order.resize(n);
        return order;
    }
};

}  // namespace

std::vector<int32_t> amd_order(int32_t n, const std::vector<int64_t>& colptr, const std::vector<int32_t>& rowind) {
    if (n == 0) return {};
    if (colptr[n] > INT32_MAX / 2) throw std::runtime_error("AMD: pattern too large for 32-bit lists");
    QuotientGraph g;
    g.n = n;
    g.init(colptr, rowind);
    g.eliminate();
    return g.postorder();
}

// ---------------------------------------------------------------------------------
// Pattern utilities
// ---------------------------------------------------------------------------------
Pattern transpose(const Pattern& A) {
    Pattern B;
    B.nrows = A.ncols; B.ncols = A.nrows;
    B.p.assign(B.ncols + 1, 0);
    for (int32_t r : A.i) B.p[r + 1]++;
    for (int32_t c = 0; c < B.ncols; c++) B.p[c + 1] += B.p[c];
    B.i.resize(A.i.size());
    std::vector<int64_t> pos(B.p.begin(), B.p.end() - 1);
    for (int32_t j = 0; j < A.ncols; j++)
        for (int64_t q = A.p[j]; q < A.p[j + 1]; q++) B.i[pos[A.i[q]]++] = j;
    return B;
}

Pattern pattern_union(const std::vector<const Pattern*>& parts) {
    Pattern U;
    U.nrows = parts[0]->nrows; U.ncols = parts[0]->ncols;
    U.p.assign(U.ncols + 1, 0);
    std::vector<int32_t> mark(U.nrows, -1), buf;
    for (int32_t j = 0; j < U.ncols; j++) {
        buf.clear();
        for (const Pattern* P : parts)
            for (int64_t q = P->p[j]; q < P->p[j + 1]; q++) {
                const int32_t r = P->i[q];
                if (mark[r] != j) { mark[r] = j; buf.push_back(r); }
            }
        std::sort(buf.begin(), buf.end());
        U.i.insert(U.i.end(), buf.begin(), buf.end());
        U.p[j + 1] = (int64_t)U.i.size();
    }
    return U;
}

std::vector<int64_t> locate(const Pattern& sup, const Pattern& sub) {
    std::vector<int64_t> out(sub.i.size(), -1);
    for (int32_t j = 0; j < sub.ncols; j++) {
        int64_t q = sup.p[j];
        const int64_t qe = sup.p[j + 1];
        for (int64_t s = sub.p[j]; s < sub.p[j + 1]; s++) {
            const int32_t r = sub.i[s];
            while (q < qe && sup.i[q] < r) q++;
            if (q < qe && sup.i[q] == r) out[s] = q;
        }
    }
    return out;
}

Pattern lower_triangle(const Pattern& A) {
    Pattern L;
    L.nrows = A.nrows; L.ncols = A.ncols;
    L.p.assign(A.ncols + 1, 0);
    for (int32_t j = 0; j < A.ncols; j++) {
        for (int64_t q = A.p[j]; q < A.p[j + 1]; q++)
            if (A.i[q] >= j) L.i.push_back(A.i[q]);
        L.p[j + 1] = (int64_t)L.i.size();
    }
    return L;
}

LancasterBlocks lancaster_blocks(const Pattern& K, const Pattern& M, const Pattern& G, int which) {
    const int32_t n = K.ncols;
    LancasterBlocks L;
    L.P.nrows = L.P.ncols = 2 * n;
    L.P.p.assign(2 * (size_t)n + 1, 0);
    auto put = [&](int32_t r, int64_t k, int64_t m, int64_t g, int8_t b) {
        L.P.i.push_back(r);
        L.srcK.push_back(k); L.srcM.push_back(m); L.srcG.push_back(g); L.blk.push_back(b);
    };
    for (int32_t j = 0; j < n; j++) {              // block column 0: [D - sigma M; K] or [M; 0]
        int64_t qm = M.p[j], qg = which == 0 ? G.p[j] : 0;
        const int64_t em = M.p[j + 1], eg = which == 0 ? G.p[j + 1] : 0;
        while (qm < em || qg < eg) {               // sorted merge of the M and G columns
            const int32_t rm = qm < em ? M.i[qm] : INT32_MAX;
            const int32_t rg = qg < eg ? G.i[qg] : INT32_MAX;
            const int32_t r = std::min(rm, rg);
            put(r, -1, rm == r ? qm : -1, rg == r ? qg : -1, 0);
            if (rm == r) qm++;
            if (rg == r) qg++;
        }
        if (which == 0)
            for (int64_t q = K.p[j]; q < K.p[j + 1]; q++) put(n + K.i[q], q, -1, -1, 2);
        L.P.p[j + 1] = (int64_t)L.P.i.size();
    }
    for (int32_t j = 0; j < n; j++) {              // block column 1: [K; -sigma K] or [0; K]
        if (which == 0)
            for (int64_t q = K.p[j]; q < K.p[j + 1]; q++) put(K.i[q], q, -1, -1, 1);
        for (int64_t q = K.p[j]; q < K.p[j + 1]; q++) put(n + K.i[q], q, -1, -1, 3);
        L.P.p[n + j + 1] = (int64_t)L.P.i.size();
    }
    return L;
}

Product product(const Pattern& A, const Pattern& B) {
    Product P;
    P.C.nrows = A.nrows; P.C.ncols = B.ncols;
    P.C.p.assign(B.ncols + 1, 0);
    P.cptr.assign(1, 0);
    std::vector<int32_t> slot(A.nrows, -1);      // position in current column buffer
    std::vector<int32_t> rows;
    std::vector<std::vector<std::pair<int64_t, int64_t>>> contrib;
    for (int32_t j = 0; j < B.ncols; j++) {
        rows.clear();
        contrib.clear();
        for (int64_t qb = B.p[j]; qb < B.p[j + 1]; qb++) {
            const int32_t k = B.i[qb];
            for (int64_t qa = A.p[k]; qa < A.p[k + 1]; qa++) {
                const int32_t r = A.i[qa];
                if (slot[r] < 0) { slot[r] = (int32_t)rows.size(); rows.push_back(r); contrib.emplace_back(); }
                contrib[slot[r]].push_back({qa, qb});
            }
        }
        std::vector<int32_t> order(rows.size());
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return rows[a] < rows[b]; });
        for (int32_t o : order) {
            P.C.i.push_back(rows[o]);
            for (auto& pr : contrib[o]) { P.a_slot.push_back(pr.first); P.b_slot.push_back(pr.second); }
            P.cptr.push_back((int64_t)P.a_slot.size());
            slot[rows[o]] = -1;
        }
        P.C.p[j + 1] = (int64_t)P.C.i.size();
    }
    return P;
}

// ---------------------------------------------------------------------------------
// Supernodal symbolic factorisation
// ---------------------------------------------------------------------------------
Symbolic analyze(const Pattern& lower, double relax, int32_t relax_max_width, const std::vector<int32_t>* amd) {
    Symbolic S;
    const int32_t n = lower.ncols;
    S.n = n;
    if (amd && (int32_t)amd->size() == n) {   // the order of an earlier analysis of this pattern
        S.amd = *amd;
    } else {
        // full symmetric pattern with diagonal, rows sorted
        Pattern up = transpose(lower);
        Pattern full = pattern_union({&lower, &up});
        S.amd = amd_order(n, full.p, full.i);
    }
    std::vector<int32_t> P(n);
    for (int32_t k = 0; k < n; k++) P[S.amd[k]] = k;
    // permuted upper pattern (AMD numbering): column max(pi,pj) holds row min(pi,pj)
    Pattern ap;
    ap.nrows = ap.ncols = n;
    ap.p.assign(n + 1, 0);
    for (int32_t j = 0; j < n; j++)
        for (int64_t q = lower.p[j]; q < lower.p[j + 1]; q++) {
            const int32_t i = lower.i[q];
            if (i < j) continue;
            ap.p[std::max(P[i], P[j]) + 1]++;
        }
    for (int32_t c = 0; c < n; c++) ap.p[c + 1] += ap.p[c];
    ap.i.resize(ap.p[n]);
    {
        std::vector<int64_t> pos(ap.p.begin(), ap.p.end() - 1);
        for (int32_t j = 0; j < n; j++)
            for (int64_t q = lower.p[j]; q < lower.p[j + 1]; q++) {
                const int32_t i = lower.i[q];
                if (i < j) continue;
                ap.i[pos[std::max(P[i], P[j])]++] = std::min(P[i], P[j]);
            }
    }
    // elimination tree and column counts by row-subtree traversal
    S.etree.assign(n, -1);
    S.colcount.assign(n, 0);
    {
        std::vector<int32_t> tags(n);
        for (int32_t k = 0; k < n; k++) {
            tags[k] = k;
            for (int64_t q = ap.p[k]; q < ap.p[k + 1]; q++) {
                int32_t i = ap.i[q];
                if (i >= k) continue;
                for (; tags[i] != k; i = S.etree[i]) {
                    if (S.etree[i] == -1) S.etree[i] = k;
                    S.colcount[i]++;
                    tags[i] = k;
                }
            }
        }
    }
    S.nnz_l = 0;
    for (int32_t c : S.colcount) { S.nnz_l += c; S.flops_real += (double)c * (double)c; }

    // etree postorder (children visited in increasing index) -> factor numbering
    std::vector<int32_t> post(n);
    {
        std::vector<int32_t> head(n, -1), nxt(n, -1), stack(n);
        for (int32_t j = n - 1; j >= 0; j--)
            if (S.etree[j] != -1) { nxt[j] = head[S.etree[j]]; head[S.etree[j]] = j; }
        int32_t k = 0;
        for (int32_t r = 0; r < n; r++) {
            if (S.etree[r] != -1) continue;
            int32_t top = 0;
            stack[0] = r;
            while (top >= 0) {
                const int32_t p = stack[top];
                const int32_t c = head[p];
                if (c == -1) { top--; post[k++] = p; }
                else { head[p] = nxt[c]; stack[++top] = c; }
            }
        }
    }
    std::vector<int32_t> ipost(n);
    for (int32_t k = 0; k < n; k++) ipost[post[k]] = k;
    S.perm.resize(n);
    S.iperm.resize(n);
    for (int32_t j = 0; j < n; j++) { S.perm[j] = S.amd[post[j]]; S.iperm[S.perm[j]] = j; }
    std::vector<int32_t> par(n), cc(n), nchild(n, 0);
    for (int32_t j = 0; j < n; j++) {
        const int32_t a = post[j];
        par[j] = S.etree[a] == -1 ? -1 : ipost[S.etree[a]];
        cc[j] = S.colcount[a];
        if (par[j] >= 0) nchild[par[j]]++;
    }

    // fundamental supernodes, then optional relaxed merging of chains
    std::vector<int32_t> first;
    for (int32_t j = 0; j < n; j++) {
        const bool cont = j > 0 && par[j - 1] == j && cc[j - 1] == cc[j] + 1 && nchild[j] == 1;
        if (!cont) first.push_back(j);
    }
    first.push_back(n);
    int32_t ns = (int32_t)first.size() - 1;
    std::vector<int32_t> col2sn(n);
    for (int32_t s = 0; s < ns; s++)
        for (int32_t j = first[s]; j < first[s + 1]; j++) col2sn[j] = s;
    if (relax > 0.0) {
        // Amalgamation: a run of supernodes [start, end) takes in the next supernode t when t is
        // the parent of the run's last column (t's first column == end in postorder, so the
        // merged columns stay contiguous; t may have other children, which then update the
        // merged front) and the explicit zeros stay within `relax` of the stored entries.  The
        // merged front holds the run's columns plus t's front rows (the run's fill below t is
        // inside t's front), so its height at the first column is (end - start) + cc[first[t]] + 1.
        std::vector<int32_t> nf;
        int32_t s = 0;
        while (s < ns) {
            int32_t start = first[s];
            int32_t end = first[s + 1];
            while (true) {
                const int32_t t = col2sn[end - 1] + 1;   // next supernode
                if (t >= ns) break;
                if (par[end - 1] != first[t]) break;
                const int32_t wt = first[t + 1] - first[t];
                const int32_t w = end - start;
                if (relax_max_width > 0 && w + wt > relax_max_width) break;
                const double H = (double)w + cc[first[t]] + 1;
                double stored = 0, real = 0;
                for (int32_t j = start; j < first[t + 1]; j++) {
                    stored += H - (j - start);
                    real += cc[j] + 1;
                }
                if (stored - real > relax * stored) break;
                end = first[t + 1];
            }
            nf.push_back(start);
            s = col2sn[end - 1] + 1;
        }
        nf.push_back(n);
        first = nf;
        ns = (int32_t)first.size() - 1;
        for (int32_t t = 0; t < ns; t++)
            for (int32_t j = first[t]; j < first[t + 1]; j++) col2sn[j] = t;
    }
    S.ns = ns;
    S.sn_first = first;

    // permuted lower pattern in factor numbering: column c holds rows >= c
    Pattern pl;
    pl.nrows = pl.ncols = n;
    pl.p.assign(n + 1, 0);
    for (int32_t j = 0; j < n; j++)
        for (int64_t q = lower.p[j]; q < lower.p[j + 1]; q++) {
            const int32_t i = lower.i[q];
            if (i < j) continue;
            pl.p[std::min(S.iperm[i], S.iperm[j]) + 1]++;
        }
    for (int32_t c = 0; c < n; c++) pl.p[c + 1] += pl.p[c];
    pl.i.resize(pl.p[n]);
    {
        std::vector<int64_t> pos(pl.p.begin(), pl.p.end() - 1);
        for (int32_t j = 0; j < n; j++)
            for (int64_t q = lower.p[j]; q < lower.p[j + 1]; q++) {
                const int32_t i = lower.i[q];
                if (i < j) continue;
                pl.i[pos[std::min(S.iperm[i], S.iperm[j])]++] = std::max(S.iperm[i], S.iperm[j]);
            }
    }
    // supernodal tree and children
    S.sn_parent.assign(ns, -1);
    for (int32_t s = 0; s < ns; s++) {
        const int32_t pj = par[first[s + 1] - 1];
        S.sn_parent[s] = pj < 0 ? -1 : col2sn[pj];
    }
    S.child_ptr.assign(ns + 1, 0);
    for (int32_t s = 0; s < ns; s++)
        if (S.sn_parent[s] >= 0) S.child_ptr[S.sn_parent[s] + 1]++;
    for (int32_t s = 0; s < ns; s++) S.child_ptr[s + 1] += S.child_ptr[s];
    S.child_list.resize(S.child_ptr[ns]);
    {
        std::vector<int32_t> pos(S.child_ptr.begin(), S.child_ptr.end() - 1);
        for (int32_t s = 0; s < ns; s++)
            if (S.sn_parent[s] >= 0) S.child_list[pos[S.sn_parent[s]]++] = s;
    }
    // front row structures (children precede parents in postorder)
    S.sn_row_ptr.assign(ns + 1, 0);
    std::vector<int32_t> mark(n, -1), buf;
    std::vector<std::vector<int32_t>> rows(ns);
    for (int32_t s = 0; s < ns; s++) {
        const int32_t f = first[s], l = first[s + 1];
        buf.clear();
        for (int32_t j = f; j < l; j++) { mark[j] = s; buf.push_back(j); }
        for (int32_t j = f; j < l; j++)
            for (int64_t q = pl.p[j]; q < pl.p[j + 1]; q++) {
                const int32_t r = pl.i[q];
                if (r >= l && mark[r] != s) { mark[r] = s; buf.push_back(r); }
            }
        for (int32_t c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
            const int32_t ch = S.child_list[c];
            const int32_t wc = first[ch + 1] - first[ch];
            for (size_t q = wc; q < rows[ch].size(); q++) {
                const int32_t r = rows[ch][q];
                if (r >= l && mark[r] != s) { mark[r] = s; buf.push_back(r); }
            }
        }
        std::sort(buf.begin(), buf.end());
        rows[s] = buf;
        S.sn_row_ptr[s + 1] = S.sn_row_ptr[s] + (int64_t)buf.size();
        S.max_front = std::max<int32_t>(S.max_front, (int32_t)buf.size());
    }
    S.sn_rows.resize(S.sn_row_ptr[ns]);
    S.front_off.assign(ns + 1, 0);
    for (int32_t s = 0; s < ns; s++) {
        std::copy(rows[s].begin(), rows[s].end(), S.sn_rows.begin() + S.sn_row_ptr[s]);
        const int64_t m = (int64_t)rows[s].size();
        S.front_off[s + 1] = S.front_off[s] + m * m;
    }
    // relative indices of each child's update rows inside its parent's front
    S.rel_ptr.assign(ns + 1, 0);
    std::vector<int32_t> local(n, -1);
    for (int32_t s = 0; s < ns; s++) {
        const int32_t w = first[s + 1] - first[s];
        const int64_t m = (int64_t)rows[s].size();
        S.rel_ptr[s + 1] = S.rel_ptr[s] + (S.sn_parent[s] >= 0 ? m - w : 0);
    }
    S.rel.resize(S.rel_ptr[ns]);
    for (int32_t p = 0; p < ns; p++) {
        for (size_t q = 0; q < rows[p].size(); q++) local[rows[p][q]] = (int32_t)q;
        for (int32_t c = S.child_ptr[p]; c < S.child_ptr[p + 1]; c++) {
            const int32_t ch = S.child_list[c];
            const int32_t wc = first[ch + 1] - first[ch];
            int64_t o = S.rel_ptr[ch];
            for (size_t q = wc; q < rows[ch].size(); q++) {
                const int32_t li = local[rows[ch][q]];
                if (li < 0) throw std::runtime_error("symbolic: child row missing from parent front");
                S.rel[o++] = li;
            }
        }
        for (size_t q = 0; q < rows[p].size(); q++) local[rows[p][q]] = -1;
    }
    // levels by height
    std::vector<int32_t> lev(ns, 0);
    int32_t maxlev = 0;
    for (int32_t s = 0; s < ns; s++) {
        for (int32_t c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++)
            lev[s] = std::max(lev[s], lev[S.child_list[c]] + 1);
        maxlev = std::max(maxlev, lev[s]);
    }
    S.level_ptr.assign(maxlev + 2, 0);
    for (int32_t s = 0; s < ns; s++) S.level_ptr[lev[s] + 1]++;
    for (int32_t l = 0; l <= maxlev; l++) S.level_ptr[l + 1] += S.level_ptr[l];
    S.level_sn.resize(ns);
    {
        std::vector<int32_t> pos(S.level_ptr.begin(), S.level_ptr.end() - 1);
        for (int32_t s = 0; s < ns; s++) S.level_sn[pos[lev[s]]++] = s;
    }
    return S;
}

void scatter_map(const Symbolic& S, const Pattern& lower, std::vector<int64_t>& dest, std::vector<uint8_t>& conj) {
    const int32_t n = S.n;
    std::vector<int32_t> col2sn(n);
    for (int32_t s = 0; s < S.ns; s++)
        for (int32_t j = S.sn_first[s]; j < S.sn_first[s + 1]; j++) col2sn[j] = s;
    dest.assign(lower.i.size(), -1);
    conj.assign(lower.i.size(), 0);
    for (int32_t j = 0; j < lower.ncols; j++)
        for (int64_t q = lower.p[j]; q < lower.p[j + 1]; q++) {
            const int32_t i = lower.i[q];
            if (i < j) continue;
            int32_t r = S.iperm[i], c = S.iperm[j];
            uint8_t cj = 0;
            if (r < c) { std::swap(r, c); cj = 1; }
            const int32_t s = col2sn[c];
            const int64_t m = S.sn_row_ptr[s + 1] - S.sn_row_ptr[s];
            const int32_t* rb = S.sn_rows.data() + S.sn_row_ptr[s];
            const int32_t* it = std::lower_bound(rb, rb + m, r);
            if (it == rb + m || *it != r) throw std::runtime_error("scatter_map: row not in front");
            const int64_t lr = it - rb;
            const int64_t lc = c - S.sn_first[s];
            dest[q] = S.front_off[s] + lc * m + lr;
            conj[q] = cj;
        }
}

SolvePlan build_solve_plan(const Symbolic& S, int nb, int rows_per_rect, std::vector<int32_t>& si,
                           int64_t subtree_entries) {
    SolvePlan P;
    P.nb = nb;
    const int nlev = (int)S.level_ptr.size() - 1;
    P.levels.assign(std::max(nlev, 0), SolveLevel{});
    auto width = [&](int s) { return S.sn_first[s + 1] - S.sn_first[s]; };
    auto height = [&](int s) { return S.sn_row_ptr[s + 1] - S.sn_row_ptr[s]; };
    // subtrees solved whole by one warp: every front at most nb wide, at most subtree_entries
    // panel entries in all, and the subtree a contiguous range of supernodes (postorder)
    std::vector<int64_t> ent(S.ns, 0);
    std::vector<int32_t> lo(S.ns), cnt(S.ns, 1);
    std::vector<char> small(S.ns, 0);
    for (int s = 0; s < S.ns; s++) {
        bool ok = width(s) <= nb;
        int64_t e = (int64_t)width(s) * height(s);
        lo[s] = s;
        for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
            const int ch = S.child_list[c];
            if (ch >= s) { ok = false; continue; }   // not a postorder: never merged
            ok = ok && small[ch];
            e += ent[ch];
            cnt[s] += cnt[ch];
            lo[s] = std::min(lo[s], lo[ch]);
        }
        ent[s] = e;
        small[s] = ok && e <= subtree_entries && s - lo[s] + 1 == cnt[s];
    }
    std::vector<std::pair<int64_t, int>> roots;
    for (int s = 0; s < S.ns; s++) {
        const int par = S.sn_parent[s];
        if (small[s] && (par < 0 || !small[par])) roots.push_back({ent[s], s});
    }
    std::stable_sort(roots.begin(), roots.end(), [](const auto& x, const auto& y) { return x.first > y.first; });
    P.sub_off = (int64_t)si.size();
    for (auto [e, s] : roots) {
        si.push_back(lo[s]); si.push_back(s); P.sub_cnt++;
        P.sub_fronts += cnt[s];
    }
    for (int l = 0; l < nlev; l++) {
        SolveLevel& L = P.levels[l];
        std::vector<int32_t> up;                   // the level's upper fronts
        for (int q = S.level_ptr[l]; q < S.level_ptr[l + 1]; q++)
            if (!small[S.level_sn[q]]) up.push_back(S.level_sn[q]);
        L.gath_off = (int64_t)si.size();
        for (int s : up) {
            si.push_back(s); L.gath_cnt++;
            L.maxw = std::max(L.maxw, width(s));
            L.maxu = std::max<int64_t>(L.maxu, height(s) - width(s));
        }
        const int nbk = (L.maxw + nb - 1) / nb;   // diagonal blocks of the widest upper front
        L.ftri_off.assign(std::max(nbk, 1), 0);
        L.ftri_cnt.assign(std::max(nbk, 1), 0);
        L.btri_off.assign(std::max(nbk, 1), 0);
        L.btri_cnt.assign(std::max(nbk, 1), 0);
        for (int b = 0; b + 1 < nbk; b++) {              // forward triangle launches
            L.ftri_off[b] = (int64_t)si.size();
            for (int s : up)
                for (int r0 = (b + 1) * nb; r0 < width(s); r0 += nb) { si.push_back(s); si.push_back(r0); L.ftri_cnt[b]++; }
        }
        for (int b = 1; b < nbk; b++) {                  // backward triangle launches
            L.btri_off[b] = (int64_t)si.size();
            for (int s : up) {
                if (width(s) <= b * nb) continue;
                for (int c0 = 0; c0 < b * nb; c0 += nb) { si.push_back(s); si.push_back(c0); L.btri_cnt[b]++; }
            }
        }
        L.frect_off = (int64_t)si.size();
        for (int s : up)
            for (int64_t r0 = width(s); r0 < height(s); r0 += rows_per_rect) {
                si.push_back(s); si.push_back((int32_t)r0); L.frect_cnt++;
            }
        L.brect_off = (int64_t)si.size();
        for (int s : up)
            for (int c0 = 0; c0 < width(s); c0 += nb) { si.push_back(s); si.push_back(c0); L.brect_cnt++; }
    }
    // diagonal blocks to invert after the factorisation
    P.inv_small_off = (int64_t)si.size();
    for (int s = 0; s < S.ns; s++)
        for (int b = 0; b * nb < width(s); b++) {
            const int nbb = std::min(nb, width(s) - b * nb);
            if (nbb <= 32 && nbb > 1) { si.push_back(s); si.push_back(b); P.inv_small_cnt++; }
        }
    P.inv_large_off = (int64_t)si.size();
    for (int s = 0; s < S.ns; s++)
        for (int b = 0; b * nb < width(s); b++)
            if (std::min(nb, width(s) - b * nb) > 32) { si.push_back(s); si.push_back(b); P.inv_large_cnt++; }
    return P;
}

}  // namespace tmg
