// Host check of the triangular-solve schedule (tests/test_solve_schedule.py): builds the
// supernodal analysis and the solve plan with the library's own host code (sym.cpp), replays
// every launch item with the index arithmetic of the device kernels (mf.cu: k_inv_*, k_sub_fwd,
// k_fwd_gather, k_fwd_tri, k_fwd_rect, k_bwd_rect, k_bwd_tri, k_sub_bwd) with bounds checks, and
// checks that every supernode is solved exactly once per direction, by one subtree task (whose
// fronts are at most 64 wide and whose children lie inside the task) or by its level; compares
// the result with a plain column-by-column supernodal solve on the same random unit-lower L and
// positive D, and checks every column's fill against the rows its front stores.  Optional
// arguments: supernode relaxation and its width limit (analyze()).  Prints
// "max_rel_err=<e> bounds_errors=<k> launches=<n> supernodes=<s> struct_errors=<f> subtrees=<t>
// subtree_fronts=<u>".
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "sym.hpp"

using namespace tmg;

static long nerr = 0;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t hdr[2];
    if (std::fread(hdr, 8, 2, f) != 2) return 2;
    Pattern P;
    P.nrows = P.ncols = (int32_t)hdr[0];
    P.p.resize(hdr[0] + 1);
    P.i.resize(hdr[1]);
    if (std::fread(P.p.data(), 8, hdr[0] + 1, f) != (size_t)hdr[0] + 1) return 2;
    if (std::fread(P.i.data(), 4, hdr[1], f) != (size_t)hdr[1]) return 2;
    std::fclose(f);
    const int NB = 64, RR = 64, CH = 2048;
    const double relax = argc > 2 ? std::atof(argv[2]) : 0.0;
    const int relax_w = argc > 3 ? std::atoi(argv[3]) : 0;
    const Symbolic S = analyze(P, relax, relax_w);
    std::vector<int32_t> items;
    const SolvePlan plan = build_solve_plan(S, NB, RR, items);
    const int ns = S.ns, n = S.n;
    auto W = [&](int s) { return S.sn_first[s + 1] - S.sn_first[s]; };
    auto H = [&](int s) { return (int64_t)(S.sn_row_ptr[s + 1] - S.sn_row_ptr[s]); };
    std::vector<int64_t> lo(ns + 1, 0);
    for (int s = 0; s < ns; s++) lo[s + 1] = lo[s] + H(s) * W(s);
    std::vector<double> L(lo[ns]), L0;
    std::mt19937 g(7);
    std::uniform_real_distribution<double> U(-0.3, 0.3);
    for (int s = 0; s < ns; s++)
        for (int j = 0; j < W(s); j++)
            for (int64_t r = 0; r < H(s); r++)
                L[lo[s] + j * H(s) + r] = r == j ? 1.0 + std::fabs(U(g)) : (r > j ? U(g) / std::sqrt((double)H(s)) : 1e300);
    L0 = L;
    std::vector<double> b(n);
    for (auto& v : b) v = U(g);
    // reference: L y = b, x = D^-1 y, L^T x = x (supernode order = etree postorder)
    std::vector<double> xr(b);
    for (int s = 0; s < ns; s++) {
        const int32_t* rows = &S.sn_rows[S.sn_row_ptr[s]];
        for (int j = 0; j < W(s); j++)
            for (int64_t r = j + 1; r < H(s); r++) xr[rows[r]] -= L0[lo[s] + j * H(s) + r] * xr[S.sn_first[s] + j];
    }
    for (int s = 0; s < ns; s++)
        for (int j = 0; j < W(s); j++) xr[S.sn_first[s] + j] /= L0[lo[s] + j * H(s) + j];
    for (int s = ns - 1; s >= 0; s--) {
        const int32_t* rows = &S.sn_rows[S.sn_row_ptr[s]];
        for (int j = W(s) - 1; j >= 0; j--) {
            double a = xr[S.sn_first[s] + j];
            for (int64_t r = j + 1; r < H(s); r++) a -= L0[lo[s] + j * H(s) + r] * xr[rows[r]];
            xr[S.sn_first[s] + j] = a;
        }
    }
    // bounds-checked accessors of the kernels' address arithmetic
    auto Lat = [&](int s, int64_t idx) -> double& {
        if (!(idx >= 0 && idx < H(s) * W(s))) nerr++;
        return L[lo[s] + std::max<int64_t>(0, std::min<int64_t>(idx, H(s) * W(s) - 1))];
    };
    std::vector<double> t(S.sn_row_ptr[ns], 0.0), x(b);
    auto Tat = [&](int s, int64_t r) -> double& {
        if (!(r >= 0 && r < H(s))) nerr++;
        return t[S.sn_row_ptr[s] + std::max<int64_t>(0, std::min<int64_t>(r, H(s) - 1))];
    };
    auto Xat = [&](int64_t i) -> double& {
        if (!(i >= 0 && i < n)) nerr++;
        return x[std::max<int64_t>(0, std::min<int64_t>(i, n - 1))];
    };
    auto item = [&](int64_t off, int k, int c) { return items[off + 2 * k + c]; };
    long launches = 0;
    // k_inv_small / k_inv_large: unit-lower inverse of every listed diagonal block
    for (int pass = 0; pass < 2; pass++) {
        const int64_t off = pass == 0 ? plan.inv_small_off : plan.inv_large_off;
        const int cnt = pass == 0 ? plan.inv_small_cnt : plan.inv_large_cnt;
        launches++;
        for (int it = 0; it < cnt; it++) {
            const int s = item(off, it, 0), bb = item(off, it, 1);
            const int b0 = bb * NB, nbb = std::min(NB, W(s) - b0);
            if (pass == 0 && (nbb < 2 || nbb > 32)) nerr++;
            std::vector<double> Lb(64 * 64, 0.0);
            for (int k = 0; k < nbb; k++)
                for (int i = k + 1; i < nbb; i++) Lb[i * 64 + k] = Lat(s, (int64_t)(b0 + k) * H(s) + b0 + i);
            for (int j = 0; j < nbb - 1; j++) {
                std::vector<double> v(nbb, 0.0);
                v[j] = 1.0;
                for (int k = j; k < nbb - 1; k++)
                    for (int i = k + 1; i < nbb; i++) v[i] -= Lb[i * 64 + k] * v[k];
                for (int i = j + 1; i < nbb; i++) Lat(s, (int64_t)(b0 + j) * H(s) + b0 + i) = v[i];
            }
        }
    }
    const int nlev = (int)plan.levels.size();
    auto applyX = [&](int s, int c0, int nbk, const std::vector<double>& u, std::vector<double>& v) {
        for (int i = 0; i < nbk; i++) {
            double a = u[i];
            for (int k = 0; k < i; k++) a += Lat(s, (int64_t)(c0 + k) * H(s) + c0 + i) * u[k];
            v[i] = a;
        }
    };
    auto applyXt = [&](int s, int c0, int nbk, const std::vector<double>& u, std::vector<double>& v) {
        for (int i = 0; i < nbk; i++) {
            double a = u[i];
            for (int k = i + 1; k < nbk; k++) a += Lat(s, (int64_t)(c0 + i) * H(s) + c0 + k) * u[k];
            v[i] = a;
        }
    };
    std::vector<int> solved_fwd(ns, 0), solved_bwd(ns, 0);
    // forward sweep: k_sub_fwd (one warp per task, supernodes first..root in order)
    if (plan.sub_cnt) launches++;
    for (int it = 0; it < plan.sub_cnt; it++) {
        const int s0 = item(plan.sub_off, it, 0), s1 = item(plan.sub_off, it, 1);
        if (s0 > s1 || s0 < 0 || s1 >= ns) { nerr++; continue; }
        int64_t entries = 0;                                              // the plan's subtree bound
        for (int s = s0; s <= s1; s++) entries += H(s) * W(s);
        if (entries > 65536) nerr++;
        const int top = S.sn_parent[s1];
        if (top >= s0 && top <= s1) nerr++;                               // the task ends at its root
        for (int s = s0; s <= s1; s++) {
            solved_fwd[s]++;
            const int fs = S.sn_first[s], w = W(s);
            if (w > 64) nerr++;
            for (int64_t r = 0; r < H(s); r++) Tat(s, r) = r < w ? Xat(fs + r) : 0.0;
            for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
                const int ch = S.child_list[c];
                if (ch < s0 || ch >= s) nerr++;                            // solved earlier by this warp
                const int64_t nu = H(ch) - W(ch);
                for (int64_t a = 0; a < nu; a++) Tat(s, S.rel[S.rel_ptr[ch] + a]) += Tat(ch, H(ch) - nu + a);
            }
            std::vector<double> y(64, 0.0);
            for (int i = 0; i < w; i++) {
                double a = Tat(s, i);
                for (int k = 0; k < i; k++) a += Lat(s, (int64_t)k * H(s) + i) * Tat(s, k);
                y[i] = a;
            }
            for (int i = 0; i < w; i++) Xat(fs + i) = y[i] / Lat(s, (int64_t)i * H(s) + i);
            for (int64_t r = w; r < H(s); r++) {
                double a = 0.0;
                for (int j = 0; j < w; j++) a += Lat(s, (int64_t)j * H(s) + r) * y[j];
                Tat(s, r) -= a;
            }
        }
    }
    for (int l = 0; l < nlev; l++) {
        const SolveLevel& Lv = plan.levels[l];
        if (Lv.gath_cnt) launches++;
        for (int q = 0; q < Lv.gath_cnt; q++) {                           // k_fwd_gather
            const int s = items[Lv.gath_off + q], fs = S.sn_first[s];
            solved_fwd[s]++;
            if (W(s) > Lv.maxw || H(s) - W(s) > Lv.maxu) nerr++;          // staging sized by the level
            for (int64_t r = 0; r < H(s); r++) Tat(s, r) = r < W(s) ? Xat(fs + r) : 0.0;
            for (int c = S.child_ptr[s]; c < S.child_ptr[s + 1]; c++) {
                const int ch = S.child_list[c];
                for (int64_t a = 0; a < H(ch) - W(ch); a++) Tat(s, S.rel[S.rel_ptr[ch] + a]) += Tat(ch, W(ch) + a);
            }
            const int nb0 = std::min(NB, W(s));
            std::vector<double> u(nb0), v(nb0);
            for (int i = 0; i < nb0; i++) u[i] = Tat(s, i);
            applyX(s, 0, nb0, u, v);
            for (int i = 0; i < nb0; i++) { Tat(s, i) = v[i]; Xat(fs + i) = v[i] / Lat(s, (int64_t)i * H(s) + i); }
        }
        for (size_t bb = 0; bb < Lv.ftri_cnt.size(); bb++) {             // k_fwd_tri
            if (!Lv.ftri_cnt[bb]) continue;
            launches++;
            for (int it = 0; it < Lv.ftri_cnt[bb]; it++) {
                const int s = item(Lv.ftri_off[bb], it, 0), r0 = item(Lv.ftri_off[bb], it, 1);
                const int fs = S.sn_first[s], b0 = (int)bb * NB, rend = std::min(r0 + NB, W(s));
                std::vector<double> ys(NB), tn(NB, 0.0), yn(NB, 0.0);
                for (int j = 0; j < NB; j++) ys[j] = Tat(s, b0 + j);
                for (int r = r0; r < rend; r++) {
                    double a = 0.0;
                    for (int j = 0; j < NB; j++) a += Lat(s, (int64_t)(b0 + j) * H(s) + r) * ys[j];
                    Tat(s, r) -= a;
                    tn[r - r0] = Tat(s, r);
                }
                if (r0 == b0 + NB) {
                    applyX(s, r0, rend - r0, tn, yn);
                    for (int i = 0; i < rend - r0; i++) {
                        Tat(s, r0 + i) = yn[i];
                        Xat(fs + r0 + i) = yn[i] / Lat(s, (int64_t)(r0 + i) * H(s) + r0 + i);
                    }
                }
            }
        }
        if (Lv.frect_cnt) launches++;
        for (int it = 0; it < Lv.frect_cnt; it++) {                        // k_fwd_rect
            const int s = item(Lv.frect_off, it, 0), r0 = item(Lv.frect_off, it, 1);
            for (int64_t r = r0; r < std::min<int64_t>(r0 + RR, H(s)); r++) {
                double a = 0.0;
                for (int j = 0; j < W(s); j++) a += Lat(s, (int64_t)j * H(s) + r) * Tat(s, j);
                Tat(s, r) -= a;
            }
        }
    }
    // backward sweep
    for (int l = nlev - 1; l >= 0; l--) {
        const SolveLevel& Lv = plan.levels[l];
        if (Lv.brect_cnt) launches++;
        for (int it = 0; it < Lv.brect_cnt; it++) {                        // k_bwd_rect
            const int s = item(Lv.brect_off, it, 0), c0 = item(Lv.brect_off, it, 1);
            const int fs = S.sn_first[s], nc = std::min(NB, W(s) - c0);
            const int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(CH, Lv.maxu));
            const int32_t* rows = &S.sn_rows[S.sn_row_ptr[s]];
            std::vector<double> zs(NB, 0.0), xo(NB, 0.0);
            for (int64_t q0 = W(s); q0 < H(s); q0 += chunk) {
                const int len = (int)std::min<int64_t>(chunk, H(s) - q0);
                if (len > chunk) nerr++;
                for (int jj = 0; jj < nc; jj++) {
                    double a = 0.0;
                    for (int q = 0; q < len; q++) a += Lat(s, (int64_t)(c0 + jj) * H(s) + q0 + q) * Xat(rows[q0 + q]);
                    zs[jj] += a;
                }
            }
            for (int jj = 0; jj < nc; jj++) { const double z = Xat(fs + c0 + jj) - zs[jj]; Tat(s, c0 + jj) = z; zs[jj] = z; }
            if (c0 + nc == W(s)) {
                if (nc > std::min(64, std::max(1, Lv.maxw))) nerr++;     // staged block fits the level's size
                applyXt(s, c0, nc, zs, xo);
                for (int i = 0; i < nc; i++) Xat(fs + c0 + i) = xo[i];
            }
        }
        for (int bb = (int)Lv.btri_cnt.size() - 1; bb >= 1; bb--) {      // k_bwd_tri
            if (!Lv.btri_cnt[bb]) continue;
            launches++;
            for (int it = 0; it < Lv.btri_cnt[bb]; it++) {
                const int s = item(Lv.btri_off[bb], it, 0), c0 = item(Lv.btri_off[bb], it, 1);
                const int fs = S.sn_first[s], b0 = bb * NB, nbb = std::min(NB, W(s) - b0);
                std::vector<double> xb(nbb), zs(NB), xo(NB);
                for (int r = 0; r < nbb; r++) xb[r] = Xat(fs + b0 + r);
                for (int jj = 0; jj < NB; jj++) {
                    double a = 0.0;
                    for (int r = 0; r < nbb; r++) a += Lat(s, (int64_t)(c0 + jj) * H(s) + b0 + r) * xb[r];
                    const double z = Tat(s, c0 + jj) - a;
                    Tat(s, c0 + jj) = z;
                    zs[jj] = z;
                }
                if (c0 + NB == b0) {
                    applyXt(s, c0, NB, zs, xo);
                    for (int i = 0; i < NB; i++) Xat(fs + c0 + i) = xo[i];
                }
            }
        }
    }
    // k_sub_bwd (one warp per task, supernodes root..first)
    if (plan.sub_cnt) launches++;
    for (int it = 0; it < plan.sub_cnt; it++) {
        const int s0 = item(plan.sub_off, it, 0), s1 = item(plan.sub_off, it, 1);
        if (s0 > s1 || s0 < 0 || s1 >= ns) continue;
        for (int s = s1; s >= s0; s--) {
            const int fs = S.sn_first[s], w = W(s);
            const int32_t* rows = &S.sn_rows[S.sn_row_ptr[s]];
            std::vector<double> z(64, 0.0);
            for (int j = 0; j < w; j++) {
                double a = 0.0;
                for (int64_t r = w; r < H(s); r++) a += Lat(s, (int64_t)j * H(s) + r) * Xat(rows[r]);
                z[j] = Xat(fs + j) - a;
            }
            for (int i = 0; i < w; i++) {
                double a = z[i];
                for (int k = i + 1; k < w; k++) a += Lat(s, (int64_t)i * H(s) + k) * z[k];
                Xat(fs + i) = a;
            }
        }
    }
    for (int it = 0; it < plan.sub_cnt; it++)
        for (int s = item(plan.sub_off, it, 0); s <= item(plan.sub_off, it, 1) && s < ns; s++) solved_bwd[s]++;
    for (const SolveLevel& Lv : plan.levels)
        for (int q = 0; q < Lv.gath_cnt; q++) solved_bwd[items[Lv.gath_off + q]]++;
    for (int s = 0; s < ns; s++)
        if (solved_fwd[s] != 1 || solved_bwd[s] != 1) nerr++;
    double err = 0.0, sc = 0.0;
    for (int i = 0; i < n; i++) {
        err = std::max(err, std::fabs(x[i] - xr[i]));
        sc = std::max(sc, std::fabs(xr[i]));
    }
    // independent structure check: the fill of every factor column (its lower pattern in factor
    // numbering united with its children's structures, children taken from that fill) must be
    // inside the rows its supernode's front stores
    long struct_errors = 0;
    int64_t fill = 0;
    {
        std::vector<std::vector<int32_t>> col(n);
        for (int32_t c = 0; c < P.ncols; c++)
            for (int64_t q = P.p[c]; q < P.p[c + 1]; q++) {
                const int32_t i = S.iperm[P.i[q]], j = S.iperm[c];
                if (i != j) col[std::min(i, j)].push_back(std::max(i, j));
            }
        std::vector<std::vector<int32_t>> kids(n);
        std::vector<int32_t> col2sn(n);
        for (int s2 = 0; s2 < ns; s2++)
            for (int j = S.sn_first[s2]; j < S.sn_first[s2 + 1]; j++) col2sn[j] = s2;
        std::vector<char> in_front(n, 0);
        for (int j = 0; j < n; j++) {
            std::vector<int32_t> st = col[j];
            for (int32_t c : kids[j])   // children precede j in factor numbering: col[c] is complete
                for (int32_t r : col[c])
                    if (r > j) st.push_back(r);
            std::sort(st.begin(), st.end());
            st.erase(std::unique(st.begin(), st.end()), st.end());
            col[j] = st;
            fill += (int64_t)st.size();
            if (!st.empty()) kids[st[0]].push_back(j);
            const int s2 = col2sn[j];
            const int32_t* rows = &S.sn_rows[S.sn_row_ptr[s2]];
            const int64_t h = S.sn_row_ptr[s2 + 1] - S.sn_row_ptr[s2];
            for (int64_t r = 0; r < h; r++) in_front[rows[r]] = 1;
            for (int32_t r : st)
                if (!in_front[r]) struct_errors++;
            for (int64_t r = 0; r < h; r++) in_front[rows[r]] = 0;
        }
    }
    if (fill != S.nnz_l) struct_errors++;   // the recomputed fill must be the analysis's nnz(L)
    std::printf("max_rel_err=%.3e bounds_errors=%ld launches=%ld supernodes=%d struct_errors=%ld subtrees=%d "
                "subtree_fronts=%d\n", err / sc, nerr, launches, ns, struct_errors, plan.sub_cnt, plan.sub_fronts);
    return 0;
}
