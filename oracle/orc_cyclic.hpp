// Oracle (test infrastructure only): global assembly and the cyclic-symmetry modal solve.
//   assembly + drop rule ........ src/assembler.cpp:11-289
//   DOF classes / constraints ... src/cyclic_solver.cpp:88-238
//   T(k) ........................ src/cyclic_solver.cpp:240-330
//   static prestress ............ src/cyclic_solver.cpp:456-558 (SparseLU restated as LDL^T:
//                                 the reduced stiffness is symmetric positive definite)
//   projections ................. src/cyclic_solver.cpp:560-723, :858-899
//   per-harmonic solve .......... src/cyclic_solver.cpp:937-1224, pool :1226-1357
//   modal solver front-end ...... src/modal_solver.cpp:12-312
#pragma once
#include <atomic>
#include <mutex>
#include <optional>
#include <set>
#include <thread>

#include "orc_eig.hpp"
#include "orc_fe.hpp"

namespace orc {

constexpr double PI = 3.14159265358979323846;

struct ModalResult {
    int harmonic_index = 0;
    double rpm = 0.0;
    std::vector<double> frequencies;
    std::vector<cd> mode_shapes;     // ndof x m column-major
    std::vector<int> whirl;
    bool converged = true;
    int iterations = 0, steps = 0, num_converged = 0;
};

struct ThreadSolver {               // per-thread symbolic cache (src/cyclic_solver.cpp:1288)
    SimplicialLDL<cd> herm, qep;
    bool herm_set = false, qep_set = false;
};

struct Model {
    int nn = 0, ne = 0;
    std::vector<double> X;            // nn x 3
    std::vector<int> conn;            // ne x 10
    Mat mat{};
    int num_sectors = 0, axis = 2;
    std::vector<int> left, right, hub;
    std::vector<std::pair<int, int>> pairs;
    bool has_constraints = false;
    std::vector<int> interior_dofs, left_dofs, right_dofs;

    // cached / per-rpm state
    CscD K_base, M_base, K_omega, G, K_sigma, K_eff;
    bool base_assembled = false;
    CscZ T0, Kcf, Kpf, Mcf, Mpf, KpfH, MpfH, Gcf, Gpf, GpfH;
    CscD K0r, M0r, Khr, Mhr;
    std::vector<int> free_reduced_map;
    int n_reduced = 0, n_free = 0;
    std::vector<double> u_static;

    int ndof() const { return 3 * nn; }

    void elem_coords(int e, double Xe[10][3]) const {
        for (int a = 0; a < 10; a++) {
            const int nid = conn[(size_t)e * 10 + a];
            for (int c = 0; c < 3; c++) Xe[a][c] = X[(size_t)nid * 3 + c];
        }
    }

    // classify_dofs (cyclic_solver.cpp:214-238)
    void classify() {
        interior_dofs.clear(); left_dofs.clear(); right_dofs.clear();
        std::set<int> ls(left.begin(), left.end()), rs(right.begin(), right.end());
        for (int i = 0; i < nn; i++) {
            const bool isl = ls.count(i) > 0, isr = rs.count(i) > 0;
            for (int d = 0; d < 3; d++) {
                const int dof = 3 * i + d;
                if (isr) right_dofs.push_back(dof);
                else if (isl) left_dofs.push_back(dof);
                else interior_dofs.push_back(dof);
            }
        }
        has_constraints = !hub.empty();
    }

    std::vector<int> constrained_dofs() const {     // FIXED hub group (cyclic_solver.cpp:117-191)
        std::set<int> s;
        for (int nid : hub) { s.insert(3 * nid); s.insert(3 * nid + 1); s.insert(3 * nid + 2); }
        return std::vector<int>(s.begin(), s.end());
    }

    // add_element_matrix drop rule: keep |v| > 1e-15 * max|Ke| (assembler.cpp:274-289)
    static void add_elem(std::vector<Trip<double>>& t, const double Ke[30][30], const int dm[30]) {
        double nrm = 0.0;
        for (int a = 0; a < 30; a++)
            for (int b = 0; b < 30; b++) nrm = std::max(nrm, std::fabs(Ke[a][b]));
        const double tol = 1e-15 * nrm;
        for (int a = 0; a < 30; a++)
            for (int b = 0; b < 30; b++)
                if (std::fabs(Ke[a][b]) > tol) t.push_back({dm[a], dm[b], Ke[a][b]});
    }

    void dofmap(int e, int dm[30]) const {
        for (int a = 0; a < 10; a++) {
            const int nid = conn[(size_t)e * 10 + a];
            dm[3 * a] = 3 * nid; dm[3 * a + 1] = 3 * nid + 1; dm[3 * a + 2] = 3 * nid + 2;
        }
    }

    // kind: 0 = K, 1 = M, 2 = K_omega(omega), 3 = G, 4 = K_sigma(u)
    CscD assemble(int kind, double omega = 0.0, const std::vector<double>* u = nullptr) const {
        std::vector<Trip<double>> t;
        t.reserve((size_t)ne * 900);
        double Xe[10][3], Ke[30][30], sig[14][6], ue[30];
        int dm[30];
        for (int e = 0; e < ne; e++) {
            elem_coords(e, Xe);
            dofmap(e, dm);
            if (kind == 0) stiffness(Xe, mat, Ke);
            else if (kind == 1) mass(Xe, mat, Ke);
            else if (kind == 2) spin_softening(Xe, mat, omega, axis, Ke);
            else if (kind == 3) gyroscopic(Xe, mat, axis, Ke);
            else {
                for (int a = 0; a < 30; a++) ue[a] = (*u)[dm[a]];
                prestress14(Xe, mat, ue, sig);
                stress_stiffening(Xe, sig, Ke);
            }
            add_elem(t, Ke, dm);
        }
        return from_triplets<double>(ndof(), ndof(), t);
    }

    std::vector<double> centrifugal_load(double omega) const {   // assembler.cpp:220-272
        std::vector<double> F(ndof(), 0.0);
        double Xe[10][3], Fe[30];
        int dm[30];
        for (int e = 0; e < ne; e++) {
            elem_coords(e, Xe);
            dofmap(e, dm);
            centrifugal(Xe, mat, omega, axis, Fe);
            for (int a = 0; a < 30; a++) F[dm[a]] += Fe[a];
        }
        return F;
    }

    // build_cyclic_transformation (cyclic_solver.cpp:240-330)
    CscZ transformation(int k) const {
        const int full = ndof();
        const int red = (int)(interior_dofs.size() + left_dofs.size());
        const double alpha = 2.0 * PI / num_sectors;
        const cd phase(std::cos(k * alpha), std::sin(k * alpha));
        std::vector<int> f2r(full, -1);
        int idx = 0;
        for (int d : interior_dofs) f2r[d] = idx++;
        for (int d : left_dofs) f2r[d] = idx++;
        std::vector<int> r2l(nn, -1);
        for (auto& pr : pairs) r2l[pr.second] = pr.first;
        std::vector<Trip<cd>> t;
        t.reserve(full);
        for (int d : interior_dofs) t.push_back({d, f2r[d], cd(1.0, 0.0)});
        for (int d : left_dofs) t.push_back({d, f2r[d], cd(1.0, 0.0)});
        const double ca = std::cos(alpha), sa = std::sin(alpha);
        int c1, c2, cax;
        if (axis == 0) { c1 = 1; c2 = 2; cax = 0; }
        else if (axis == 1) { c1 = 0; c2 = 2; cax = 1; }
        else { c1 = 0; c2 = 1; cax = 2; }
        std::vector<char> done(nn, 0);
        for (int rd : right_dofs) {
            const int rn = rd / 3;
            if (done[rn]) continue;
            done[rn] = 1;
            const int ln = r2l[rn];
            if (ln < 0) throw std::runtime_error("Right boundary node has no matched left partner");
            const int rb = 3 * rn;
            const int l1 = f2r[3 * ln + c1], l2 = f2r[3 * ln + c2], lax = f2r[3 * ln + cax];
            t.push_back({rb + c1, l1, phase * ca});
            t.push_back({rb + c1, l2, phase * (-sa)});
            t.push_back({rb + c2, l1, phase * sa});
            t.push_back({rb + c2, l2, phase * ca});
            t.push_back({rb + cax, lax, phase});
        }
        return from_triplets<cd>(full, red, t);
    }

    void base() {
        if (base_assembled) return;
        K_base = assemble(0);
        M_base = assemble(1);
        base_assembled = true;
    }

    // static_centrifugal (cyclic_solver.cpp:456-558)
    std::vector<double> static_centrifugal(double omega) {
        std::vector<double> F = centrifugal_load(omega);
        const CscD& K = K_base;
        CscZ Tc = transformation(0);
        const int red = Tc.cols;
        std::vector<Trip<double>> tr;
        for (int c = 0; c < Tc.cols; c++)
            for (int q = Tc.p[c]; q < Tc.p[c + 1]; q++) {
                const double rv = Tc.x[q].real();
                if (std::fabs(rv) > 1e-15) tr.push_back({Tc.i[q], c, rv});
            }
        CscD Tr = from_triplets<double>(ndof(), red, tr);
        CscD TrT = transpose(Tr, false);
        CscD Kc = multiply(multiply(TrT, K, false, 0.0), Tr, true, 1e-15 * 1e-12);
        std::vector<double> Fc(red, 0.0);
        spmv(TrT, F.data(), Fc.data());
        std::vector<int> r2f;
        for (int d : interior_dofs) r2f.push_back(d);
        for (int d : left_dofs) r2f.push_back(d);
        std::vector<int> cons = constrained_dofs();
        std::set<int> cs(cons.begin(), cons.end());
        std::vector<int> freec, c2f(red, -1);
        for (int i = 0; i < red; i++)
            if (!cs.count(r2f[i])) { c2f[i] = (int)freec.size(); freec.push_back(i); }
        const int nf = (int)freec.size();
        if (nf == 0) return std::vector<double>(ndof(), 0.0);
        std::vector<Trip<double>> tk;
        for (int c = 0; c < Kc.cols; c++)
            for (int q = Kc.p[c]; q < Kc.p[c + 1]; q++) {
                const int ri = c2f[Kc.i[q]], rj = c2f[c];
                if (ri >= 0 && rj >= 0) tk.push_back({ri, rj, Kc.x[q]});
            }
        CscD Kf = from_triplets<double>(nf, nf, tk);
        std::vector<double> Ff(nf), uf(nf);
        for (int i = 0; i < nf; i++) Ff[i] = Fc[freec[i]];
        SimplicialLDL<double> ldl;
        ldl.analyze(Kf);
        if (!ldl.factorize(Kf)) throw std::runtime_error("static solve failed");
        ldl.solve(Ff.data(), uf.data());
        std::vector<double> uc(red, 0.0), u(ndof(), 0.0);
        for (int i = 0; i < nf; i++) uc[freec[i]] = uf[i];
        spmv(Tr, uc.data(), u.data());
        return u;
    }

    // partition by right-DOF membership (cyclic_solver.cpp:606-623)
    std::pair<CscZ, CscZ> partition(const CscZ& A, const std::vector<char>& isr) const {
        std::vector<Trip<cd>> ts, tnr;
        for (int c = 0; c < A.cols; c++) {
            const bool cr = isr[c];
            for (int q = A.p[c]; q < A.p[c + 1]; q++) {
                const bool rr = isr[A.i[q]];
                if (rr == cr) ts.push_back({A.i[q], c, A.x[q]});
                else if (!rr && cr) tnr.push_back({A.i[q], c, A.x[q]});
            }
        }
        return {from_triplets<cd>(A.rows, A.cols, ts), from_triplets<cd>(A.rows, A.cols, tnr)};
    }

    CscZ extract_free(const CscZ& A, const std::vector<int>& r2fv) const {
        std::vector<Trip<cd>> t;
        for (int c = 0; c < A.cols; c++) {
            const int rj = r2fv[c];
            if (rj < 0) continue;
            for (int q = A.p[c]; q < A.p[c + 1]; q++) {
                const int ri = r2fv[A.i[q]];
                if (ri >= 0) t.push_back({ri, rj, A.x[q]});
            }
        }
        return from_triplets<cd>(n_free, n_free, t);
    }

    std::vector<int> reduced_to_free() const {
        std::vector<int> v(n_reduced, -1);
        for (int i = 0; i < (int)free_reduced_map.size(); i++) v[free_reduced_map[i]] = i;
        return v;
    }

    std::pair<CscZ, CscZ> project_pair(const CscD& A, const std::vector<char>& isr) {
        CscZ Ac = to_complex(A);
        auto [As, Anr] = partition(Ac, isr);
        CscZ T0H = transpose(T0, true);
        CscZ cp = multiply(multiply(T0H, As, false, 0.0), T0, true, 1e-27);
        CscZ pp = multiply(multiply(T0H, Anr, false, 0.0), T0, true, 1e-27);
        auto r2fv = reduced_to_free();
        return {extract_free(cp, r2fv), extract_free(pp, r2fv)};
    }

    static CscD real_filter(const CscZ& A) {
        std::vector<Trip<double>> t;
        for (int c = 0; c < A.cols; c++)
            for (int q = A.p[c]; q < A.p[c + 1]; q++)
                if (std::fabs(A.x[q].real()) > 1e-15) t.push_back({A.i[q], c, A.x[q].real()});
        return from_triplets<double>(A.rows, A.cols, t);
    }

    // precompute_cyclic_projections + precompute_real_matrices (cyclic_solver.cpp:560-723)
    void projections(const CscD& Keff, const CscD& Msec) {
        std::vector<int> cons = constrained_dofs();
        std::set<int> cs(cons.begin(), cons.end());
        std::vector<int> r2f;
        for (int d : interior_dofs) r2f.push_back(d);
        for (int d : left_dofs) r2f.push_back(d);
        T0 = transformation(0);
        n_reduced = T0.cols;
        free_reduced_map.clear();
        for (int i = 0; i < n_reduced; i++)
            if (!cs.count(r2f[i])) free_reduced_map.push_back(i);
        n_free = (int)free_reduced_map.size();
        std::vector<char> isr(ndof(), 0);
        for (int d : right_dofs) isr[d] = 1;
        std::tie(Kcf, Kpf) = project_pair(Keff, isr);
        std::tie(Mcf, Mpf) = project_pair(Msec, isr);
        KpfH = transpose(Kpf, true);
        MpfH = transpose(Mpf, true);
        K0r = real_filter(add<cd>(add<cd>(Kcf, 1.0, Kpf, 1.0), 1.0, KpfH, 1.0));
        M0r = real_filter(add<cd>(add<cd>(Mcf, 1.0, Mpf, 1.0), 1.0, MpfH, 1.0));
        if (num_sectors % 2 == 0 && num_sectors / 2 > 0) {
            Khr = real_filter(add<cd>(add<cd>(Kcf, 1.0, Kpf, -1.0), 1.0, KpfH, -1.0));
            Mhr = real_filter(add<cd>(add<cd>(Mcf, 1.0, Mpf, -1.0), 1.0, MpfH, -1.0));
        }
    }

    // Steps 1-3 of solve_at_rpm (cyclic_solver.cpp:735-899)
    void prepare(double rpm, bool coriolis) {
        const double omega = rpm * 2.0 * PI / 60.0;
        base();
        K_eff = K_base;
        if (std::fabs(omega) > 0.0) {
            K_omega = assemble(2, omega);
            G = assemble(3);
            K_eff = add<double>(K_base, 1.0, K_omega, -1.0);
            if (has_constraints) {
                u_static = static_centrifugal(omega);
                K_sigma = assemble(4, omega, &u_static);
                K_eff = add<double>(K_eff, 1.0, K_sigma, 1.0);
            }
        }
        projections(K_eff, M_base);
        if (coriolis && std::fabs(omega) > 0.0) {
            std::vector<char> isr(ndof(), 0);
            for (int d : right_dofs) isr[d] = 1;
            std::tie(Gcf, Gpf) = project_pair(G, isr);
            GpfH = transpose(Gpf, true);
        }
    }

    CscZ k_operator(const CscZ& c, const CscZ& p, const CscZ& pH, int k) const {
        const double alpha = 2.0 * PI / num_sectors;
        const cd P(std::cos(k * alpha), std::sin(k * alpha));
        return add<cd>(add<cd>(c, 1.0, p, P), 1.0, pH, std::conj(P));
    }

    std::optional<ModalResult> solve_harmonic(int k, double rpm, int num_modes, bool coriolis_active,
                                              double min_frequency, ThreadSolver& ts);
};

// solve_real (modal_solver.cpp:12-94) with the Spectra IRL restated by the same Lanczos
inline std::pair<ModalResult, bool> solve_real(const CscD& K, const CscD& M, const LanczosConfig& c0,
                                               int* iters) {
    ModalResult r;
    const int n = K.rows;
    LanczosConfig c = c0;
    c.nev = std::min(c0.nev, n - 1);
    c.max_iterations = 1000;
    auto res = lanczos_solve<double>(K, M, c);
    *iters = res.restarts;
    const int m = res.nconv;
    std::vector<int> idx(m);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return res.eigenvalues[a] < res.eigenvalues[b]; });
    r.frequencies.resize(m);
    r.mode_shapes.resize((size_t)n * m);
    for (int t = 0; t < m; t++) {
        const double lam = res.eigenvalues[idx[t]];
        r.frequencies[t] = lam > 0.0 ? std::sqrt(lam) / (2.0 * PI) : 0.0;
        for (int i = 0; i < n; i++) r.mode_shapes[(size_t)t * n + i] = cd(res.vectors[(size_t)idx[t] * n + i], 0.0);
    }
    r.whirl.assign(m, 0);
    r.num_converged = m;
    r.converged = res.converged;
    return {r, res.converged};
}

// solve_complex_hermitian (modal_solver.cpp:96-147)
inline std::pair<ModalResult, bool> solve_complex(const CscZ& K, const CscZ& M, const LanczosConfig& c0,
                                                  int* iters) {
    ModalResult r;
    const int n = K.rows;
    LanczosConfig c = c0;
    c.nev = std::min(c0.nev, n - 1);
    c.max_iterations = 1000;
    auto res = lanczos_solve<cd>(K, M, c);
    *iters = res.restarts;
    const int m = res.nconv;
    r.frequencies.resize(m);
    r.mode_shapes.assign(res.vectors.begin(), res.vectors.end());
    for (int t = 0; t < m; t++) {
        const double lam = res.eigenvalues[t];
        r.frequencies[t] = lam > 0.0 ? std::sqrt(lam) / (2.0 * PI) : 0.0;
    }
    r.whirl.assign(m, 0);
    r.num_converged = m;
    r.converged = res.converged;
    return {r, res.converged};
}

// solve_lancaster_qep (modal_solver.cpp:151-312)
inline std::pair<ModalResult, bool> solve_qep(const CscZ& K, const CscZ& M, const CscZ& D, int num_modes,
                                              double shift_cfg, int* iters, int* nconv_out) {
    ModalResult r;
    const int n = K.rows, n2 = 2 * n;
    std::vector<Trip<cd>> t1, t2;
    for (int c = 0; c < n; c++) {
        for (int q = D.p[c]; q < D.p[c + 1]; q++) t1.push_back({D.i[q], c, D.x[q]});
        for (int q = K.p[c]; q < K.p[c + 1]; q++) t1.push_back({K.i[q], c + n, K.x[q]});
        for (int q = K.p[c]; q < K.p[c + 1]; q++) t1.push_back({K.i[q] + n, c, K.x[q]});
        for (int q = M.p[c]; q < M.p[c + 1]; q++) t2.push_back({M.i[q], c, M.x[q]});
        for (int q = K.p[c]; q < K.p[c + 1]; q++) t2.push_back({K.i[q] + n, c + n, K.x[q]});
    }
    CscZ L1 = from_triplets<cd>(n2, n2, t1), L2 = from_triplets<cd>(n2, n2, t2);
    const int nev_req = n2 <= 200 ? n2 - 1 : std::min(6 * num_modes, n2 - 1);
    *nconv_out = 0;
    if (nev_req <= 0) return {r, false};
    LanczosConfig c;
    c.nev = nev_req;
    c.ncv = std::min(std::max(4 * nev_req + 1, 40), n2);
    c.shift = shift_cfg > 0 ? std::sqrt(shift_cfg) : 0.1;
    c.tolerance = 1e-8;
    c.max_iterations = 20;
    auto res = lanczos_solve<cd>(L1, L2, c);
    *iters = res.restarts;
    if (res.nconv == 0) return {r, false};
    struct E { double om; int idx; int wh; };
    std::vector<E> ent;
    for (int i = 0; i < res.nconv; i++) {
        const double om = res.eigenvalues[i];
        if (std::fabs(om) < 1e-6) continue;
        ent.push_back({om, i, om > 0 ? 1 : -1});
    }
    auto byabs = [](const E& a, const E& b) { return std::fabs(a.om) < std::fabs(b.om); };
    std::sort(ent.begin(), ent.end(), byabs);
    int nfw = 0, nbw = 0;
    std::vector<E> sel;
    for (auto& e : ent) {
        if (e.wh == 1 && nfw < num_modes) { sel.push_back(e); nfw++; }
        else if (e.wh == -1 && nbw < num_modes) { sel.push_back(e); nbw++; }
        if (nfw >= num_modes && nbw >= num_modes) break;
    }
    std::sort(sel.begin(), sel.end(), byabs);
    const int m = (int)sel.size();
    r.frequencies.resize(m);
    r.whirl.resize(m);
    r.mode_shapes.resize((size_t)n * m);
    for (int t = 0; t < m; t++) {
        r.frequencies[t] = std::fabs(sel[t].om) / (2.0 * PI);
        r.whirl[t] = sel[t].wh;
        for (int i = 0; i < n; i++) r.mode_shapes[(size_t)t * n + i] = res.vectors[(size_t)sel[t].idx * n2 + i];
    }
    *nconv_out = m;
    r.num_converged = m;
    r.converged = res.converged;
    return {r, res.converged};
}

inline std::optional<ModalResult> Model::solve_harmonic(int k, double rpm, int num_modes, bool coriolis_active,
                                                        double min_frequency, ThreadSolver& ts) {
    (void)ts;
    try {
        if (n_free <= 1) return std::nullopt;
        const double alpha = 2.0 * PI / num_sectors;
        const cd P(std::cos(k * alpha), std::sin(k * alpha));
        const int max_k = num_sectors / 2;
        const double omega = rpm * 2.0 * PI / 60.0;
        CscZ Kf = k_operator(Kcf, Kpf, KpfH, k);
        CscZ Mf = k_operator(Mcf, Mpf, MpfH, k);
        const bool is_degenerate = (k > 0) && !(num_sectors % 2 == 0 && k == max_k);
        const bool will_qep = coriolis_active && k > 0;
        const int nev_target = (is_degenerate && !will_qep) ? (num_modes + 1) / 2 : num_modes;
        ModalResult res;
        bool conv = false;
        bool used_qep = false;
        int iters = 0;
        int numc = 0;
        if (will_qep) {
            CscZ Gf = k_operator(Gcf, Gpf, GpfH, k);
            CscZ Df = scale<cd>(Gf, cd(0.0, 2.0 * omega));
            const double kn = fro(Kf), mn = fro(Mf);
            const double shift = mn > 0 ? kn / mn : 1.0;
            auto pr = solve_qep(Kf, Mf, Df, nev_target, shift, &iters, &numc);
            res = pr.first; conv = pr.second;
            used_qep = true;
        } else {
            const int n_extra = min_frequency > 0.0 ? 6 : 0;
            LanczosConfig c;
            c.nev = std::min(nev_target + n_extra, n_free - 1);
            if (c.nev <= 0) return std::nullopt;
            c.ncv = std::min(std::max(4 * c.nev + 1, 40), n_free);
            c.shift = 1.0;
            const bool is_real = (k == 0) || (num_sectors % 2 == 0 && k == max_k);
            if (is_real) {
                auto pr = solve_real(k == 0 ? K0r : Khr, k == 0 ? M0r : Mhr, c, &iters);
                res = pr.first; conv = pr.second;
            } else {
                auto pr = solve_complex(Kf, Mf, c, &iters);
                res = pr.first; conv = pr.second;
            }
            numc = res.num_converged;
        }
        if (!conv && numc == 0) return std::nullopt;
        const int nrows = n_free;
        if (min_frequency > 0.0) {
            std::vector<int> keep;
            for (int m = 0; m < (int)res.frequencies.size(); m++)
                if (res.frequencies[m] > min_frequency) keep.push_back(m);
            if (keep.size() < res.frequencies.size()) {
                if (keep.empty()) return std::nullopt;
                ModalResult nr = res;
                nr.frequencies.clear(); nr.whirl.clear(); nr.mode_shapes.clear();
                for (int m : keep) {
                    nr.frequencies.push_back(res.frequencies[m]);
                    nr.whirl.push_back(m < (int)res.whirl.size() ? res.whirl[m] : 0);
                    nr.mode_shapes.insert(nr.mode_shapes.end(), res.mode_shapes.begin() + (size_t)m * nrows,
                                          res.mode_shapes.begin() + (size_t)(m + 1) * nrows);
                }
                res = nr;
            }
        }
        if ((int)res.frequencies.size() > nev_target) {
            res.frequencies.resize(nev_target);
            res.whirl.resize(nev_target);
            res.mode_shapes.resize((size_t)nev_target * nrows);
        }
        if (!used_qep) res.whirl.assign(res.frequencies.size(), 0);
        if (is_degenerate && !used_qep) {
            const int nu = (int)res.frequencies.size();
            const int nx = std::min(2 * nu, num_modes);
            ModalResult ex = res;
            ex.frequencies.resize(nx); ex.whirl.resize(nx); ex.mode_shapes.resize((size_t)nx * nrows);
            for (int m = 0; m < nx; m++) {
                const int src = m / 2;
                ex.frequencies[m] = res.frequencies[src];
                for (int i = 0; i < nrows; i++) {
                    const cd v = res.mode_shapes[(size_t)src * nrows + i];
                    ex.mode_shapes[(size_t)m * nrows + i] = (m % 2 == 0) ? v : std::conj(v);
                }
                ex.whirl[m] = (m % 2 == 0) ? 1 : -1;
            }
            res = ex;
        }
        // expansion: u_full = T0 u_reduced, right rows * P (cyclic_solver.cpp:1185-1211)
        const int nm = (int)res.frequencies.size();
        std::vector<cd> full((size_t)ndof() * nm, cd(0.0));
        std::vector<cd> red(n_reduced), out(ndof());
        std::vector<char> isr(ndof(), 0);
        for (int d : right_dofs) isr[d] = 1;
        for (int m = 0; m < nm; m++) {
            std::fill(red.begin(), red.end(), cd(0.0));
            for (int i = 0; i < nrows && i < (int)free_reduced_map.size(); i++)
                red[free_reduced_map[i]] = res.mode_shapes[(size_t)m * nrows + i];
            spmv(T0, red.data(), out.data());
            for (int r = 0; r < ndof(); r++) full[(size_t)m * ndof() + r] = isr[r] ? out[r] * P : out[r];
        }
        res.mode_shapes = full;
        res.harmonic_index = k;
        res.rpm = rpm;
        res.converged = conv;
        res.iterations = iters;
        return res;
    } catch (const std::exception&) {
        return std::nullopt;
    }
}

// solve_at_rpm (cyclic_solver.cpp:725-1357) with the std::thread pool over harmonics
inline std::vector<ModalResult> solve_at_rpm(Model& md, double rpm, int num_modes, const std::vector<int>& hi,
                                             int max_threads, bool coriolis, double min_frequency) {
    const double omega = rpm * 2.0 * PI / 60.0;
    md.prepare(rpm, coriolis);
    const bool cor_active = coriolis && std::fabs(omega) > 0.0;
    const int max_k = md.num_sectors / 2;
    std::vector<int> hs;
    if (hi.empty()) for (int k = 0; k <= max_k; k++) hs.push_back(k);
    else for (int k : hi) if (k >= 0 && k <= max_k) hs.push_back(k);
    const int nh = (int)hs.size();
    int nt = max_threads > 0 ? max_threads : std::max(1, (int)std::thread::hardware_concurrency());
    nt = std::min(nt, nh);
    std::vector<std::optional<ModalResult>> out(nh);
    std::atomic<int> next{0};
    std::vector<int> failed;
    std::mutex mu;
    std::vector<std::thread> workers;
    for (int w = 0; w < nt; w++)
        workers.emplace_back([&]() {
            ThreadSolver ts;
            while (true) {
                const int idx = next.fetch_add(1);
                if (idx >= nh) break;
                out[idx] = md.solve_harmonic(hs[idx], rpm, num_modes, cor_active, min_frequency, ts);
                if (!out[idx]) { std::lock_guard<std::mutex> lk(mu); failed.push_back(idx); }
            }
        });
    for (auto& t : workers) t.join();
    if (!failed.empty()) {
        ThreadSolver ts;
        for (int idx : failed) out[idx] = md.solve_harmonic(hs[idx], rpm, num_modes, cor_active, min_frequency, ts);
    }
    std::vector<ModalResult> res;
    for (auto& o : out) if (o) res.push_back(std::move(*o));
    std::sort(res.begin(), res.end(), [](const ModalResult& a, const ModalResult& b) {
        return a.harmonic_index < b.harmonic_index; });
    return res;
}

}  // namespace orc
