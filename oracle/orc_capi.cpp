// Oracle (test infrastructure only): C entry points over the CPU restatement, loaded with
// ctypes by tests/, by the smoke check and by the bench's CPU-baseline leg.  The product
// library never links or loads this file.
#include <cstring>

#include "orc_cyclic.hpp"
#include "orc_window.hpp"

using namespace orc;

namespace {
struct Handle {
    Model m;
    CscD rd;
    CscZ zd;
    bool is_complex = false;
    std::vector<ModalResult> results;
};

template <typename T>
void set_out(Handle* h, const Csc<T>& A);
template <>
void set_out(Handle* h, const CscD& A) { h->rd = A; h->is_complex = false; }
template <>
void set_out(Handle* h, const CscZ& A) { h->zd = A; h->is_complex = true; }

CscZ csc_z(int n, const int* p, const int* i, const double* x) {
    CscZ A;
    A.rows = A.cols = n;
    A.p.assign(p, p + n + 1);
    A.i.assign(i, i + p[n]);
    A.x.resize(p[n]);
    for (int k = 0; k < p[n]; k++) A.x[k] = cd(x[2 * k], x[2 * k + 1]);
    return A;
}
}  // namespace

extern "C" {

void* orc_model_create(int nn, const double* X, int ne, const int* conn, double E, double nu, double rho,
                       int num_sectors, int axis, int nleft, const int* left, int nright, const int* right,
                       int npairs, const int* pairs, int nhub, const int* hub) {
    auto* h = new Handle();
    Model& m = h->m;
    m.nn = nn; m.ne = ne;
    m.X.assign(X, X + (size_t)3 * nn);
    m.conn.assign(conn, conn + (size_t)10 * ne);
    m.mat = Mat{E, nu, rho};
    m.num_sectors = num_sectors;
    m.axis = axis;
    m.left.assign(left, left + nleft);
    m.right.assign(right, right + nright);
    for (int k = 0; k < npairs; k++) m.pairs.push_back({pairs[2 * k], pairs[2 * k + 1]});
    m.hub.assign(hub, hub + nhub);
    m.classify();
    return h;
}

void orc_model_free(void* h) { delete static_cast<Handle*>(h); }

// kind: 0 K, 1 M, 2 K_omega, 3 G, 4 K_sigma(ue), 5 centrifugal load (out30)
void orc_element(const double* X30, double E, double nu, double rho, int kind, double omega, int axis,
                 const double* ue, double* out) {
    double Xe[10][3], Ke[30][30], sig[14][6];
    for (int a = 0; a < 10; a++)
        for (int c = 0; c < 3; c++) Xe[a][c] = X30[3 * a + c];
    Mat mt{E, nu, rho};
    if (kind == 5) { centrifugal(Xe, mt, omega, axis, out); return; }
    if (kind == 0) stiffness(Xe, mt, Ke);
    else if (kind == 1) mass(Xe, mt, Ke);
    else if (kind == 2) spin_softening(Xe, mt, omega, axis, Ke);
    else if (kind == 3) gyroscopic(Xe, mt, axis, Ke);
    else { prestress14(Xe, mt, ue, sig); stress_stiffening(Xe, sig, Ke); }
    for (int a = 0; a < 30; a++)
        for (int b = 0; b < 30; b++) out[a * 30 + b] = Ke[a][b];
}

int orc_prepare(void* hv, double rpm, int coriolis) {
    auto* h = static_cast<Handle*>(hv);
    try { h->m.prepare(rpm, coriolis != 0); } catch (...) { return -1; }
    return 0;
}

// Matrix selector (see the tests for the meaning of each code).  Returns nnz, -1 on error.
long long orc_matrix(void* hv, int which, double param, int k) {
    auto* h = static_cast<Handle*>(hv);
    Model& m = h->m;
    try {
        switch (which) {
            case 0: m.base(); set_out(h, m.K_base); break;
            case 1: m.base(); set_out(h, m.M_base); break;
            case 2: set_out(h, m.assemble(2, param)); break;
            case 3: set_out(h, m.assemble(3)); break;
            case 4: set_out(h, m.K_sigma); break;
            case 5: set_out(h, m.K_eff); break;
            case 6: set_out(h, m.transformation(k)); break;
            case 10: set_out(h, m.Kcf); break;
            case 11: set_out(h, m.Kpf); break;
            case 12: set_out(h, m.Mcf); break;
            case 13: set_out(h, m.Mpf); break;
            case 14: set_out(h, m.Gcf); break;
            case 15: set_out(h, m.Gpf); break;
            case 20: set_out(h, m.K0r); break;
            case 21: set_out(h, m.M0r); break;
            case 22: set_out(h, m.Khr); break;
            case 23: set_out(h, m.Mhr); break;
            case 30: set_out(h, m.k_operator(m.Kcf, m.Kpf, m.KpfH, k)); break;
            case 31: set_out(h, m.k_operator(m.Mcf, m.Mpf, m.MpfH, k)); break;
            case 32: set_out(h, m.k_operator(m.Gcf, m.Gpf, m.GpfH, k)); break;
            default: return -1;
        }
    } catch (...) { return -1; }
    return h->is_complex ? h->zd.nnz() : h->rd.nnz();
}

void orc_matrix_shape(void* hv, int* rows, int* cols, int* is_complex) {
    auto* h = static_cast<Handle*>(hv);
    *is_complex = h->is_complex;
    *rows = h->is_complex ? h->zd.rows : h->rd.rows;
    *cols = h->is_complex ? h->zd.cols : h->rd.cols;
}

void orc_matrix_copy(void* hv, int* p, int* i, double* x) {
    auto* h = static_cast<Handle*>(hv);
    if (h->is_complex) {
        std::memcpy(p, h->zd.p.data(), sizeof(int) * h->zd.p.size());
        std::memcpy(i, h->zd.i.data(), sizeof(int) * h->zd.i.size());
        std::memcpy(x, h->zd.x.data(), sizeof(double) * 2 * h->zd.x.size());
    } else {
        std::memcpy(p, h->rd.p.data(), sizeof(int) * h->rd.p.size());
        std::memcpy(i, h->rd.i.data(), sizeof(int) * h->rd.i.size());
        std::memcpy(x, h->rd.x.data(), sizeof(double) * h->rd.x.size());
    }
}

void orc_centrifugal(void* hv, double omega, double* F) {
    auto* h = static_cast<Handle*>(hv);
    auto v = h->m.centrifugal_load(omega);
    std::memcpy(F, v.data(), sizeof(double) * v.size());
}

int orc_static_u(void* hv, double* u) {
    auto* h = static_cast<Handle*>(hv);
    if (h->m.u_static.empty()) return -1;
    std::memcpy(u, h->m.u_static.data(), sizeof(double) * h->m.u_static.size());
    return 0;
}

int orc_free_map(void* hv, int* out) {
    auto* h = static_cast<Handle*>(hv);
    if (out) std::memcpy(out, h->m.free_reduced_map.data(), sizeof(int) * h->m.free_reduced_map.size());
    return h->m.n_free;
}

// AMD order, elimination tree and column counts of the Hermitian matrix whose lower
// triangle is (p, i) (values unused).  perm[k] = original index of pivot k.
void orc_ldl_symbolic(int n, const int* p, const int* i, int* perm, int* parent, int* colcount) {
    CscD A;
    A.rows = A.cols = n;
    A.p.assign(p, p + n + 1);
    A.i.assign(i, i + p[n]);
    A.x.assign(p[n], 1.0);
    SimplicialLDL<double> ldl;
    ldl.analyze(A);
    std::memcpy(perm, ldl.Pinv.data(), sizeof(int) * n);
    std::memcpy(parent, ldl.parent.data(), sizeof(int) * n);
    std::memcpy(colcount, ldl.colcount.data(), sizeof(int) * n);
}

// Hermitian Lanczos on caller matrices (complex interleaved values).  vecs: n x nev.
int orc_lanczos_z(int n, const int* Kp, const int* Ki, const double* Kx, const int* Mp, const int* Mi,
                  const double* Mx, int nev, int ncv, double shift, double tol, int maxit, double* evals,
                  double* vecs, int* info) {
    CscZ K = csc_z(n, Kp, Ki, Kx), M = csc_z(n, Mp, Mi, Mx);
    LanczosConfig c;
    c.nev = nev; c.ncv = ncv; c.shift = shift; c.tolerance = tol; c.max_iterations = maxit;
    auto r = lanczos_solve<cd>(K, M, c);
    for (int t = 0; t < r.nconv; t++) evals[t] = r.eigenvalues[t];
    std::memcpy(vecs, r.vectors.data(), sizeof(double) * 2 * r.vectors.size());
    info[0] = r.nconv; info[1] = r.converged; info[2] = r.restarts; info[3] = r.steps;
    return r.nconv;
}

int orc_solve(void* hv, double rpm, int num_modes, int nhi, const int* hi, int max_threads, int coriolis,
              double min_frequency) {
    auto* h = static_cast<Handle*>(hv);
    std::vector<int> hv2(hi, hi + nhi);
    try {
        h->results = solve_at_rpm(h->m, rpm, num_modes, hv2, max_threads, coriolis != 0, min_frequency);
    } catch (...) { return -1; }
    return (int)h->results.size();
}

void orc_result_info(void* hv, int idx, int* info, double* rpm) {
    auto* h = static_cast<Handle*>(hv);
    const ModalResult& r = h->results[idx];
    info[0] = r.harmonic_index;
    info[1] = (int)r.frequencies.size();
    info[2] = r.converged;
    info[3] = r.iterations;
    *rpm = r.rpm;
}

void orc_result_copy(void* hv, int idx, double* freqs, double* shapes, int* whirl) {
    auto* h = static_cast<Handle*>(hv);
    const ModalResult& r = h->results[idx];
    std::memcpy(freqs, r.frequencies.data(), sizeof(double) * r.frequencies.size());
    if (shapes) std::memcpy(shapes, r.mode_shapes.data(), sizeof(double) * 2 * r.mode_shapes.size());
    std::memcpy(whirl, r.whirl.data(), sizeof(int) * r.whirl.size());
}

// ---- timing samples of the reference's factorisation (orc_window.hpp) ----
// Operator given by its lower triangle (CSC, complex interleaved values).
void* orc_lw_create(int n, const int* p, const int* i, const double* x) {
    auto* w = new LdlWindows();
    try {
        w->analyze(csc_z(n, p, i, x));
    } catch (...) { delete w; return nullptr; }
    return w;
}

int orc_lw_add_slot(void* h) {
    auto* w = static_cast<LdlWindows*>(h);
    try {
        w->add_slot();
    } catch (...) { return -1; }
    return (int)w->slots.size();
}

void orc_lw_free(void* h) { delete static_cast<LdlWindows*>(h); }

// out: [0] n, [1] nnz(L), [2] total inner-loop updates, [3] slots
void orc_lw_info(void* h, double* out) {
    auto* w = static_cast<LdlWindows*>(h);
    out[0] = w->n;
    out[1] = (double)w->nnz_l();
    out[2] = (double)w->cum[w->n];
    out[3] = (double)w->slots.size();
}

// cum[0..n]: inner-loop updates of the rows before each row
void orc_lw_cumwork(void* h, long long* cum) {
    auto* w = static_cast<LdlWindows*>(h);
    for (int k = 0; k <= w->n; k++) cum[k] = w->cum[k];
}

void orc_lw_run(void* h, int nt, const int* slot, const int* a, const int* b, double* t_fact, double* t_solve) {
    static_cast<LdlWindows*>(h)->run(nt, slot, a, b, t_fact, t_solve);
}

}  // extern "C"
