// Host runtime of the GB300 cyclic modal solve: device buffers, the sector model, sector
// assembly on the candidate pattern, cyclic projections and the per-harmonic operators.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "common.cuh"
#include "lz.cuh"
#include "mf.cuh"
#include "sym.hpp"

namespace tmg {

// Owning device array.
template <typename T>
struct DVec {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t s_ = nullptr;       // stream the buffer was allocated on (freed in its order)
    ByteCount* cnt_ = nullptr;       // the owning context's byte count
    DVec() = default;
    DVec(const DVec&) = delete;
    DVec& operator=(const DVec&) = delete;
    DVec(DVec&& o) noexcept : p(o.p), n(o.n), s_(o.s_), cnt_(o.cnt_) { o.p = nullptr; o.n = 0; o.cnt_ = nullptr; }
    DVec& operator=(DVec&& o) noexcept {
        release();
        p = o.p; n = o.n; s_ = o.s_; cnt_ = o.cnt_;
        o.p = nullptr; o.n = 0; o.cnt_ = nullptr;
        return *this;
    }
    ~DVec() { release(); }
    // stream-ordered allocation on the calling context's stream
    void alloc(size_t count) {
        if (count == n && p) return;
        release();
        n = count;
        s_ = g_stream;
        if (count) {
            TMG_CUDA(pool_malloc((void**)&p, count * sizeof(T), s_));
            cnt_ = g_bytes;
            if (cnt_) cnt_->add((int64_t)(count * sizeof(T)));
        }
    }
    void zero(cudaStream_t st) { if (n) TMG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), st)); }
    void upload(const std::vector<T>& h) {
        alloc(h.size());
        if (n) {
            TMG_CUDA(cudaMemcpyAsync(p, h.data(), n * sizeof(T), cudaMemcpyHostToDevice, s_));
            TMG_CUDA(cudaStreamSynchronize(s_));
        }
    }
    std::vector<T> download() const {
        std::vector<T> h(n);
        if (n) {
            cudaStream_t st = s_ ? s_ : g_stream;
            TMG_CUDA(cudaMemcpyAsync(h.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost, st));
            TMG_CUDA(cudaStreamSynchronize(st));
        }
        return h;
    }
    void release() {
        if (p) {
            cudaFreeAsync(p, s_);
            if (cnt_) cnt_->cur -= (int64_t)(n * sizeof(T));
        }
        p = nullptr;
        n = 0;
        cnt_ = nullptr;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// A sector matrix on the candidate pattern: values and membership flags.
struct CandMat {
    DVec<double> v;
    DVec<uint8_t> f;
};

// Flagged sub-pattern of the candidate pattern with the candidate index of each entry.
struct Flagged {
    Pattern pat;
    std::vector<int64_t> cand;
};

// Symbolic two-stage projection  C = (Tt * A) * T  with the accumulation order of a
// column-by-column sparse product (see sym.hpp: product()).
struct ProjChain {
    Pattern C;                           // reduced x reduced, before pruning
    DVec<int64_t> p1, src1, p2, src2;
    DVec<double> coef1, coef2;
    int64_t n1 = 0, n2 = 0;
    DVec<double> I, Cv;                  // device values
    DVec<uint8_t> Cf;                    // |C| > tol
};

// A free-space matrix extracted from a projection: pattern + gather indices into C values.
struct FreeMat {
    Pattern pat;                         // n_free x n_free, after the reference's pruning
    DVec<int64_t> idx;                   // entry -> index in ProjChain::Cv
    DVec<double> v;                      // values (real-valued projections)
    // structural pattern: every entry the projection can produce (does not depend on the
    // values, so analyses built on it hold for every speed); pruned entries are exact zeros
    Pattern spat;
    DVec<int64_t> sidx;
    DVec<double> sv;
};

// Index maps of a union pattern onto its constituent matrices (entry index or -1).
struct UnionMaps {
    Pattern U;
    std::vector<DVec<int64_t>> maps;     // one per constituent
    DVec<int64_t> csr2csc;               // CSR position -> CSC entry
    DVec<int64_t> csr_rowptr;
    DVec<int32_t> csr_col;
    DVec<int64_t> lower2csc;             // lower-triangle entry (CSC order) -> CSC entry
    DVec<int32_t> low_row, low_col;      // (row, col) of every lower-triangle entry
    Pattern lower;
};

// Per-operator symbolic factorisation with device schedule.
struct OpSymbolic {
    Symbolic S;
    DevSymbolic D;
    bool valid = false;
};

struct Sector {
    int32_t nn = 0, ne = 0, ns = 0, axis = 2;
    double E = 0, nu = 0, rho = 0;
    std::vector<double> X;
    std::vector<int32_t> conn, left, right, hub;
    std::vector<std::pair<int32_t, int32_t>> pairs;
    // DOF classes
    std::vector<int32_t> interior_dofs, left_dofs, right_dofs, f2r, r2free, free_reduced_map;
    std::vector<uint8_t> is_right;
    int32_t n_reduced = 0, n_free = 0;
    // candidate pattern
    std::vector<int64_t> nadj_p;
    std::vector<int32_t> nadj_i;
    Pattern cand;
    int64_t npairs = 0;
    // device geometry + assembly maps
    DVec<double> dX;
    DVec<int32_t> dconn, pair_col, pair_pos, clist, nlist;
    DVec<int64_t> dnadj_p, cptr, dcand_p, nptr;
    DVec<int32_t> dcand_i;             // candidate-pattern row indices (uploaded for the modal masses)
    DVec<double> Kel, Mel, Fe;
    // transformation T(0) (complex with zero imaginary part) and its real filtered copy
    Pattern T0, T0t, Tr, Trt;
    std::vector<double> T0v, T0tv, Trv, Trtv;
};

}  // namespace tmg
