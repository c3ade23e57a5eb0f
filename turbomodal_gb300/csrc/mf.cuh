// Supernodal multifrontal LDL^H on the device, batched over problems that share one
// symbolic analysis (e.g. every complex harmonic at one speed).
//
// Storage per problem: L panels (m x w column-major per supernode, persistent) and a
// reusable workspace of update blocks ((m-w) x (m-w) per supernode, live from the start of
// the supernode's level until its parent's extend-add; offsets from a first-fit plan).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"
#include "sym.hpp"

namespace tmg {

constexpr int MF_NB = 32;      // pivot block width
constexpr int MF_TILE = 64;    // Schur-update tile
constexpr int MF_SB = 256;     // super-block: pivot blocks update inside it, one trailing update after it
constexpr int SV_RR = 64;      // rows per CTA of the forward rectangle products
constexpr int SV_CH = 2048;    // gathered solution entries staged per pass (backward rectangles)
constexpr int MF_TC_MIN_ROWS = 192;    // rows right of a super-block for the tensor-core trail update
constexpr int64_t MF_TC_GROUP_ROWS = 8192;   // staging rows per tc group (more only for one larger front)

// Width of the diagonal blocks that the triangular solves treat as dense units (the factor
// stores each block's explicit unit-lower inverse).
template <typename T>
constexpr int sv_nb() { return 64; }

// Per-supernode geometry shared by the kernels.
struct SnDev {
    const int32_t* first;      // ns+1
    const int64_t* row_ptr;    // ns+1 (front row lists; m = row_ptr[s+1]-row_ptr[s])
    const int32_t* rows;       // global factor rows of each front
    const int64_t* loff;       // ns+1 L panel offsets
    const int64_t* uoff;       // ns update-block offsets in the workspace
    const int32_t* child_ptr;
    const int32_t* child_list;
    const int64_t* rel_ptr;
    const int32_t* rel;
};

// Device copy of a Symbolic plus the launch schedules.
struct DevSymbolic {
    int32_t n = 0, ns = 0, max_front = 0;
    int64_t l_entries = 0;     // L storage per problem (sum m*w)
    int64_t u_entries = 0;     // update workspace per problem (first-fit peak)
    int64_t t_entries = 0;     // solve scratch per problem (sum m)
    int64_t l_stored = 0;      // entries of L actually read by a solve (lower trapezoids)
    int32_t *sn_first = nullptr, *sn_rows = nullptr, *rel = nullptr, *child_ptr = nullptr, *child_list = nullptr;
    int64_t *sn_row_ptr = nullptr, *loff = nullptr, *uoff = nullptr, *rel_ptr = nullptr;
    int32_t* perm = nullptr;
    int32_t* level_sn = nullptr;
    int32_t* items = nullptr;
    int32_t* sitems = nullptr;
    int64_t* dest = nullptr;   // scatter destination (L storage) of operator lower entries
    uint8_t* conj = nullptr;
    int64_t nlower = 0;
    double flops = 0.0;        // real flops of one complex factorisation (4 sum c_j^2)
    size_t bytes = 0;
    cudaStream_t alloc_stream = nullptr;   // stream the device arrays were allocated on
    ByteCount* cnt = nullptr;              // the owning context's byte count
    struct Step {
        int32_t level = 0, kb = 0;
        int64_t uzero_off = 0;                 // (s) items whose update blocks are zeroed
        int32_t uzero_cnt = 0;
        int64_t uzero_max = 0;
        std::vector<int64_t> ext_off;          // extend-add lists (parent, child), one per child rank
        std::vector<int32_t> ext_cnt, ext_max;
        int64_t diag_off = 0, panel_off = 0, upd_off = 0, trail_off = 0;
        int32_t diag_cnt = 0, panel_cnt = 0, upd_cnt = 0, trail_cnt = 0;
        // The trail items of fronts that qualify for the tensor-core update (at least
        // MF_TC_MIN_ROWS rows right of the super-block) come last: trail_simt of them belong to
        // the other fronts.  The complex FP32 factor runs those last items as tc groups instead.
        int32_t trail_simt = 0;
        struct TcGroup {
            int64_t stage_off = 0, upd_off = 0;   // items: (s, r0, dst) and (s, i0, j0, abase, bbase)
            int32_t stage_cnt = 0, upd_cnt = 0;
        };
        std::vector<TcGroup> tc;
    };
    std::vector<Step> steps;
    int64_t tc_rows = 0;       // staging rows (complex) per problem of the largest tc group
    int32_t tc_min_rows = MF_TC_MIN_ROWS;   // set before upload: tensor-core threshold of the plan
    using SolveLevel = tmg::SolveLevel;
    using SolvePlan = tmg::SolvePlan;
    SolvePlan plan64;          // the solve schedule for 64-wide diagonal blocks
    std::vector<int32_t> level_ptr;
    SnDev sn() const {
        return SnDev{sn_first, sn_row_ptr, sn_rows, loff, uoff, child_ptr, child_list, rel_ptr, rel};
    }
    void upload(const Symbolic& S, const std::vector<int64_t>& dest_h, const std::vector<uint8_t>& conj_h);
    void release();
    void swap(DevSymbolic& o) noexcept;   // exchanges every field (device arrays change owner)
    DevSymbolic() = default;
    DevSymbolic(const DevSymbolic&) = delete;
    DevSymbolic& operator=(const DevSymbolic&) = delete;
    ~DevSymbolic() { release(); }
};

// B problems sharing one DevSymbolic; per-problem arrays are strided.
template <typename T>
struct Batch {
    int B = 1;
    T* L = nullptr;            // B * lstride
    T* U = nullptr;            // B * ustride
    int64_t lstride = 0, ustride = 0;
};

// Scatter operator values (B x nlower, problem stride nlower) into zeroed L panels.
template <typename T>
void mf_scatter(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, const T* vals);

// Numeric factorisation; status[p] receives 1 + the first zero-pivot column of problem p.
// On return every diagonal block of width sv_nb<T>() of every panel holds, below its
// diagonal, the strict lower part of the block's unit-lower inverse (the diagonal keeps D),
// which is the form mf_solve reads.
// tensor_cores: the complex FP32 factor runs its large trailing updates on tcgen05 (mf_tc.cu);
// other types ignore it.
template <typename T>
void mf_factor(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, int* status, bool tensor_cores = true);

// x (B x n, factor numbering, factor precision) <- L^-H D^-1 L^-1 x ; tbuf: B x t_entries.
// skip (device, B flags, may be null): problems with a nonzero flag are left untouched.
template <typename T>
void mf_solve(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, T* x, T* tbuf, const int* skip = nullptr);

// Permutation with precision conversion between user vectors (problem stride ld) and the
// factor-numbering work vectors (problem stride n); optional per-problem diagonal scaling
// (problem stride n, original numbering).
template <typename T, typename U>
void mf_permute_in(cudaStream_t st, const DevSymbolic& S, int B, const U* b, int64_t ldb, T* x, const double* scale);
template <typename T, typename U>
void mf_permute_out(cudaStream_t st, const DevSymbolic& S, int B, const T* x, U* out, int64_t ldo, const double* scale);

// Count non-positive pivots of each problem into cnt[p].
template <typename T>
void mf_count_nonpos(cudaStream_t st, const DevSymbolic& S, const Batch<T>& bt, int* cnt);

}  // namespace tmg
