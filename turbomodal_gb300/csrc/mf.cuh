// Supernodal multifrontal LDL^H on the device: factorisation and triangular solves.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "common.cuh"
#include "sym.hpp"

namespace tmg {

constexpr int MF_NB = 32;      // pivot block width
constexpr int MF_TILE = 64;    // Schur-update tile
constexpr int SV_B = 64;       // triangular-solve column block
constexpr int SV_RC = 256;     // rows per CTA in the forward sweep
constexpr int SV_CC = 32;      // columns per CTA (four per warp) in the backward sweeps

// Device copy of a Symbolic plus the host-side launch schedule.
struct DevSymbolic {
    int32_t n = 0, ns = 0, max_front = 0;
    int64_t front_entries = 0;
    int32_t *sn_first = nullptr, *sn_rows = nullptr, *rel = nullptr, *child_ptr = nullptr, *child_list = nullptr;
    int64_t *sn_row_ptr = nullptr, *front_off = nullptr, *rel_ptr = nullptr;
    int32_t *perm = nullptr;
    int32_t *level_sn = nullptr;               // supernodes grouped by level (device copy)
    // factorisation work lists (device), with host offsets per (level, kb)
    int32_t* items = nullptr;                  // packed int32 work items
    struct Step {
        std::vector<int64_t> ext_off;          // extend-add lists, one per child rank
        std::vector<int32_t> ext_cnt, ext_max; // items and largest update size per list
        int64_t diag_off = 0, panel_off = 0, upd_off = 0;
        int32_t diag_cnt = 0, panel_cnt = 0, upd_cnt = 0, kb = 0;
    };
    std::vector<Step> steps;                   // in execution order
    // triangular-solve schedule: per level, forward block sweeps (s, row0) and backward
    // sweeps (s, col0), one list per column block
    struct SolveLevel {
        int64_t off_items = 0;                 // backward off-diagonal items (s, col0)
        int32_t off_cnt = 0;
        std::vector<int64_t> fwd_off, bwd_off;
        std::vector<int32_t> fwd_cnt, bwd_cnt;
    };
    std::vector<SolveLevel> solve_levels;
    int32_t* sitems = nullptr;
    std::vector<int32_t> level_ptr;            // host copy
    std::vector<int32_t> level_max_m;          // max front size per level
    int64_t* dest = nullptr;                   // scatter destination of operator lower entries
    uint8_t* conj = nullptr;
    int64_t nlower = 0;
    double flops = 0.0;                        // real flops of one complex factorisation
    int64_t l_entries = 0;                     // stored L entries (panels)
    size_t bytes = 0;
    void upload(const Symbolic& S, const std::vector<int64_t>& dest_h, const std::vector<uint8_t>& conj_h);
    void release();
};

// Numeric factorisation of the fronts in F (already holding the scattered operator).
// status[0] receives 1 + the first zero-pivot column, or stays 0.
template <typename T>
void mf_factor(cudaStream_t st, const DevSymbolic& S, T* F, int* status);

template <typename T>
void mf_scatter(cudaStream_t st, const DevSymbolic& S, const T* vals, T* F);

// x_work (factor precision, factor numbering) <- L^-H D^-1 L^-1 x_work
template <typename T>
void mf_solve(cudaStream_t st, const DevSymbolic& S, const T* F, T* x, T* tbuf);

// Permutation with precision conversion between the user vector (FP64) and the factor
// numbering work vector.
// scale (nullable, original numbering): x[j] = b[perm[j]] * scale[perm[j]] on the way in,
// out[perm[j]] = x[j] * scale[perm[j]] on the way out.
template <typename T, typename U>
void mf_permute_in(cudaStream_t st, const DevSymbolic& S, const U* b, T* x, int nvec, int64_t ldb,
                   const double* scale = nullptr);
template <typename T, typename U>
void mf_permute_out(cudaStream_t st, const DevSymbolic& S, const T* x, U* out, int nvec, int64_t ldo,
                    const double* scale = nullptr);

}  // namespace tmg
