// Host-side symbolic analysis for the GB300 supernodal LDL^H: fill-reducing order,
// elimination tree, supernode partition, frontal structure and level schedule.
// Pattern-only work runs once per sparsity pattern on the host; all arithmetic on
// matrix values runs on the device.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace tmg {

// Compressed sparse column pattern (rows sorted inside each column).
struct Pattern {
    int32_t nrows = 0, ncols = 0;
    std::vector<int64_t> p{0};
    std::vector<int32_t> i;
    int64_t nnz() const { return (int64_t)i.size(); }
};

// Approximate minimum degree order of a symmetric pattern given with both triangles
// and its diagonal.  Returns order[k] = index of the k-th pivot.  The algorithm is the
// published AMD of Amestoy, Davis & Duff in the cs_amd formulation (T. A. Davis, Direct
// Methods for Sparse Linear Systems, SIAM 2006), in the variant that keeps the diagonal
// in the quotient graph (a node whose only entry is its diagonal is eliminated at once,
// a node without a diagonal entry is ordered last) — the ordering Eigen 3.4.0's
// AMDOrdering computes for the reference's SimplicialLDLT.
std::vector<int32_t> amd_order(int32_t n, const std::vector<int64_t>& colptr, const std::vector<int32_t>& rowind);

// Supernodal symbolic factorisation of a Hermitian matrix given by its lower triangle.
struct Symbolic {
    int32_t n = 0;
    // Reference-equivalent analysis (bit-exact targets): AMD order, etree, column counts
    // in AMD numbering, as SimplicialLDLT::analyzePattern computes them.
    std::vector<int32_t> amd;           // amd[k] = original index of pivot k
    std::vector<int32_t> etree;         // parent in AMD numbering (-1 = root)
    std::vector<int32_t> colcount;      // off-diagonal nonzeros of L per column (AMD numbering)
    int64_t nnz_l = 0;                  // sum of colcount
    // Factorisation numbering: the etree postorder of the AMD order (same fill, same tree).
    std::vector<int32_t> perm;          // perm[j] = original index of factor column j
    std::vector<int32_t> iperm;         // iperm[orig] = factor column
    // Supernodes (contiguous factor columns with nested structure)
    int32_t ns = 0;
    std::vector<int32_t> sn_first;      // ns + 1
    std::vector<int32_t> sn_parent;     // supernodal tree, -1 = root
    std::vector<int64_t> sn_row_ptr;    // ns + 1, into sn_rows
    std::vector<int32_t> sn_rows;       // sorted global factor rows of each front
    std::vector<int64_t> front_off;     // ns + 1, front storage offsets (m*m entries each)
    std::vector<int64_t> rel_ptr;       // ns + 1, into rel (update rows of s -> parent local)
    std::vector<int32_t> rel;
    std::vector<int32_t> child_ptr, child_list;   // children of each supernode (ascending)
    std::vector<int32_t> level_ptr, level_sn;     // supernodes grouped by tree height
    int32_t max_front = 0;
    double flops_real = 0.0;            // sum_j c_j^2 (multiply-adds of the factorisation)
    int64_t front_entries() const { return front_off.empty() ? 0 : front_off.back(); }
};

// lower: lower-triangle pattern (orig numbering) of the operator.  relax: merge a child
// supernode into its parent when the combined front adds at most this fraction of
// explicit zeros (0 = fundamental supernodes only).
Symbolic analyze(const Pattern& lower, double relax = 0.0, int32_t relax_max_width = 0,
                 const std::vector<int32_t>* amd = nullptr);

// Triangular-solve schedule for diagonal blocks of width nb (host side; the device kernels
// read the item lists).
//
// Subtrees: the largest subtrees whose fronts are all at most nb columns wide and that hold
// at most `subtree_entries` panel entries in all are solved whole, one warp per subtree (in
// postorder forward, in reverse postorder backward), in one launch per direction.  Supernodes
// are numbered in postorder, so a subtree is the contiguous range (first, root); the tasks
// are listed heaviest first.
//
// The other ("upper") fronts go level by level.  Forward: gather (the level's upper fronts;
// it also solves each front's first diagonal block), triangle launches b = 0.. (items
// (s, r0): rows [r0, r0 + nb) of the triangle below block b), one rectangle launch (items
// (s, r0): rows [r0, r0 + rows_per_rect) below the triangle).  Backward: one rectangle launch
// (items (s, c0): columns [c0, c0 + nb); it also solves each front's last diagonal block),
// triangle launches b = last .. 1 (items (s, c0): columns [c0, c0 + nb) left of block b).
// The forward subtree launch runs before the levels and the backward one after them.  Inverse
// lists: items (s, b) of the diagonal blocks to invert after a factorisation (small: width
// <= 32).
struct SolveLevel {
    std::vector<int64_t> ftri_off, btri_off;   // index b
    std::vector<int32_t> ftri_cnt, btri_cnt;
    int64_t gath_off = 0, frect_off = 0, brect_off = 0;
    int32_t gath_cnt = 0, frect_cnt = 0, brect_cnt = 0;
    int32_t maxw = 0;                          // widest upper front of the level
    int64_t maxu = 0;                          // most rows below a triangle (m - w)
};
struct SolvePlan {
    int nb = 0;
    int64_t sub_off = 0;                       // subtree tasks (first, root), heaviest first
    int32_t sub_cnt = 0;
    int32_t sub_fronts = 0;                    // fronts inside the subtrees
    std::vector<SolveLevel> levels;
    int64_t inv_small_off = 0, inv_large_off = 0;
    int32_t inv_small_cnt = 0, inv_large_cnt = 0;
};
// Builds the schedule of S; its items are appended to `items` (offsets index that array).
SolvePlan build_solve_plan(const Symbolic& S, int nb, int rows_per_rect, std::vector<int32_t>& items,
                           int64_t subtree_entries = 65536);

// Destination of every lower-triangle entry of `lower` (in its CSC order) inside the
// front storage of `S`; conj flag set when the entry lands transposed.
void scatter_map(const Symbolic& S, const Pattern& lower, std::vector<int64_t>& dest, std::vector<uint8_t>& conj);

// Symbolic sparse product C = A*B recording, for every C entry, its contributions in the
// accumulation order (for each B(k,j) in row order, each A(i,k) in row order).
struct Product {
    Pattern C;
    std::vector<int64_t> cptr;          // C.nnz()+1
    std::vector<int64_t> a_slot, b_slot;
};
Product product(const Pattern& A, const Pattern& B);

// Block layout of the Lancaster linearisation of the Coriolis QEP (src/modal_solver.cpp:151-198):
// L1 = [[D, K], [K, 0]], L2 = [[M, 0], [0, K]] with D = i 2 omega G.  `which` = 0 gives the
// pattern of the shifted operator L1 - sigma L2 = [[D - sigma M, K], [K, -sigma K]] (also the
// union of L1 and L2); `which` = 1 the pattern of L2 alone.  K, M, G are the n x n patterns
// of the harmonic's stiffness, mass and gyroscopic matrices; every 2n x 2n entry records its
// source entry in each of them (-1 when absent) and its block (0: top-left, 1: top-right,
// 2: bottom-left, 3: bottom-right).
struct LancasterBlocks {
    Pattern P;
    std::vector<int64_t> srcK, srcM, srcG;
    std::vector<int8_t> blk;
};
LancasterBlocks lancaster_blocks(const Pattern& K, const Pattern& M, const Pattern& G, int which);

Pattern transpose(const Pattern& A);
// Union of patterns (same shape).
Pattern pattern_union(const std::vector<const Pattern*>& parts);
// Position of every entry of `sub` inside `sup` (-1 when absent).
std::vector<int64_t> locate(const Pattern& sup, const Pattern& sub);
Pattern lower_triangle(const Pattern& A);

}  // namespace tmg
