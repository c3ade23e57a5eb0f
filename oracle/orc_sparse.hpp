// Oracle (test infrastructure only): compressed-sparse-column matrices with the
// semantics the reference gets from Eigen 3.4.0's SparseMatrix (Eigen is a third-party
// dependency not present in the reference tree; its behaviour at the reference's call
// sites is restated here):
//   * setFromTriplets: duplicates summed in triplet order, rows sorted in each column;
//   * sparse + sparse: union pattern, structural entries kept even when values cancel;
//   * sparse * sparse: symbolic union of products, accumulated column by column in the
//     order (rhs entry, lhs entry);
//   * (A*B).pruned(ref): same product, entries with |v| <= |ref| * 1e-12 dropped.
#pragma once
#include <algorithm>
#include <complex>
#include <cstdint>
#include <vector>

namespace orc {

using cd = std::complex<double>;

template <typename T>
struct Csc {
    int rows = 0, cols = 0;
    std::vector<int> p{0}, i;
    std::vector<T> x;
    int64_t nnz() const { return (int64_t)i.size(); }
};
using CscD = Csc<double>;
using CscZ = Csc<cd>;

template <typename T>
struct Trip { int r, c; T v; };

inline double absval(double v) { return std::fabs(v); }
inline double absval(const cd& v) { return std::abs(v); }
inline double conjv(double v) { return v; }
inline cd conjv(const cd& v) { return std::conj(v); }

// Eigen SparseMatrix::setFromTriplets: stable bucket by column, then by row within column;
// values of equal (row, col) are summed in triplet order: ((v1 + v2) + v3) ...
template <typename T>
Csc<T> from_triplets(int rows, int cols, const std::vector<Trip<T>>& t) {
    Csc<T> A;
    A.rows = rows; A.cols = cols;
    std::vector<int64_t> rcount(rows + 1, 0);
    for (auto& e : t) rcount[e.r + 1]++;
    for (int r = 0; r < rows; r++) rcount[r + 1] += rcount[r];
    std::vector<int64_t> byrow(t.size());
    {
        std::vector<int64_t> pos(rcount.begin(), rcount.end() - 1);
        for (int64_t k = 0; k < (int64_t)t.size(); k++) byrow[pos[t[k].r]++] = k;
    }
    // collapse duplicates within each row (first occurrence keeps the slot)
    std::vector<int> colmark(cols, -1);
    std::vector<int64_t> slot_of_col(cols, -1);
    std::vector<int> ur, uc;
    std::vector<T> uv;
    ur.reserve(t.size()); uc.reserve(t.size()); uv.reserve(t.size());
    for (int r = 0; r < rows; r++) {
        for (int64_t q = rcount[r]; q < rcount[r + 1]; q++) {
            const auto& e = t[byrow[q]];
            if (colmark[e.c] == r) {
                uv[slot_of_col[e.c]] = uv[slot_of_col[e.c]] + e.v;
            } else {
                colmark[e.c] = r;
                slot_of_col[e.c] = (int64_t)uv.size();
                ur.push_back(r); uc.push_back(e.c); uv.push_back(e.v);
            }
        }
    }
    // transpose copy: columns, rows ascending (row-major scan order)
    A.p.assign(cols + 1, 0);
    for (int c : uc) A.p[c + 1]++;
    for (int c = 0; c < cols; c++) A.p[c + 1] += A.p[c];
    A.i.resize(uc.size());
    A.x.resize(uc.size());
    std::vector<int> pos(A.p.begin(), A.p.end() - 1);
    for (size_t k = 0; k < uc.size(); k++) {
        const int d = pos[uc[k]]++;
        A.i[d] = ur[k];
        A.x[d] = uv[k];
    }
    return A;
}

template <typename T>
Csc<T> transpose(const Csc<T>& A, bool conjugate) {
    Csc<T> B;
    B.rows = A.cols; B.cols = A.rows;
    B.p.assign(B.cols + 1, 0);
    for (int r : A.i) B.p[r + 1]++;
    for (int c = 0; c < B.cols; c++) B.p[c + 1] += B.p[c];
    B.i.resize(A.i.size());
    B.x.resize(A.x.size());
    std::vector<int> pos(B.p.begin(), B.p.end() - 1);
    for (int j = 0; j < A.cols; j++)
        for (int q = A.p[j]; q < A.p[j + 1]; q++) {
            const int d = pos[A.i[q]]++;
            B.i[d] = j;
            B.x[d] = conjugate ? conjv(A.x[q]) : A.x[q];
        }
    return B;
}

// alpha*A + beta*B with the union pattern; missing operands contribute an exact zero:
// both -> (alpha*a) + (beta*b); A only -> (alpha*a) + 0; B only -> 0 + (beta*b).
template <typename T>
Csc<T> add(const Csc<T>& A, T alpha, const Csc<T>& B, T beta) {
    Csc<T> C;
    C.rows = A.rows; C.cols = A.cols;
    C.p.assign(A.cols + 1, 0);
    C.i.reserve(A.i.size() + B.i.size());
    C.x.reserve(A.i.size() + B.i.size());
    for (int j = 0; j < A.cols; j++) {
        int qa = A.p[j], qb = B.p[j];
        const int ea = A.p[j + 1], eb = B.p[j + 1];
        while (qa < ea || qb < eb) {
            const int ra = qa < ea ? A.i[qa] : INT32_MAX;
            const int rb = qb < eb ? B.i[qb] : INT32_MAX;
            if (ra == rb) { C.i.push_back(ra); C.x.push_back(alpha * A.x[qa] + beta * B.x[qb]); qa++; qb++; }
            else if (ra < rb) { C.i.push_back(ra); C.x.push_back(alpha * A.x[qa] + T(0)); qa++; }
            else { C.i.push_back(rb); C.x.push_back(T(0) + beta * B.x[qb]); qb++; }
        }
        C.p[j + 1] = (int)C.i.size();
    }
    return C;
}

// C = A*B.  For each column j of B, for each B(k,j) in row order, for each A(i,k) in row
// order: c_i = first ? a*b : c_i + a*b.  Entries with |c| <= tol are dropped when prune.
template <typename T>
Csc<T> multiply(const Csc<T>& A, const Csc<T>& B, bool prune, double tol) {
    Csc<T> C;
    C.rows = A.rows; C.cols = B.cols;
    C.p.assign(B.cols + 1, 0);
    std::vector<char> mark(A.rows, 0);
    std::vector<T> acc(A.rows, T(0));
    std::vector<int> idx;
    for (int j = 0; j < B.cols; j++) {
        idx.clear();
        for (int q = B.p[j]; q < B.p[j + 1]; q++) {
            const int k = B.i[q];
            const T bv = B.x[q];
            for (int r = A.p[k]; r < A.p[k + 1]; r++) {
                const int i = A.i[r];
                if (!mark[i]) { mark[i] = 1; acc[i] = A.x[r] * bv; idx.push_back(i); }
                else acc[i] += A.x[r] * bv;
            }
        }
        std::sort(idx.begin(), idx.end());
        for (int i : idx) {
            if (!prune || absval(acc[i]) > tol) { C.i.push_back(i); C.x.push_back(acc[i]); }
            mark[i] = 0;
        }
        C.p[j + 1] = (int)C.i.size();
    }
    return C;
}

template <typename T>
Csc<T> scale(const Csc<T>& A, T s) {
    Csc<T> B = A;
    for (auto& v : B.x) v = s * v;
    return B;
}

// Frobenius norm (Eigen SparseMatrix::norm)
template <typename T>
double fro(const Csc<T>& A) {
    double s = 0.0;
    for (auto& v : A.x) s += std::norm(cd(v));
    return std::sqrt(s);
}

template <typename T>
void spmv(const Csc<T>& A, const T* x, T* y) {  // y = A x
    for (int r = 0; r < A.rows; r++) y[r] = T(0);
    for (int j = 0; j < A.cols; j++) {
        const T xj = x[j];
        for (int q = A.p[j]; q < A.p[j + 1]; q++) y[A.i[q]] += A.x[q] * xj;
    }
}

inline CscZ to_complex(const CscD& A) {
    CscZ B;
    B.rows = A.rows; B.cols = A.cols; B.p = A.p; B.i = A.i;
    B.x.resize(A.x.size());
    for (size_t k = 0; k < A.x.size(); k++) B.x[k] = cd(A.x[k], 0.0);
    return B;
}

}  // namespace orc
