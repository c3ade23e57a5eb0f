// Host check of the Lancaster block layout (tests/test_qep.py): reads the n x n CSC patterns of
// K, M and G, runs the library's lancaster_blocks (sym.cpp) for the shifted operator (which = 0)
// and for L2 (which = 1), and writes each result as
//   int64 nnz, int64 colptr[2n + 1], int32 rows[nnz], int64 srcK[nnz], srcM[nnz], srcG[nnz], int8 blk[nnz]
// Input file: int64 n, then for K, M, G in turn: int64 nnz, int64 colptr[n + 1], int32 rows[nnz].
#include <cstdio>
#include <vector>

#include "sym.hpp"

using namespace tmg;

static bool read_pattern(FILE* f, int64_t n, Pattern& P) {
    int64_t nnz = 0;
    if (std::fread(&nnz, 8, 1, f) != 1) return false;
    P.nrows = P.ncols = (int32_t)n;
    P.p.resize(n + 1);
    P.i.resize(nnz);
    if (std::fread(P.p.data(), 8, n + 1, f) != (size_t)n + 1) return false;
    return std::fread(P.i.data(), 4, nnz, f) == (size_t)nnz;
}

static void write_blocks(FILE* f, const LancasterBlocks& L) {
    const int64_t nnz = L.P.nnz();
    std::fwrite(&nnz, 8, 1, f);
    std::fwrite(L.P.p.data(), 8, L.P.p.size(), f);
    std::fwrite(L.P.i.data(), 4, L.P.i.size(), f);
    std::fwrite(L.srcK.data(), 8, L.srcK.size(), f);
    std::fwrite(L.srcM.data(), 8, L.srcM.size(), f);
    std::fwrite(L.srcG.data(), 8, L.srcG.size(), f);
    std::fwrite(L.blk.data(), 1, L.blk.size(), f);
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t n = 0;
    if (std::fread(&n, 8, 1, f) != 1) return 2;
    Pattern K, M, G;
    if (!read_pattern(f, n, K) || !read_pattern(f, n, M) || !read_pattern(f, n, G)) return 2;
    std::fclose(f);
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    write_blocks(o, lancaster_blocks(K, M, G, 0));
    write_blocks(o, lancaster_blocks(K, M, G, 1));
    std::fclose(o);
    return 0;
}
