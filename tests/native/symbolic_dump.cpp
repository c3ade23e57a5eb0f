// Host check of the symbolic analysis (tests/test_symbolic_host.py): reads a lower-triangle CSC
// pattern (int64 n, int64 nnz, int64 colptr[n + 1], int32 rows[nnz]), runs the library's
// analyze() (sym.cpp) and writes its reference-equivalent outputs, each int32[n]: the AMD order
// (pivot k -> original index), the elimination tree (parent, -1 = root) and the L column counts.
#include <cstdio>
#include <vector>

#include "sym.hpp"

using namespace tmg;

int main(int argc, char** argv) {
    if (argc < 3) return 2;
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
    const Symbolic S = analyze(P, 0.0, 0);
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(S.amd.data(), 4, S.amd.size(), o);
    std::fwrite(S.etree.data(), 4, S.etree.size(), o);
    std::fwrite(S.colcount.data(), 4, S.colcount.size(), o);
    std::fclose(o);
    return 0;
}
