// Launch wrappers of the element and sector-assembly kernels (fe.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace tmg {
void launch_elem_KM(cudaStream_t st, int ne, const double* X, const int32_t* conn, double E, double nu,
                    double rho, double* Ke, double* Me, int* neg_jac);
void launch_elem_rot(cudaStream_t st, int ne, const double* X, const int32_t* conn, double rho, double omega,
                     int axis, double* Kw, double* Ge);
void launch_elem_ksig(cudaStream_t st, int ne, const double* X, const int32_t* conn, double E, double nu,
                      const double* u, double* Ks, int* bad);
void launch_elem_fc(cudaStream_t st, int ne, const double* X, const int32_t* conn, double rho, double omega,
                    int axis, double* Fe);
void launch_gather_blocks(cudaStream_t st, int64_t npairs, const int32_t* pair_col, const int32_t* pair_pos,
                          const int64_t* nadj_p, const int64_t* cptr, const int32_t* clist, const int64_t* cand_p,
                          const double* Kel, double* vals, uint8_t* flags);
void launch_gather_load(cudaStream_t st, int nn, const int64_t* nptr, const int32_t* nlist, const double* Fe,
                        double* F);
void launch_cand_axpy3(cudaStream_t st, int64_t n, double a, const double* A, const uint8_t* fa, double b,
                       const double* B, const uint8_t* fb, double c, const double* C, const uint8_t* fc,
                       double* out, uint8_t* fout);
}  // namespace tmg
