// Tensor-core (tcgen05) trailing Schur updates of the complex FP32 factorisation.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "mf.cuh"

namespace tmg {

// Staging buffer and tensor map of the tensor-core updates of one factorisation (allocated on
// first use, in the stream's order).
struct TcWork {
    void* stg = nullptr;         // 6 BF16 planes x B problems x 2 tc_rows real rows x 256 entries
    int* err = nullptr;          // nonzero: a bounded wait of k_update_tc expired
    int64_t rows = 0, bytes = 0;
    ByteCount* cnt = nullptr;
    cudaStream_t stream = nullptr;
    alignas(64) unsigned char map[128];
    void release();
    int read_error(cudaStream_t st);
    ~TcWork() { release(); }
};

// The tensor-core trailing updates of one schedule step (the step's tc groups).
void mf_trail_tc(cudaStream_t st, const DevSymbolic& S, const Batch<zf>& bt, const DevSymbolic::Step& stp,
                 TcWork& wk);

}  // namespace tmg
