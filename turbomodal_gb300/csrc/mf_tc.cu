// Trailing Schur updates of the complex FP32 factorisation on the 5th-generation tensor cores.
//
// When a 256-column super-block of a front is factorised, the rest of the front is updated
//     C(i, j) -= sum_{l in super-block} L(i, l) d_l conj(L(j, l)),   i >= j >= kend,
// a complex product with K <= 256 (the reference's counterpart is the column-by-column
// update inside Eigen's SimplicialLDLT, src/hermitian_lanczos.cpp:12-56).  Here it runs as a
// real product of interleaved operands: complex row i of A = L(rows, SB) becomes real rows
// 2i (Re) and 2i+1 (Im), and likewise for B = L(rows, SB) diag(d), so
//     P = A_r B_r^T,  Re C(i, j) = P(2i, 2j) + P(2i+1, 2j+1),  Im C(i, j) = P(2i+1, 2j) - P(2i, 2j+1),
// four real multiply-adds per complex one, none wasted.  FP32 accuracy comes from a three-way
// BF16 split x = x1 + x2 + x3 (each x_k = bf16(x - x1 - ... - x_{k-1}); 3 x 8 significand bits
// hold the 24 of an FP32 value): A B^T ~ sum over the pieces of order below 2^-16,
//     A1 B1 + A1 B2 + A2 B1 + A1 B3 + A3 B1 + A2 B2,
// six kind::f16 products with exact BF16 x BF16 terms and FP32 accumulation.  The dropped terms
// are below 2^-23 of |A||B|, the rounding level of the FP32 SIMT update they replace.  The
// tensor core's accumulation rounds every partial sum, so the terms go to three TMEM
// accumulators summed in FP32 by the epilogue: the leading product A1 B1 of even and of odd
// 64-wide K chunks in two of them (each sees half the K steps), the five smaller products in
// the third (their rounding then scales with their own size, 2^-8 of the leading one).
//
// k_stage_tc writes, once per super-block and front, the rows [kend, m) of the six operand
// planes (A1, A2, A3, B1, B2, B3) K-major (256 BF16 per real row) into a staging tensor.
// k_update_tc computes one 64x64 complex tile (a 128x128 real accumulator in TMEM) per CTA:
// warp 0 issues TMA loads of 128 x 64-BF16 boxes (128-byte swizzle) into a 2-stage ring,
// warp 1 issues tcgen05.mma kind::f16 (BF16 in, FP32 accumulate; M = N = 128, K = 16; six per
// K step), and all four warps read the accumulator back with tcgen05.ld, combine the real parts
// into complex entries and subtract them from the front.  Every mbarrier wait is bounded
// (about one second of clock): on expiry the kernel records an error code, stops issuing,
// waits (again bounded) for what it issued, frees its TMEM and returns without writing.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstring>
#include <mutex>

#include "mf.cuh"
#include "mf_tc.cuh"

namespace tmg {

namespace {

constexpr int TC_STAGES = 2;
constexpr int TC_STAGE_ROWS = 16;                  // complex rows per staging item
constexpr int TC_PLANES = 6;                       // A1, A2, A3, B1, B2, B3
constexpr int TC_KS = 256;                         // BF16 per staged real row (one super-block)
constexpr int TC_BOX_K = 64;                       // BF16 per TMA box row (128 bytes)
constexpr int TC_ROWS = 128;                       // real rows per operand tile
constexpr int TC_TILE_BYTES = TC_ROWS * TC_BOX_K * 2;   // 16 KB
constexpr int TC_STAGE_BYTES = TC_PLANES * TC_TILE_BYTES;
constexpr int TC_SMEM = TC_STAGES * TC_STAGE_BYTES + 1024 /* alignment slack */ + 256 /* barriers */;
constexpr int TC_ACC_COLS = 128;                   // f32 columns of one 128x128 accumulator
constexpr int TC_TMEM_COLS = 512;                  // three accumulators (power of two)
constexpr long long TC_WAIT_CYCLES = 2000000000LL;      // ~1 s at 2 GHz

// instruction descriptor of tcgen05.mma kind::f16: D F32, A/B BF16, both K-major, M = 128, N = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                       // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;             // stride byte offset
    d |= (uint64_t)1 << 46;                       // descriptor version
    d |= (uint64_t)2 << 61;                       // 128-byte swizzle
    return d;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false when the phase did not complete within TC_WAIT_CYCLES
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > TC_WAIT_CYCLES) return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(TC_IDESC), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// three-way BF16 split: x = p[0] + p[1] + p[2] up to the last bits of an FP32 significand
__device__ __forceinline__ void split3(float x, __nv_bfloat16 (&p)[3]) {
    p[0] = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p[0]);
    p[1] = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(p[1]);
    p[2] = __float2bfloat16_rn(r2);
}

// ------------------------------------------------------------------------------------
// Staging.  Item (s, r0, dst0): complex rows r0 .. r0+15 of front s (rows >= m skipped) go to
// staging rows dst0 .. of every problem's block; columns l in [kl, kl + Kp) of the current
// super-block, zero beyond kend.  Plane q (0-2: the pieces of A = L, 3-5: those of
// B = L diag(d)) of problem p, real row t: staging row q * plane_rows + p * prob_rows + t,
// TC_KS BF16 each.
__global__ void __launch_bounds__(256) k_stage_tc(const int32_t* __restrict__ items, int kb, SnDev S,
                                                  const zf* __restrict__ L, int64_t lstride,
                                                  __nv_bfloat16* __restrict__ stg, int64_t prob_rows,
                                                  int64_t plane_rows) {
    __shared__ zf tile[256][TC_STAGE_ROWS + 1];   // [column l][row rr]
    __shared__ float dsh[256];
    const int64_t p = blockIdx.y;
    const int s = items[3 * blockIdx.x];
    const int64_t r0 = items[3 * blockIdx.x + 1];
    const int64_t dst0 = items[3 * blockIdx.x + 2];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const int kl = (kb * MF_NB / MF_SB) * MF_SB;
    const int kend = min((kb + 1) * MF_NB, w);
    const int K = kend - kl;
    const int Kp = (K + TC_BOX_K - 1) / TC_BOX_K * TC_BOX_K;
    const zf* Fs = L + p * lstride + S.loff[s];
    // 16 threads per column: two columns per warp and pass
    const int rr0 = threadIdx.x % TC_STAGE_ROWS, lc = threadIdx.x / TC_STAGE_ROWS;
    for (int l = lc; l < Kp; l += 256 / TC_STAGE_ROWS) {
        zf v{0.f, 0.f};
        if (l < K && r0 + rr0 < m) v = Fs[(int64_t)(kl + l) * m + r0 + rr0];
        tile[l][rr0] = v;
    }
    for (int l = threadIdx.x; l < Kp; l += 256) dsh[l] = l < K ? Fs[(int64_t)(kl + l) * m + kl + l].x : 0.f;
    __syncthreads();
    const int nrows = (int)min((int64_t)TC_STAGE_ROWS, m - r0);
    // 2 x 16 real rows x Kp columns per plane; consecutive threads write consecutive columns
    for (int q = threadIdx.x; q < 2 * TC_STAGE_ROWS * Kp; q += 256) {
        const int t = q / Kp, l = q % Kp;
        const int rr = t >> 1, c = t & 1;
        if (rr >= nrows) continue;
        const zf z = tile[l][rr];
        const float x = c ? z.y : z.x;
        __nv_bfloat16 a[3], b[3];
        split3(x, a);
        split3(dsh[l] * x, b);
        const int64_t row = p * prob_rows + 2 * (dst0 + rr) + c;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            stg[((int64_t)k * plane_rows + row) * TC_KS + l] = a[k];
            stg[((int64_t)(3 + k) * plane_rows + row) * TC_KS + l] = b[k];
        }
    }
}

// ------------------------------------------------------------------------------------
// One 64x64 complex tile per CTA.  Item (s, i0, j0, abase, bbase): tile rows i0.., columns
// j0.. of front s; abase / bbase: the staging rows (complex) of rows i0 and j0.
__global__ void __launch_bounds__(128, 1) k_update_tc(const int32_t* __restrict__ items, int kb, SnDev S,
                                                      zf* __restrict__ L, zf* __restrict__ U, int64_t lstride,
                                                      int64_t ustride, const __grid_constant__ CUtensorMap tmap,
                                                      int64_t prob_rows, int64_t plane_rows, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    // 1024-byte aligned ring (the 128-byte swizzle pattern repeats every 1024 bytes)
    const uint32_t raw = smem_u32(tc_smem_raw);
    const uint32_t ring = (raw + 1023u) & ~1023u;
    const uint32_t bars = ring + TC_STAGES * TC_STAGE_BYTES;   // full[3], empty[3], done
    unsigned char* bars_gen = tc_smem_raw + (bars - raw);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars_gen + 8 * (2 * TC_STAGES + 1));
    int* abort_flag = reinterpret_cast<int*>(bars_gen + 8 * (2 * TC_STAGES + 1) + 8);
    auto full = [&](int st) { return bars + 8u * st; };
    auto empty = [&](int st) { return bars + 8u * (TC_STAGES + st); };
    const uint32_t done = bars + 8u * (2 * TC_STAGES);

    const int64_t p = blockIdx.y;
    const int s = items[5 * blockIdx.x];
    const int64_t i0 = items[5 * blockIdx.x + 1], j0 = items[5 * blockIdx.x + 2];
    const int64_t abase = items[5 * blockIdx.x + 3], bbase = items[5 * blockIdx.x + 4];
    const int64_t m = S.row_ptr[s + 1] - S.row_ptr[s];
    const int w = S.first[s + 1] - S.first[s];
    const int kl = (kb * MF_NB / MF_SB) * MF_SB;
    const int kend = min((kb + 1) * MF_NB, w);
    const int nK = (kend - kl + TC_BOX_K - 1) / TC_BOX_K;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int st = 0; st < TC_STAGES; st++) { mbar_init(full(st), 1); mbar_init(empty(st), 1); }
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmap)) : "memory");
    }
    if (warp == 0) {   // TMEM accumulator: 128 lanes x 128 f32 columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const int ya = (int)(p * prob_rows + 2 * abase), yb = (int)(p * prob_rows + 2 * bbase);
    int issued = 0;   // TMA stages issued (producer thread)
    if (warp == 0 && lane == 0) {
        for (int kc = 0; kc < nK; kc++) {
            const int st = kc % TC_STAGES;
            if (kc >= TC_STAGES && !mbar_wait(empty(st), ((kc / TC_STAGES) - 1) & 1)) {
                atomicExch(err, 1);
                atomicExch(abort_flag, 1);
                break;
            }
            if (*(volatile int*)abort_flag) break;
            const uint32_t sb = ring + st * TC_STAGE_BYTES;
            mbar_expect_tx(full(st), TC_STAGE_BYTES);
            const int x = kc * TC_BOX_K;
#pragma unroll
            for (int q = 0; q < TC_PLANES; q++)
                tma_load_2d(sb + q * TC_TILE_BYTES, &tmap, x, (int)(q * plane_rows) + (q < 3 ? ya : yb), full(st));
            issued++;
        }
    } else if (warp == 1 && lane == 0) {
        bool ok = true;
        for (int kc = 0; kc < nK; kc++) {
            const int st = kc % TC_STAGES;
            if (!mbar_wait(full(st), (kc / TC_STAGES) & 1)) {
                atomicExch(err, 2);
                atomicExch(abort_flag, 1);
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sb = ring + st * TC_STAGE_BYTES;
#pragma unroll
            for (int ks = 0; ks < TC_BOX_K / 16; ks++) {
                const uint32_t off = ks * 32;   // 16 BF16 = 32 bytes along K inside the swizzled row
                const uint64_t a1 = smem_desc(sb + 0 * TC_TILE_BYTES + off);
                const uint64_t a2 = smem_desc(sb + 1 * TC_TILE_BYTES + off);
                const uint64_t a3 = smem_desc(sb + 2 * TC_TILE_BYTES + off);
                const uint64_t b1 = smem_desc(sb + 3 * TC_TILE_BYTES + off);
                const uint64_t b2 = smem_desc(sb + 4 * TC_TILE_BYTES + off);
                const uint64_t b3 = smem_desc(sb + 5 * TC_TILE_BYTES + off);
                const uint32_t big = tmem + (uint32_t)((kc & 1) * TC_ACC_COLS);   // A1 B1, by K chunk parity
                const uint32_t small = tmem + 2u * TC_ACC_COLS;                   // the five smaller terms
                mma_bf16(small, a2, b2, (kc > 0 || ks > 0) ? 1u : 0u);
                mma_bf16(small, a1, b3, 1u);
                mma_bf16(small, a3, b1, 1u);
                mma_bf16(small, a1, b2, 1u);
                mma_bf16(small, a2, b1, 1u);
                mma_bf16(big, a1, b1, (kc > 1 || ks > 0) ? 1u : 0u);
            }
            mma_commit(empty(st));   // this stage's smem may be refilled once these MMAs are done
        }
        (void)ok;             // on abort, completion of the MMAs already issued still signals done
        mma_commit(done);
    }
    // epilogue: every warp reads its 32 TMEM lanes (accumulator rows 32 warp .. +31)
    const bool got = mbar_wait(done, 0);
    if (!got) { atomicExch(err, 3); atomicExch(abort_flag, 1); }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncwarp();
    const bool write = got && nK > 0 && !*(volatile int*)abort_flag;
    zf* Lp = L + p * lstride;
    zf* Up = U + p * ustride;
    const int r = 32 * warp + lane;                 // accumulator row: complex row r / 2, part r % 2
    const int64_t i = i0 + (r >> 1);
    const bool odd = lane & 1;
#pragma unroll 1
    for (int c0 = 0; c0 < TC_ACC_COLS; c0 += 32) {
        float own[32], other[32];
#pragma unroll
        for (int q = 0; q < 32; q++) own[q] = 0.f;
        // accumulator 2 (smaller terms), then 0 and 1 (leading product; 1 only with a second K chunk)
        for (int a = 2; a >= 0; a--) {
            if (a == 1 && nK < 2) continue;
            uint32_t v[32];
            const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(a * TC_ACC_COLS + c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < 32; q++) own[q] += __uint_as_float(v[q]);
        }
#pragma unroll
        for (int q = 0; q < 32; q++) other[q] = __shfl_xor_sync(0xffffffffu, own[q], 1);
        if (!write) continue;
        // the even lane of a pair takes complex columns 0..7 of this chunk, the odd lane 8..15
#pragma unroll
        for (int h = 0; h < 8; h++) {
            const int jj = odd ? 8 + h : h;
            const float pe0 = odd ? other[2 * jj] : own[2 * jj];          // P(2i,   2j)
            const float pe1 = odd ? other[2 * jj + 1] : own[2 * jj + 1];  // P(2i,   2j+1)
            const float po0 = odd ? own[2 * jj] : other[2 * jj];          // P(2i+1, 2j)
            const float po1 = odd ? own[2 * jj + 1] : other[2 * jj + 1];  // P(2i+1, 2j+1)
            const int64_t j = j0 + (c0 >> 1) + jj;
            if (i < m && j < m && i >= j) {
                zf* dst = j < w ? Lp + S.loff[s] + j * m + i : Up + S.uoff[s] + (j - w) * (m - w) + (i - w);
                zf cur = *dst;
                cur.x -= pe0 + po1;
                cur.y -= po0 - pe1;
                *dst = cur;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0 && lane == 0 && *(volatile int*)abort_flag) {
        // an aborted CTA still waits (bounded) for the TMA loads it issued before its shared
        // memory goes away: the last load of each ring stage completes that stage's phase
        for (int kc = max(0, issued - TC_STAGES); kc < issued; kc++)
            if (!mbar_wait(full(kc % TC_STAGES), (kc / TC_STAGES) & 1)) break;
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) throw cuda_error("cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

}  // namespace

void mf_trail_tc(cudaStream_t st, const DevSymbolic& S, const Batch<zf>& bt, const DevSymbolic::Step& stp,
                 TcWork& wk) {
    if (stp.tc.empty()) return;
    const int64_t prob_rows = 2 * S.tc_rows;               // real staging rows per problem
    const int64_t plane_rows = prob_rows * bt.B;
    if (!wk.stg || wk.rows < TC_PLANES * plane_rows) {
        wk.release();
        const size_t bytes = (size_t)TC_PLANES * plane_rows * TC_KS * sizeof(__nv_bfloat16);
        TMG_CUDA(pool_malloc((void**)&wk.stg, bytes, st));
        wk.bytes = (int64_t)bytes;
        wk.cnt = g_bytes;
        if (wk.cnt) wk.cnt->add(wk.bytes);
        TMG_CUDA(cudaMemsetAsync(wk.stg, 0, bytes, st));
        TMG_CUDA(pool_malloc((void**)&wk.err, sizeof(int), st));
        TMG_CUDA(cudaMemsetAsync(wk.err, 0, sizeof(int), st));
        wk.rows = TC_PLANES * plane_rows;
        wk.stream = st;
        CUtensorMap map;
        const cuuint64_t dims[2] = {TC_KS, (cuuint64_t)wk.rows};
        const cuuint64_t strides[1] = {TC_KS * sizeof(__nv_bfloat16)};
        const cuuint32_t box[2] = {TC_BOX_K, TC_ROWS};
        const cuuint32_t estr[2] = {1, 1};
        const CUresult r = encode_fn()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, wk.stg, dims, strides, box, estr,
                                       CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) throw cuda_error("cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
        static_assert(sizeof(map) == sizeof(wk.map), "tensor map size");
        std::memcpy(wk.map, &map, sizeof(map));
        static std::once_flag attr_once;
        std::call_once(attr_once, []() {
            TMG_CUDA(cudaFuncSetAttribute(k_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
        });
    }
    CUtensorMap map;
    std::memcpy(&map, wk.map, sizeof(map));
    const SnDev sn = S.sn();
    const unsigned B = bt.B;
    for (const auto& g : stp.tc) {
        TMG_LAUNCH(k_stage_tc, dim3(g.stage_cnt, B), 256, 0, st, S.items + g.stage_off, stp.kb, sn, bt.L, bt.lstride,
                   static_cast<__nv_bfloat16*>(wk.stg), prob_rows, plane_rows);
        TMG_LAUNCH(k_update_tc, dim3(g.upd_cnt, B), 128, TC_SMEM, st, S.items + g.upd_off, stp.kb, sn, bt.L, bt.U,
                   bt.lstride, bt.ustride, map, prob_rows, plane_rows, wk.err);
    }
    TMG_CHECK_LAUNCH();
}

void TcWork::release() {
    if (stg) cudaFreeAsync(stg, stream);
    if (stg && cnt) cnt->cur -= bytes;
    cnt = nullptr;
    bytes = 0;
    if (err) cudaFreeAsync(err, stream);
    stg = nullptr;
    err = nullptr;
    rows = 0;
}

int TcWork::read_error(cudaStream_t st) {
    if (!err) return 0;
    int h = 0;
    TMG_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    TMG_CUDA(cudaStreamSynchronize(st));
    return h;
}

}  // namespace tmg
