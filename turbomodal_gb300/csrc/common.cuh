// Shared device/host helpers: complex types, error handling, launch accounting.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <stdexcept>
#include <string>

namespace tmg {

struct cuda_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct numeric_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

#define TMG_CUDA(call)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            throw ::tmg::cuda_error(std::string(#call) + ": " + cudaGetErrorString(e_) +      \
                                    " (" __FILE__ ":" + std::to_string(__LINE__) + ")");      \
    } while (0)

// Every kernel launch of this library goes through TMG_LAUNCH so the host can report
// how many of its kernels ran in a timed region (counted per host thread: a context is
// driven by one thread at a time).
extern thread_local int64_t g_kernel_launches;
// Stream of the context the calling thread is working for (set on entry to every C-ABI call
// that touches the device); device buffers are allocated, copied and freed in its order.
extern thread_local cudaStream_t g_stream;
// Device bytes held by the context the calling thread is working for (its stream-ordered
// buffers; null outside a C-ABI call).
struct ByteCount {
    std::atomic<int64_t> cur{0}, peak{0};
    void add(int64_t b) {
        const int64_t v = cur.fetch_add(b) + b;
        int64_t pk = peak.load();
        while (v > pk && !peak.compare_exchange_weak(pk, v)) {}
    }
};
extern thread_local ByteCount* g_bytes;
#define TMG_LAUNCH(kernel, grid, block, smem, stream, ...)                                    \
    do {                                                                                      \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);                            \
        ::tmg::g_kernel_launches++;                                                           \
    } while (0)
#define TMG_CHECK_LAUNCH() TMG_CUDA(cudaGetLastError())

// Programmatic dependent launch: the kernel may start while its predecessor in the stream is
// still running.  Such kernels call pdl_trigger() on entry (letting their own successor
// launch early), load only data no earlier kernel of the sequence writes, then call
// pdl_wait(), which returns once the predecessor has completed and its writes are visible.
// Every CTA of such a kernel executes pdl_wait(), so completion is transitive along the chain.
#define TMG_LAUNCH_PDL(kern_, grid_, block_, smem_, strm_, ...)                              \
    do {                                                                                      \
        cudaLaunchConfig_t cfg_{};                                                            \
        cfg_.gridDim = (grid_);                                                               \
        cfg_.blockDim = (block_);                                                             \
        cfg_.dynamicSmemBytes = (smem_);                                                      \
        cfg_.stream = (strm_);                                                                \
        cudaLaunchAttribute at_[1];                                                           \
        at_[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;                      \
        at_[0].val.programmaticStreamSerializationAllowed = 1;                               \
        cfg_.attrs = at_;                                                                     \
        cfg_.numAttrs = 1;                                                                    \
        TMG_CUDA(cudaLaunchKernelEx(&cfg_, kern_, __VA_ARGS__));                              \
        ::tmg::g_kernel_launches++;                                                           \
    } while (0)

#ifdef __CUDACC__
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#endif

// Minimal complex types (interleaved re/im), usable on host and device.
template <typename R>
struct cpx {
    R x, y;
};
using zd = cpx<double>;
using zf = cpx<float>;

template <typename T> struct real_of { using type = T; };
template <typename R> struct real_of<cpx<R>> { using type = R; };

#define HD __host__ __device__ __forceinline__
template <typename R> HD cpx<R> mk(R a, R b) { return cpx<R>{a, b}; }
template <typename R> HD cpx<R> operator+(cpx<R> a, cpx<R> b) { return {a.x + b.x, a.y + b.y}; }
template <typename R> HD cpx<R> operator-(cpx<R> a, cpx<R> b) { return {a.x - b.x, a.y - b.y}; }
template <typename R> HD cpx<R> operator*(cpx<R> a, cpx<R> b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
template <typename R> HD cpx<R> operator*(R s, cpx<R> a) { return {s * a.x, s * a.y}; }
template <typename R> HD cpx<R> operator*(cpx<R> a, R s) { return {s * a.x, s * a.y}; }
template <typename R> HD cpx<R> operator/(cpx<R> a, R s) { return {a.x / s, a.y / s}; }
template <typename R> HD cpx<R>& operator+=(cpx<R>& a, cpx<R> b) { a.x += b.x; a.y += b.y; return a; }
template <typename R> HD cpx<R>& operator-=(cpx<R>& a, cpx<R> b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename R> HD cpx<R> conj(cpx<R> a) { return {a.x, -a.y}; }
template <typename R> HD R re(cpx<R> a) { return a.x; }
template <typename R> HD R abs2(cpx<R> a) { return a.x * a.x + a.y * a.y; }
HD double conj(double a) { return a; }
HD float conj(float a) { return a; }
HD double re(double a) { return a; }
HD float re(float a) { return a; }
HD double abs2(double a) { return a * a; }
HD float abs2(float a) { return a * a; }

template <typename T> HD T zero_of();
template <> HD double zero_of<double>() { return 0.0; }
template <> HD float zero_of<float>() { return 0.0f; }
template <> HD zd zero_of<zd>() { return zd{0.0, 0.0}; }
template <> HD zf zero_of<zf>() { return zf{0.0f, 0.0f}; }
template <typename T> HD T one_of();
template <> HD double one_of<double>() { return 1.0; }
template <> HD float one_of<float>() { return 1.0f; }
template <> HD zd one_of<zd>() { return zd{1.0, 0.0}; }
template <> HD zf one_of<zf>() { return zf{1.0f, 0.0f}; }

// conversion between precisions (used at the mixed-precision boundary)
template <typename To, typename From> HD To conv(From a);
template <> HD double conv<double, double>(double a) { return a; }
template <> HD float conv<float, double>(double a) { return (float)a; }
template <> HD double conv<double, float>(float a) { return (double)a; }
template <> HD zd conv<zd, zd>(zd a) { return a; }
template <> HD zf conv<zf, zd>(zd a) { return zf{(float)a.x, (float)a.y}; }
template <> HD zd conv<zd, zf>(zf a) { return zd{(double)a.x, (double)a.y}; }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Stream-ordered allocation from the device's default pool.  The pool keeps freed blocks (its
// release threshold is unlimited), so a large request can fail while the pool holds enough
// memory in smaller free blocks: on an out-of-memory error the stream is synchronised, the pool
// returns its unused memory to the device, and the allocation is tried once more.
inline cudaError_t pool_malloc(void** p, size_t bytes, cudaStream_t st) {
    cudaError_t e = cudaMallocAsync(p, bytes, st);
    if (e != cudaErrorMemoryAllocation) return e;
    (void)cudaGetLastError();
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess || cudaMemPoolTrimTo(pool, 0) != cudaSuccess)
        return e;
    e = cudaMallocAsync(p, bytes, st);
    if (e != cudaSuccess) (void)cudaGetLastError();
    return e;
}

}  // namespace tmg
