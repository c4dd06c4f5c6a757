// Shared device/host helpers for the sm_103a SenK kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

namespace senkgpu {

// ------------------------------------------------------------------ errors
// Status codes returned by every extern "C" entry point (0 = success).
enum Status : int {
    kOk = 0,
    kErrArg = 1,         // invalid argument (sizes, unsupported block shape, null pointer)
    kErrCuda = 2,        // a CUDA runtime call failed
    kErrAlloc = 3,       // device or host allocation failed
    kErrBreakdown = 4,   // a Krylov scalar became zero/NaN (division by zero in the reference)
    kErrZeroPivot = 5,   // ILU(0) met a zero pivot (the reference exits)
    kErrNotConverged = 6 // iteration limit reached (informational; x is still updated)
};

void set_last_error(const std::string &msg);

struct CudaError {
    cudaError_t code;
    const char *what;
    const char *file;
    int line;
};

#define SENK_CUDA(call)                                                               \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) throw ::senkgpu::CudaError{e_, #call, __FILE__, __LINE__}; \
    } while (0)

#define SENK_LAUNCH_CHECK() SENK_CUDA(cudaGetLastError())

// ---------------------------------------------------------------- geometry
constexpr int kNumSMs = 152;    // GB300 (2 dies x 76 SMs): used only if the device query fails
constexpr int kThreads = 256;   // default CTA size of the streaming kernels

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// SMs of the current device (cudaDevAttrMultiProcessorCount), looked up once per
// device; kNumSMs if the query fails.
inline int sm_count()
{
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kNumSMs;
    if (cache[dev] <= 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return kNumSMs;
        cache[dev] = v;
    }
    return cache[dev];
}

// Grid size for a grid-stride streaming kernel: enough CTAs for every SM to hold
// `per_sm` resident CTAs, but never more than the work needs.
inline int stream_grid(long long n_items, int items_per_cta, int per_sm = 4)
{
    long long need = (n_items + items_per_cta - 1) / items_per_cta;
    long long cap = (long long)sm_count() * per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

// ------------------------------------------------------------ load helpers
// Streamed matrix data: read once per sweep, should not evict the vectors that
// the gathers reuse from L2.
template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }

template <typename T>
__device__ __forceinline__ T ld_keep(const T *p) { return __ldg(p); }

// ------------------------------------------------- TMA bulk copy + mbarrier
__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// One bulk copy global -> shared (both 16-byte aligned, bytes a multiple of 16);
// completion is counted on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned phase)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait for phase `phase` of `bar`: returns false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned phase, unsigned limit)
{
    for (unsigned i = 0; i < limit; i++)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Programmatic dependent launch: let the next kernel in the stream start its
// prologue, and wait until the previous kernel has completed and its writes are
// visible.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ------------------------------------------------------- warp reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the CTA; result valid in thread 0. `sh` holds one value per warp.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    T r = 0;
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        r = lane < nw ? sh[lane] : T(0);
        r = warp_sum(r);
    }
    __syncthreads();
    return r;
}

// "Last CTA finishes" protocol for grid-wide reductions without a second launch.
// Every CTA writes its partials, fences, and bumps a ticket; the CTA that draws
// the last ticket sees all partials and finalizes (then resets the ticket so the
// same counter serves the next launch, including inside a replayed CUDA graph).
__device__ __forceinline__ bool last_cta_arrives(unsigned int *ticket, unsigned int total)
{
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(ticket, 1u);
        is_last = (t == total - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        if (threadIdx.x == 0) *ticket = 0;
    }
    return is_last;
}

}  // namespace senkgpu
