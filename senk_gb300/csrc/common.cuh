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

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Barrier `id` (1..15) over the first `nthreads` threads of the CTA (a multiple
// of 32); returns whether any of them passed v = true.
__device__ __forceinline__ bool named_bar_or(int id, int nthreads, bool v)
{
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.s32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.s32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((int)v), "r"(id), "r"(nthreads)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void named_bar(int id, int nthreads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
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

// Sum of the grid's partials p[0..P), by every thread of the (last) CTA; the
// total is returned in thread 0, as block_sum. Thread t adds p[t],
// p[t + blockDim.x], ... into eight independent sums, so its loads are in
// flight together instead of one memory latency apart. The order of the
// additions depends only on P and the block size.
__device__ __forceinline__ double cta_sum_partials(const double *p, int P, double *sh)
{
    double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int S = blockDim.x;
    int i = threadIdx.x;
    for (; i + 7 * S < P; i += 8 * S) {
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] += __ldcg(p + i + u * S);
    }
    for (; i < P; i += S) a[0] += __ldcg(p + i);
    return block_sum(((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7])), sh);
}

// Per-column totals of the grid's partials part[k * P + p] (k < nv), by every
// thread of the (last) CTA: one column uses the whole CTA (cta_sum_partials),
// several take a warp each, every lane with eight independent sums.
// store(k, total) runs once per column. Fixed order for given P, nv and block.
template <typename F>
__device__ __forceinline__ void cta_sum_columns(const double *part, int P, int nv, double *sh, F store)
{
    if (nv == 1) {
        const double s = cta_sum_partials(part, P, sh);
        if (threadIdx.x == 0) store(0, s);
        return;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = wid; k < nv; k += nw) {
        const double *p = part + (long long)k * P;
        double a[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        int i = lane;
        for (; i + 7 * 32 < P; i += 256) {
#pragma unroll
            for (int u = 0; u < 8; u++) a[u] += __ldcg(p + i + 32 * u);
        }
        for (; i < P; i += 32) a[0] += __ldcg(p + i);
        const double s = warp_sum(((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7])));
        if (lane == 0) store(k, s);
    }
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
