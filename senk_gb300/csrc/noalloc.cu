// Column dot products of tall-skinny vectors that allocate no device memory.
//
// Some callers cannot allocate device memory at the point where they need a
// reduction: an application that reserves all of the GPU's memory for its own
// pool at start-up and forbids any later cudaMalloc, or a latency-critical loop
// in which cudaMalloc/cudaFree (which can synchronise the whole device) would
// stall other streams. senk_dev_dot_d keeps its reduction scratch in buffers it
// allocates on first use; this entry point runs the same kernel with its scratch
// in a fixed-size array that is part of the library's device image instead.
// The caller still provides the inputs and the output.
#include <mutex>

#include "device.hpp"

namespace senkgpu {
namespace {

constexpr int kNoAllocMaxCols = 16;           // most columns per call
constexpr int kNoAllocCtas = 2 * kNumSMs;     // most CTAs per column block (grid x): 2 per SM of a GB300
constexpr size_t kNoAllocTicketBytes = 256;   // ticket, padded to keep the partials aligned
constexpr size_t kNoAllocScratchBytes =
    kNoAllocTicketBytes + sizeof(double) * (size_t)kNoAllocMaxCols * kNoAllocCtas;  // 39,168 bytes

// Reduction scratch: [0, 4) the last-CTA ticket, [256, ...) one FP64 partial per
// CTA and column. Every device that loads the library holds this array until the
// process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[64] = {};  // device address of g_noalloc_scratch, per device

// The array's name is only a host-side stand-in in host code; its device
// address is looked up once per device, with that device current, and kept for
// the life of the process (a cudaDeviceReset between calls is not supported: the
// kept address would belong to the destroyed context).
unsigned char *noalloc_scratch()
{
    int dev = 0;
    SENK_CUDA(cudaGetDevice(&dev));
    SENK_REQUIRE(dev >= 0 && dev < 64, "device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        SENK_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[dev] = p;
    }
    return static_cast<unsigned char *>(g_noalloc_addr[dev]);
}

}  // namespace
}  // namespace senkgpu

using namespace senkgpu;

extern "C" int senk_dev_multidot_d_noalloc(const double *V, long long ldv, int nv, const double *w, int N,
                                           double *out, void *stream)
{
    return guarded("senk_dev_multidot_d_noalloc", [&] {
        SENK_REQUIRE(nv >= 1 && nv <= kNoAllocMaxCols,
                     "nv = " + std::to_string(nv) + " columns is outside [1, 16], the most this entry point's "
                     "fixed scratch holds");
        SENK_REQUIRE(N >= 0, "N must be non-negative");
        SENK_REQUIRE(out != nullptr, "out is null");
        cudaStream_t s = (cudaStream_t)stream;
        if (N == 0) {
            SENK_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * nv, s));
            return (int)kOk;
        }
        SENK_REQUIRE(V && w && ldv >= N, "null input or ldv < N");
        unsigned char *base = noalloc_scratch();
        unsigned *ticket = reinterpret_cast<unsigned *>(base);
        double *part = reinterpret_cast<double *>(base + kNoAllocTicketBytes);
        // The ticket must start at zero; a call that failed part-way could have
        // left it set.
        SENK_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s));
        // 2 CTAs per SM of this device, capped by the partials the array holds
        const int grid = std::min(stream_grid(N, kThreads, 2), kNoAllocCtas);
        k_multidot<double, false><<<dim3(grid, (nv + 7) / 8), kThreads, 0, s>>>(V, ldv, nv, w, N, part, ticket, out,
                                                                               nullptr, nullptr);
        SENK_LAUNCH_CHECK();
        return (int)kOk;
    });
}
