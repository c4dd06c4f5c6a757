// Tensor-core GEMMs of the learned preconditioner (tcgen05, BF16 operands,
// FP32 accumulation in TMEM), with the epilogues of its node MLPs fused in.
#pragma once

#include <cuda_bf16.h>

#include "tc.cuh"

namespace senkgpu {

constexpr unsigned kTcWaitLimit = 1u << 22;  // polls of an MMA-completion wait before it is declared failed

enum TcEpilogue : int {
    kTcPlain = 0,     // c[row][j] = acc                                    (fp32, ld NO)
    kTcLayerFwd = 1,  // z = acc + bias; zb = bf16(z); h' = h + relu(z); x'[:, :64] = bf16(h')
    kTcDx = 2,        // dh'[j] = dh[j] + acc[j] (j < 64);  dm[j - 64] = acc[j] (j >= 64)
};

struct TcArgs {
    float *c = nullptr;               // kTcPlain output
    const float *bias = nullptr;      // [NO]
    const float *hin = nullptr;       // N x 64 fp32 (residual stream / incoming gradient)
    float *hout = nullptr;            // N x 64 fp32
    __nv_bfloat16 *xout = nullptr;    // next layer's input, N x xld bf16 (columns [0, 64)); may be null
    int xld = 128;
    __nv_bfloat16 *zout = nullptr;    // N x 64 bf16 pre-activation (may be null)
    float *dm = nullptr;              // N x 64 fp32 (kTcDx, columns 64..127 of the product)
};

// Y = epilogue(A * Bt^T) for one tile of 128 rows: A is n x K (bf16, row
// stride lda, 16-byte aligned rows), Bt is NO x K (bf16, row stride K). One CTA
// of 128 threads: all threads stage both tiles into shared memory in the
// K-major core-matrix layout, thread 0 issues K/16 MMAs into a 128 x NO FP32
// TMEM accumulator and commits them to an mbarrier, and warp w reads TMEM lanes
// [32w, 32w+32) (rows) for the epilogue. A wait that runs out sets *status; the
// CTA then waits once more (bounded), frees its TMEM and leaves.
template <int K, int NO, int EPI>
__global__ void __launch_bounds__(128)
k_tc_gemm(const __nv_bfloat16 *__restrict__ A, int lda, const __nv_bfloat16 *__restrict__ Bt, int n, TcArgs args,
          int *status)
{
    static_assert(K % 16 == 0 && K <= 256, "K must be a multiple of 16");
    static_assert(NO == 64 || NO == 128, "NO must be 64 or 128");
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tslot;
    unsigned char *sa = tc_smem;
    unsigned char *sb = tc_smem + 128 * K * 2;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long row0 = (long long)blockIdx.x * 128;

    if (warp == 0) {
        tc::tmem_alloc(&tslot, NO);
        tc::tmem_relinquish();
    }
    if (tid == 0) mbar_init(&bar, 1);
    // stage A (128 x K) and Bt (NO x K): 16-byte chunks of 8 elements
    constexpr int CPR = K / 8;  // chunks per row
    for (int c = tid; c < 128 * CPR; c += 128) {
        const int r = c / CPR, kc = c % CPR;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (row0 + r < n) v = *reinterpret_cast<const uint4 *>(A + (row0 + r) * lda + kc * 8);
        *reinterpret_cast<uint4 *>(sa + tc::kmajor_offset(r, kc * 8, K)) = v;
    }
    for (int c = tid; c < NO * CPR; c += 128) {
        const int r = c / CPR, kc = c % CPR;
        const uint4 v = *reinterpret_cast<const uint4 *>(Bt + (long long)r * K + kc * 8);
        *reinterpret_cast<uint4 *>(sb + tc::kmajor_offset(r, kc * 8, K)) = v;
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tslot;
    if (tid == 0) {
        constexpr uint32_t idesc = tc::idesc_bf16_f32(128, NO);
        const uint32_t a0 = smem_addr(sa), b0 = smem_addr(sb);
#pragma unroll
        for (int s = 0; s < K / 16; s++) {
            const uint64_t ad = tc::smem_desc(a0 + 256u * s, tc::kLbo, K * 16);
            const uint64_t bd = tc::smem_desc(b0 + 256u * s, tc::kLbo, K * 16);
            tc::mma_bf16(tbase, ad, bd, idesc, s > 0 ? 1u : 0u);
        }
        tc::mma_commit(&bar);
    }
    bool ok = mbar_wait_bounded(&bar, 0, kTcWaitLimit);
    if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicExch(status, 1);
        mbar_wait_bounded(&bar, 0, kTcWaitLimit);
        ok = false;
    }
    tc::fence_after_sync();
    if (ok) {
        const long long row = row0 + warp * 32 + lane;
        const bool live = row < n;
#pragma unroll
        for (int c0 = 0; c0 < NO; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (!live) continue;
            if (EPI == kTcPlain) {
#pragma unroll
                for (int q = 0; q < 16; q++) args.c[row * NO + c0 + q] = v[q];
            } else if (EPI == kTcLayerFwd) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int j = c0 + q;
                    const float z = v[q] + args.bias[j];
                    if (args.zout) args.zout[row * 64 + j] = __float2bfloat16_rn(z);
                    const float h = args.hin[row * 64 + j] + fmaxf(z, 0.f);
                    args.hout[row * 64 + j] = h;
                    if (args.xout) args.xout[row * args.xld + j] = __float2bfloat16_rn(h);
                }
            } else {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int j = c0 + q;
                    if (j < 64) args.hout[row * 64 + j] = args.hin[row * 64 + j] + v[q];
                    else args.dm[row * 64 + (j - 64)] = v[q];
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tbase, NO);
    }
}

// out[128][64] += X^T dZ over all n nodes: X is n x 128 (bf16, row stride xld),
// dZ is n x 64 (bf16). Split over node chunks of KC: each CTA accumulates its
// chunks in one TMEM accumulator (lanes = the 128 columns of X, columns = the
// 64 of dZ), transposing both tiles into the K-major layout while staging them,
// and adds its sum to `out` with FP32 atomics. (The launch may add dynamic
// shared memory that the kernel does not touch, to cap resident CTAs.)
template <int KC>
__global__ void __launch_bounds__(128)
k_tc_gemm_tn(const __nv_bfloat16 *__restrict__ X, int xld, const __nv_bfloat16 *__restrict__ dZ, int n,
             float *__restrict__ out, int *status)
{
    static_assert(KC % 16 == 0, "KC must be a multiple of 16");
    __shared__ __align__(1024) unsigned char sa[128 * KC * 2];
    __shared__ __align__(1024) unsigned char sb[64 * KC * 2];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) {
        tc::tmem_alloc(&tslot, 64);
        tc::tmem_relinquish();
    }
    if (tid == 0) mbar_init(&bar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tslot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 64);
    const int nchunks = (n + KC - 1) / KC;
    unsigned phase = 0;
    bool ok = true, any = false;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const long long n0 = (long long)ch * KC;
        // X^T tile: element (feature i, node k) <- X[n0 + k][i]
        for (int c = tid; c < KC * 16; c += 128) {
            const int k = c / 16, i0 = (c % 16) * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (n0 + k < n) v = *reinterpret_cast<const uint4 *>(X + (n0 + k) * xld + i0);
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int q = 0; q < 8; q++)
                *reinterpret_cast<__nv_bfloat16 *>(sa + tc::kmajor_offset(i0 + q, k, KC)) = e[q];
        }
        // dZ^T tile: element (column j, node k) <- dZ[n0 + k][j]
        for (int c = tid; c < KC * 8; c += 128) {
            const int k = c / 8, j0 = (c % 8) * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (n0 + k < n) v = *reinterpret_cast<const uint4 *>(dZ + (n0 + k) * 64 + j0);
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int q = 0; q < 8; q++)
                *reinterpret_cast<__nv_bfloat16 *>(sb + tc::kmajor_offset(j0 + q, k, KC)) = e[q];
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t a0 = smem_addr(sa), b0 = smem_addr(sb);
#pragma unroll
            for (int s = 0; s < KC / 16; s++) {
                const uint64_t ad = tc::smem_desc(a0 + 256u * s, tc::kLbo, KC * 16);
                const uint64_t bd = tc::smem_desc(b0 + 256u * s, tc::kLbo, KC * 16);
                tc::mma_bf16(tbase, ad, bd, idesc, (any || s > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar);
        }
        any = true;
        // the tiles are overwritten next: wait for the MMAs that read them
        bool done = mbar_wait_bounded(&bar, phase, kTcWaitLimit);
        phase ^= 1u;
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicExch(status, 1);
            mbar_wait_bounded(&bar, phase ^ 1u, kTcWaitLimit);
            ok = false;
            break;
        }
        tc::fence_after_sync();
    }
    if (ok && any) {
        const int i = warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < 64; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int q = 0; q < 16; q++) atomicAdd(out + i * 64 + c0 + q, v[q]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tbase, 64);
    }
}

}  // namespace senkgpu
