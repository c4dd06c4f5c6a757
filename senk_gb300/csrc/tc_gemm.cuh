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

// Row stride (floats) of the 128 x NO FP32 result tile that the epilogue
// stages in shared memory: rows stay 16-byte aligned, and the eight lanes of a
// quarter warp that move one float4 each (a row per lane when written from
// TMEM, consecutive columns of one row when read) fall in distinct banks.
template <int NO>
constexpr int kTcTileStride = NO + 4;

// Dynamic shared memory of k_tc_gemm<K, NO>: the two operand tiles, or the
// 128 x NO FP32 result tile of the epilogue, which reuses them once the MMAs
// have completed.
__host__ __device__ constexpr int tc_gemm_smem(int K, int NO)
{
    return (128 * K * 2 + NO * K * 2) > 128 * (NO + 4) * 4 ? (128 * K * 2 + NO * K * 2) : 128 * (NO + 4) * 4;
}

__device__ __forceinline__ void st_bf16x4(__nv_bfloat16 *p, float a, float b, float c, float d)
{
    const __nv_bfloat162 lo = __floats2bfloat162_rn(a, b), hi = __floats2bfloat162_rn(c, d);
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t *>(&lo);
    u.y = *reinterpret_cast<const uint32_t *>(&hi);
    *reinterpret_cast<uint2 *>(p) = u;
}

// Epilogue of k_tc_gemm over the result tile (rows [0, rows) of it valid). Each
// thread owns one group of four consecutive columns and walks rows 128 / G
// apart (G = the row's groups), so every global access is a 16-byte (FP32) or
// 8-byte (BF16) vector and a warp's accesses cover whole rows. The global
// loads of a batch of rows are all issued before the first store.
template <int NO, int EPI>
__device__ __forceinline__ void tc_epilogue(const float *tile, long long row0, int rows, const TcArgs &args)
{
    constexpr int S = kTcTileStride<NO>;
    const int tid = threadIdx.x;
    if constexpr (EPI == kTcPlain) {
        constexpr int G = NO / 4, RP = 128 / G;  // groups per row, rows per pass
        const int j = (tid % G) * 4;
#pragma unroll 4
        for (int rr = tid / G; rr < rows; rr += RP)
            *reinterpret_cast<float4 *>(args.c + (row0 + rr) * NO + j) =
                *reinterpret_cast<const float4 *>(tile + rr * S + j);
    } else {
        // both fused epilogues: 64 columns of h per row (kTcDx: then the 64 of dm)
        constexpr int RP = 8, B = 8;  // rows per pass, passes per batch of loads
        const int j = (tid & 15) * 4, rb = tid >> 4;
        float4 bias = make_float4(0.f, 0.f, 0.f, 0.f);
        if (EPI == kTcLayerFwd) bias = make_float4(args.bias[j], args.bias[j + 1], args.bias[j + 2], args.bias[j + 3]);
#pragma unroll 1
        for (int p0 = 0; p0 < 128 / RP; p0 += B) {
            float4 h[B];
#pragma unroll
            for (int u = 0; u < B; u++) {
                const int rr = rb + RP * (p0 + u);
                h[u] = rr < rows ? __ldg(reinterpret_cast<const float4 *>(args.hin + (row0 + rr) * 64 + j))
                                 : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < B; u++) {
                const int rr = rb + RP * (p0 + u);
                if (rr >= rows) break;
                const long long row = row0 + rr;
                const float4 a = *reinterpret_cast<const float4 *>(tile + rr * S + j);
                if constexpr (EPI == kTcLayerFwd) {
                    const float4 z = make_float4(a.x + bias.x, a.y + bias.y, a.z + bias.z, a.w + bias.w);
                    if (args.zout) st_bf16x4(args.zout + row * 64 + j, z.x, z.y, z.z, z.w);
                    const float4 o = make_float4(h[u].x + fmaxf(z.x, 0.f), h[u].y + fmaxf(z.y, 0.f),
                                                 h[u].z + fmaxf(z.z, 0.f), h[u].w + fmaxf(z.w, 0.f));
                    *reinterpret_cast<float4 *>(args.hout + row * 64 + j) = o;
                    if (args.xout) st_bf16x4(args.xout + row * args.xld + j, o.x, o.y, o.z, o.w);
                } else {
                    *reinterpret_cast<float4 *>(args.hout + row * 64 + j) =
                        make_float4(h[u].x + a.x, h[u].y + a.y, h[u].z + a.z, h[u].w + a.w);
                    *reinterpret_cast<float4 *>(args.dm + row * 64 + j) =
                        *reinterpret_cast<const float4 *>(tile + rr * S + 64 + j);
                }
            }
        }
    }
}

// 16-byte copy global -> shared that completes asynchronously (cp.async);
// with pred false nothing is read and the 16 bytes are zeroed.
__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool pred)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_addr(dst)), "l"(src),
                 "r"(pred ? 16 : 0)
                 : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Y = epilogue(A * Bt^T) for one tile of 128 rows: A is n x K (bf16, row
// stride lda, 16-byte aligned rows), Bt is NO x K (bf16, row stride K). One CTA
// of 128 threads: all threads issue their 16-byte chunks of both tiles as
// asynchronous copies into the K-major core-matrix layout (all in flight at
// once; rows past n are zero-filled), thread 0 issues K/16 MMAs into a
// 128 x NO FP32 TMEM accumulator and commits them to an mbarrier, warp w reads
// TMEM lanes [32w, 32w+32) (rows) into a shared-memory tile, and the epilogue
// (tc_epilogue) then walks the tile with 16-byte vectors along the rows, so
// every global load and store of a warp covers whole rows (all pointers of
// TcArgs 16-byte aligned; xld a multiple of 4). A wait that runs out sets *status;
// the CTA then waits once more (bounded), frees its TMEM and leaves.
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
#pragma unroll 4
    for (int c = tid; c < 128 * CPR; c += 128) {
        const int r = c / CPR, kc = c % CPR;
        const bool in = row0 + r < n;
        cp_async16(sa + tc::kmajor_offset(r, kc * 8, K), in ? A + (row0 + r) * lda + kc * 8 : A, in);
    }
#pragma unroll 4
    for (int c = tid; c < NO * CPR; c += 128) {
        const int r = c / CPR, kc = c % CPR;
        cp_async16(sb + tc::kmajor_offset(r, kc * 8, K), Bt + (long long)r * K + kc * 8, true);
    }
    cp_async_wait_all();
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
        // the MMAs have read the operand tiles: their space holds the result tile
        float *tile = reinterpret_cast<float *>(tc_smem);
        const int r = warp * 32 + lane;
#pragma unroll
        for (int c0 = 0; c0 < NO; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tbase + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int q = 0; q < 16; q += 4)
                *reinterpret_cast<float4 *>(tile + r * kTcTileStride<NO> + c0 + q) =
                    make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
        }
        __syncthreads();
        tc_epilogue<NO, EPI>(tile, row0, (int)min((long long)128, (long long)n - row0), args);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tbase, NO);
    }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Waits until at most `pending` of this thread's committed cp.async groups are in flight.
template <int pending>
__device__ __forceinline__ void cp_async_wait_pending()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(pending) : "memory");
}

// Four 8x8 matrices of 16-bit elements, transposed on the way into registers
// (thread t: row t/4, columns 2(t%4), 2(t%4)+1 of each transposed matrix; the
// row addresses come from threads 8j..8j+7 for matrix j).
__device__ __forceinline__ void ldsm_x4_trans(uint32_t addr, uint32_t (&r)[4])
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr)
                 : "memory");
}

// Stores four 8x8 matrices from the same register layout, row r of matrix j
// to the address of thread 8j + r.
__device__ __forceinline__ void stsm_x4(uint32_t addr, const uint32_t (&r)[4])
{
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3])
                 : "memory");
}

// Shared-memory layout of k_tc_gemm_tn<KC>: two operand stages (A = X^T tile,
// 128 x KC, then B = dZ^T tile, 64 x KC, K-major core matrices), then two raw
// stages (the X rows, 128 features, and the dZ rows, 64, of KC nodes, each row
// padded by 16 bytes so that the eight rows one ldmatrix reads fall in
// different banks).
template <int KC>
struct TnLayout {
    static constexpr int kXrs = 128 * 2 + 16, kZrs = 64 * 2 + 16;  // raw row strides (bytes)
    static constexpr int kRaw = KC * (kXrs + kZrs);                 // one raw stage
    static constexpr int kOpA = 128 * KC * 2, kOp = kOpA + 64 * KC * 2;  // one operand stage
    static constexpr int kBytes = 2 * kOp + 2 * kRaw;
};

// Transposes a raw stage's tile of `F` features x KC nodes (rows = nodes,
// stride RS bytes) into the K-major operand tile (rows = features, K = nodes):
// each warp takes groups of four 8x8 blocks (one node block, four
// consecutive feature blocks), reads them transposed with ldmatrix and writes
// each transposed block's rows (eight nodes of one feature, 16 bytes) to its
// core matrix with stmatrix.
template <int KC, int F, int RS>
__device__ __forceinline__ void tn_transpose(const unsigned char *raw, unsigned char *op, int warp, int lane)
{
    constexpr int FB = F / 8, GROUPS = (KC / 8) * FB / 4;
    static_assert(FB % 4 == 0, "four feature blocks per group");
    const int j = lane >> 3, r = lane & 7;
    for (int g = warp; g < GROUPS; g += 4) {
        const int b = 4 * g + j;  // this lane's block: node block kb, feature block fb
        const int kb = b / FB, fb = b % FB;
        uint32_t v[4];
        ldsm_x4_trans(smem_addr(raw + (kb * 8 + r) * RS + fb * 16), v);
        stsm_x4(smem_addr(op + tc::kmajor_offset(fb * 8 + r, kb * 8, KC)), v);
    }
}

// out[128][64] += X^T dZ over all n nodes: X is n x 128 (bf16, row stride xld,
// a multiple of 8, 16-byte aligned rows), dZ is n x 64 (bf16). Split over node
// chunks of KC: CTA b takes chunks b, b + gridDim.x, ... in a two-stage
// pipeline: the raw rows of chunk i+1 are copied (cp.async, rows past n
// zero-filled) while chunk i is transposed into one of two operand stages and
// the MMAs of chunk i-1 run on the other; thread 0 issues KC/16 MMAs per chunk
// into one TMEM accumulator (lanes = the 128 columns of X, columns = the 64 of
// dZ) and commits them to the stage's mbarrier, which the CTA waits for before
// it overwrites that stage. The sum is added to `out` with FP32 atomics. A wait
// that runs out sets *status; the CTA then waits once more (bounded) for the
// last MMAs it issued, frees its TMEM and leaves.
template <int KC>
__global__ void __launch_bounds__(128)
k_tc_gemm_tn(const __nv_bfloat16 *__restrict__ X, int xld, const __nv_bfloat16 *__restrict__ dZ, int n,
             float *__restrict__ out, int *status)
{
    static_assert(KC % 16 == 0, "KC must be a multiple of 16");
    using Lt = TnLayout<KC>;
    extern __shared__ __align__(1024) unsigned char tns[];
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    auto op = [&](int b) { return tns + b * Lt::kOp; };
    auto raw = [&](int b) { return tns + 2 * Lt::kOp + b * Lt::kRaw; };
    if (warp == 0) {
        tc::tmem_alloc(&tslot, 64);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tslot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 64);
    const int nchunks = (n + KC - 1) / KC;
    auto stage_raw = [&](int ch, unsigned char *rw) {
        const long long n0 = (long long)ch * KC;
        for (int c = tid; c < KC * 16; c += 128) {
            const int k = c >> 4, q = c & 15;
            const bool in = n0 + k < n;
            cp_async16(rw + k * Lt::kXrs + q * 16, in ? X + (n0 + k) * xld + q * 8 : X, in);
        }
        for (int c = tid; c < KC * 8; c += 128) {
            const int k = c >> 3, q = c & 7;
            const bool in = n0 + k < n;
            cp_async16(rw + KC * Lt::kXrs + k * Lt::kZrs + q * 16, in ? dZ + (n0 + k) * 64 + q * 8 : dZ, in);
        }
        cp_async_commit();
    };
    if ((int)blockIdx.x < nchunks) stage_raw(blockIdx.x, raw(0));
    bool ok = true;
    int last = -1;  // the last iteration whose MMAs were issued
    for (int it = 0, ch = blockIdx.x; ch < nchunks; it++, ch += gridDim.x) {
        const int b = it & 1;
        if (ch + (int)gridDim.x < nchunks) {
            stage_raw(ch + gridDim.x, raw(b ^ 1));  // read (transposed) in the previous iteration
            cp_async_wait_pending<1>();
        } else {
            cp_async_wait_pending<0>();
        }
        __syncthreads();  // chunk ch's raw rows are in raw[b]
        if (it >= 2) {    // the MMAs of iteration it-2 read op[b]
            const bool done = mbar_wait_bounded(&bar[b], (unsigned)((it >> 1) - 1) & 1u, kTcWaitLimit);
            if (__syncthreads_or(!done)) {
                if (tid == 0) atomicExch(status, 1);
                ok = false;
                break;
            }
        }
        tn_transpose<KC, 128, Lt::kXrs>(raw(b), op(b), warp, lane);
        tn_transpose<KC, 64, Lt::kZrs>(raw(b) + KC * Lt::kXrs, op(b) + Lt::kOpA, warp, lane);
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) {
            const uint32_t a0 = smem_addr(op(b)), b0 = smem_addr(op(b) + Lt::kOpA);
#pragma unroll
            for (int s = 0; s < KC / 16; s++) {
                const uint64_t ad = tc::smem_desc(a0 + 256u * s, tc::kLbo, KC * 16);
                const uint64_t bd = tc::smem_desc(b0 + 256u * s, tc::kLbo, KC * 16);
                tc::mma_bf16(tbase, ad, bd, idesc, (it > 0 || s > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar[b]);
        }
        last = it;
    }
    cp_async_wait_pending<0>();  // copies still in flight (after an abort) land before the CTA leaves
    if (last >= 0) {
        // the last commit covers every MMA issued before it
        const bool done = mbar_wait_bounded(&bar[last & 1], (unsigned)(last >> 1) & 1u, kTcWaitLimit);
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicExch(status, 1);
            mbar_wait_bounded(&bar[last & 1], (unsigned)(last >> 1) & 1u, kTcWaitLimit);
            ok = false;
        }
    }
    tc::fence_after_sync();
    if (ok && last >= 0) {
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
