// Learned preconditioner: a message-passing network over the matrix graph whose
// output corrects the ILU(0) application,
//     K(r) = ILU(r) + (||r||_rms / d) * net(r),
// used inside flexible GCR(m). No counterpart in the reference.
//
// Network (all node-wise, N nodes = matrix rows, hidden width 64):
//   features f_i = (a_ii / d, sum_j |a_ij| / d, r_i / ||r||_rms), d = mean a_ii
//   h0 = relu(f W_in + b_in)                                       (3 -> 64)
//   layer l = 0..3: m = W h (W_ij = |a_ij| / sum_{k != i} |a_ik|, i != j)
//                   z = [h, m] Theta_l + beta_l                     (128 -> 64, tcgen05)
//                   h <- h + relu(z)
//   c = h w_out + b_out                                            (64 -> 1)
// Training objective for a residual/error pair (r, e), by default in residual
// space: q = (r - A ILU(r)) / ||r||_rms, loss = |A c / d - q|^2 / |q|^2 (what the
// correction leaves of the ILU residual); or in error space:
// t = (e - ILU(r)) d / ||r||_rms, loss = |c - t|^2 / |t|^2. GEMM operands are BF16
// with FP32 accumulation; the residual stream, gradients and Adam state are FP32.
#include <cmath>
#include <vector>

#include "device.hpp"
#include "tc_gemm.cuh"

namespace senkgpu {

namespace {

// Dynamic shared memory of the tensor-core GEMMs. Besides the two tiles it caps
// the CTAs resident on an SM so that their TMEM accumulators fit in its 512
// columns: 48 KB -> 4 CTAs x 64 columns; 66 KB -> 3 CTAs x 128 columns.
constexpr int kSmemFwd = tc_gemm_smem(128, 64);  // 48 KB of operand tiles
constexpr int kSmemDx = tc_gemm_smem(64, 128);   // 66 KB: the 128 x 132 FP32 result tile
constexpr int kSmemTn = TnLayout<64>::kBytes;    // 100 KB of pipeline stages: 2 CTAs x 64 columns

constexpr int kHid = 64;
constexpr int kLayers = 4;
constexpr int kIn = 3;
// parameter vector: W_in[3][64], b_in[64], {Theta_l[128][64], beta_l[64]} x 4, w_out[64], b_out
constexpr int kOffWin = 0;
constexpr int kOffBin = kOffWin + kIn * kHid;
constexpr int kOffLayer = kOffBin + kHid;
constexpr int kLayerSize = 2 * kHid * kHid + kHid;
constexpr int kOffWout = kOffLayer + kLayers * kLayerSize;
constexpr int kOffBout = kOffWout + kHid;
constexpr int kParams = kOffBout + 1;

using bf16 = __nv_bfloat16;

__device__ __forceinline__ float relu(float v) { return v > 0.f ? v : 0.f; }

// ||r||_rms and 1/||r||_rms of a double vector (one block per slice, last CTA finishes)
template <typename T>
__global__ void __launch_bounds__(kThreads) k_rms(const T *r, long long n, double *part, unsigned *ticket, float *out)
{
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s += (double)r[i] * (double)r[i];
    __shared__ double sh[32];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
    if (last_cta_arrives(ticket, gridDim.x)) {
        const double t = cta_sum_partials(part, gridDim.x, sh);
        if (threadIdx.x == 0) {
            const double rms = sqrt(t / (double)n);
            out[0] = (float)rms;
            out[1] = rms > 0 ? (float)(1.0 / rms) : 0.f;
        }
    }
}

// h0 = relu(f W_in + b_in), one thread per (node, feature); X0[:, :64] = bf16(h0)
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_encode(const float *fd, const float *fs, const T *r, const float *rms, const float *P, float *H, bf16 *X, long long n)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n * kHid) return;
    const long long i = idx / kHid;
    const int j = (int)(idx % kHid);
    const float f2 = (float)r[i] * rms[1];
    const float z = fd[i] * P[kOffWin + j] + fs[i] * P[kOffWin + kHid + j] + f2 * P[kOffWin + 2 * kHid + j] +
                    P[kOffBin + j];
    const float h = relu(z);
    H[idx] = h;
    X[i * 128 + j] = __float2bfloat16_rn(h);
}

// m = W h, 8 lanes per row (4 rows per warp), lane k of a row holding
// features 8k..8k+7 (one 16-byte load of bf16 per entry); h = X[:, :64]
// (bf16), m -> X[:, 64:128] (bf16), FP32 accumulation in the entries' order.
__global__ void __launch_bounds__(kThreads)
k_aggregate(const int *__restrict__ rptr, const int *__restrict__ cind, const float *__restrict__ w, bf16 *X,
            long long n)
{
    const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const int sub = threadIdx.x & 7;
    if (row >= n) return;
    float a[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int p1 = rptr[row + 1];
#pragma unroll 4
    for (int p = rptr[row]; p < p1; p++) {
        const float wv = w[p];
        const uint4 u = *reinterpret_cast<const uint4 *>(X + (long long)cind[p] * 128 + 8 * sub);
        const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            a[2 * k] += wv * __bfloat162float(h[k].x);
            a[2 * k + 1] += wv * __bfloat162float(h[k].y);
        }
    }
    uint4 o;
    uint32_t *ow = reinterpret_cast<uint32_t *>(&o);
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const __nv_bfloat162 v = __floats2bfloat162_rn(a[2 * k], a[2 * k + 1]);
        ow[k] = *reinterpret_cast<const uint32_t *>(&v);
    }
    *reinterpret_cast<uint4 *>(X + row * 128 + 64 + 8 * sub) = o;
}

// dH += W^T dM (fp32), 8 lanes per row of W^T (4 rows per warp), lane k of a
// row holding features 8k..8k+7 (two 16-byte loads per entry).
__global__ void __launch_bounds__(kThreads)
k_aggregate_back(const int *__restrict__ rptr, const int *__restrict__ cind, const float *__restrict__ w,
                 const float *__restrict__ dM, float *__restrict__ dH, long long n)
{
    const long long row = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 3;
    const int sub = threadIdx.x & 7;
    if (row >= n) return;
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    const int p1 = rptr[row + 1];
#pragma unroll 4
    for (int p = rptr[row]; p < p1; p++) {
        const float wv = w[p];
        const float4 *d = reinterpret_cast<const float4 *>(dM + (long long)cind[p] * 64 + 8 * sub);
        const float4 d0 = d[0], d1 = d[1];
        a0.x += wv * d0.x;
        a0.y += wv * d0.y;
        a0.z += wv * d0.z;
        a0.w += wv * d0.w;
        a1.x += wv * d1.x;
        a1.y += wv * d1.y;
        a1.z += wv * d1.z;
        a1.w += wv * d1.w;
    }
    float4 *o = reinterpret_cast<float4 *>(dH + row * 64 + 8 * sub);
    float4 v0 = o[0], v1 = o[1];
    v0.x += a0.x;
    v0.y += a0.y;
    v0.z += a0.z;
    v0.w += a0.w;
    v1.x += a1.x;
    v1.y += a1.y;
    v1.z += a1.z;
    v1.w += a1.w;
    o[0] = v0;
    o[1] = v1;
}

// Inference epilogue: out_i = ilu_i + (rms / d) * (h_i . w_out + b_out); warp per node.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_decode_apply(const float *H, const float *P, const float *rms, float inv_d, T *out, long long n)
{
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const float2 h = *reinterpret_cast<const float2 *>(H + i * 64 + 2 * lane);
    float s = h.x * P[kOffWout + 2 * lane] + h.y * P[kOffWout + 2 * lane + 1];
    s = warp_sum(s);
    if (lane == 0) out[i] = (T)((double)out[i] + (double)(rms[0] * inv_d) * (double)(s + P[kOffBout]));
}

// t_i = (e_i - ilu_i) d / rms; sum t^2 -> acc[0] (last CTA)
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_target(const T *e, const T *ilu, const float *rms, float d, float *t, long long n, double *part, unsigned *ticket,
         double *acc)
{
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = (float)(((double)e[i] - (double)ilu[i]) * (double)d * (double)rms[1]);
        t[i] = v;
        s += (double)v * v;
    }
    __shared__ double sh[32];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
    if (last_cta_arrives(ticket, gridDim.x)) {
        const double u = cta_sum_partials(part, gridDim.x, sh);
        if (threadIdx.x == 0) acc[0] = u;
    }
}

// dZ = bf16(dH (.) [z > 0]); grad beta += column sums of the FP32 product.
// Block of 256 threads = 16 nodes x 16 groups of 4 features (16-byte loads of
// dH, 8-byte loads of z), grid-stride over nodes.
__global__ void __launch_bounds__(kThreads)
k_relu_back(const float *dH, const bf16 *Z, bf16 *dZ, float *gbeta, long long n)
{
    const int j = (threadIdx.x & 15) * 4, sub = threadIdx.x >> 4;
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (long long i = (long long)blockIdx.x * 16 + sub; i < n; i += (long long)gridDim.x * 16) {
        const uint2 zz = __ldg(reinterpret_cast<const uint2 *>(Z + i * 64 + j));
        const float4 d = __ldg(reinterpret_cast<const float4 *>(dH + i * 64 + j));
        const __nv_bfloat162 z01 = *reinterpret_cast<const __nv_bfloat162 *>(&zz.x);
        const __nv_bfloat162 z23 = *reinterpret_cast<const __nv_bfloat162 *>(&zz.y);
        const float4 g = make_float4(__bfloat162float(z01.x) > 0.f ? d.x : 0.f, __bfloat162float(z01.y) > 0.f ? d.y : 0.f,
                                     __bfloat162float(z23.x) > 0.f ? d.z : 0.f, __bfloat162float(z23.y) > 0.f ? d.w : 0.f);
        st_bf16x4(dZ + i * 64 + j, g.x, g.y, g.z, g.w);
        s.x += g.x;
        s.y += g.y;
        s.z += g.z;
        s.w += g.w;
    }
    __shared__ float sh[16][64];
    sh[sub][j] = s.x;
    sh[sub][j + 1] = s.y;
    sh[sub][j + 2] = s.z;
    sh[sub][j + 3] = s.w;
    __syncthreads();
    if (threadIdx.x < 64) {
        float t = 0.f;
#pragma unroll
        for (int k = 0; k < 16; k++) t += sh[k][threadIdx.x];
        atomicAdd(gbeta + threadIdx.x, t);
    }
}

// Encoder backward: dz = dH0 (.) [z0 > 0] (z0 recomputed); grad W_in += f dz, grad b_in += dz.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_encode_back(const float *fd, const float *fs, const T *r, const float *rms, const float *P, const float *dH, float *G,
              long long n)
{
    const int j = threadIdx.x & 63, sub = threadIdx.x >> 6;
    float s0 = 0, s1 = 0, s2 = 0, sb = 0;
    const float w0 = P[kOffWin + j], w1 = P[kOffWin + kHid + j], w2 = P[kOffWin + 2 * kHid + j], b = P[kOffBin + j];
    for (long long i = (long long)blockIdx.x * 4 + sub; i < n; i += (long long)gridDim.x * 4) {
        const float f2 = (float)r[i] * rms[1];
        const float z = fd[i] * w0 + fs[i] * w1 + f2 * w2 + b;
        const float g = z > 0.f ? dH[i * 64 + j] : 0.f;
        s0 += g * fd[i];
        s1 += g * fs[i];
        s2 += g * f2;
        sb += g;
    }
    __shared__ float sh[4][4][64];
    sh[0][sub][j] = s0;
    sh[1][sub][j] = s1;
    sh[2][sub][j] = s2;
    sh[3][sub][j] = sb;
    __syncthreads();
    if (threadIdx.x < 64) {
        float a[4];
        for (int q = 0; q < 4; q++) a[q] = sh[q][0][j] + sh[q][1][j] + sh[q][2][j] + sh[q][3][j];
        atomicAdd(G + kOffWin + j, a[0]);
        atomicAdd(G + kOffWin + kHid + j, a[1]);
        atomicAdd(G + kOffWin + 2 * kHid + j, a[2]);
        atomicAdd(G + kOffBin + j, a[3]);
    }
}

// Adam (decoupled moments, bias-corrected), then the BF16 weight copies:
// Theta_l (128 x 64) and its transpose (64 x 128).
// ||G||^2 into *out (one CTA)
__global__ void __launch_bounds__(1024) k_grad_norm2(const float *G, int np, float *out)
{
    float s = 0.f;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += G[i] * G[i];
    __shared__ float sh[32];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) *out = s;
}

// Adam with the gradient scaled to global norm at most `clip` (clip <= 0: off).
__global__ void __launch_bounds__(kThreads)
k_adam(float *P, const float *G, float *M, float *V, int np, float lr, float b1, float b2, float eps, float c1,
       float c2, const float *norm2, float clip)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float gn = sqrtf(*norm2);
    const float gs = (clip > 0.f && gn > clip) ? clip / gn : 1.f;
    const float g = G[i] * gs;
    const float m = b1 * M[i] + (1.f - b1) * g;
    const float v = b2 * V[i] + (1.f - b2) * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m * c1) / (sqrtf(v * c2) + eps);
}

__global__ void __launch_bounds__(kThreads) k_weights_bf16(const float *P, bf16 *Wb, bf16 *WTb)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kLayers * 128 * 64) return;
    const int l = idx / (128 * 64), e = idx % (128 * 64), i = e / 64, j = e % 64;
    const bf16 v = __float2bfloat16_rn(P[kOffLayer + l * kLayerSize + e]);
    Wb[idx] = v;                                  // Theta_l[i][j]
    WTb[(long long)l * 128 * 64 + j * 128 + i] = v;  // Theta_l^T[j][i]
}

// c_i = h_i . w_out + b_out, warp per node
__global__ void __launch_bounds__(kThreads) k_decode_c(const float *H, const float *P, float *c, long long n)
{
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n) return;
    const float2 h = *reinterpret_cast<const float2 *>(H + i * 64 + 2 * lane);
    const float v = warp_sum(h.x * P[kOffWout + 2 * lane] + h.y * P[kOffWout + 2 * lane + 1]);
    if (lane == 0) c[i] = v + P[kOffBout];
}

// Least-squares step of the correction: alpha = (q . y) / (y . y) with
// q = r - A u (u = ILU(r)) and y = A c (c the scaled correction), i.e. the alpha
// that minimises |r - A (u + alpha c)|; 0 when y = 0. Last CTA finishes; part
// holds 2 * gridDim.x partials.
__global__ void __launch_bounds__(kThreads)
k_step_alpha(const double *r, const double *au, const double *y, long long n, double *part, unsigned *ticket,
             double *alpha)
{
    double a = 0, b = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double yi = y[i];
        a += (r[i] - au[i]) * yi;
        b += yi * yi;
    }
    __shared__ double sh[32];
    a = block_sum(a, sh);
    b = block_sum(b, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
    if (last_cta_arrives(ticket, gridDim.x)) {
        const double ta = cta_sum_partials(part, gridDim.x, sh);
        const double tb = cta_sum_partials(part + gridDim.x, gridDim.x, sh);
        if (threadIdx.x == 0) *alpha = tb > 0 ? ta / tb : 0.0;
    }
}

// out += alpha * c
__global__ void __launch_bounds__(kThreads) k_add_step(double *out, const double *c, const double *alpha, long long n)
{
    const double a = *alpha;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] += a * c[i];
}

// Error-space loss: dc = 2 (c - t) / acc[0]; acc[1] += sum (c - t)^2
__global__ void __launch_bounds__(kThreads) k_loss_error(const float *c, const float *t, float *dc, double *acc, long long n)
{
    const float inv = acc[0] > 0 ? (float)(1.0 / acc[0]) : 0.f;
    double ls = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float diff = c[i] - t[i];
        dc[i] = 2.f * diff * inv;
        ls += (double)diff * diff;
    }
    __shared__ double sh[32];
    ls = block_sum(ls, sh);
    if (threadIdx.x == 0) atomicAdd(acc + 1, ls);
}

// Residual-space target: qh = (r - A ILU(r)) / rms; acc[0] += sum qh^2
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_resid_target(const T *r, const T *ailu, const float *rms, float *qh, double *acc, long long n)
{
    double s = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float v = (float)(((double)r[i] - (double)ailu[i]) * (double)rms[1]);
        qh[i] = v;
        s += (double)v * v;
    }
    __shared__ double sh[32];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) atomicAdd(acc, s);
}

// y = alpha * (B x) with B in CSR (FP32 values), thread per row; with qh: the
// residual e = (B x) / d - qh, acc[1] += sum e^2.
__global__ void __launch_bounds__(kThreads)
k_spmv_loss(const int *rp, const int *ci, const float *bv, const float *x, float *y, long long n, float inv_d,
            const float *qh, double *acc)
{
    double ls = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float a = 0.f;
        for (int p = rp[i]; p < rp[i + 1]; p++) a += bv[p] * x[ci[p]];
        const float e = a * inv_d - qh[i];
        y[i] = e;
        ls += (double)e * e;
    }
    __shared__ double sh[32];
    ls = block_sum(ls, sh);
    if (threadIdx.x == 0) atomicAdd(acc + 1, ls);
}

// dc = 2 / (d acc[0]) * (B^T e), thread per row of B^T
__global__ void __launch_bounds__(kThreads)
k_spmv_grad(const int *rp, const int *ci, const float *bv, const float *e, float *dc, long long n, float inv_d,
            const double *acc)
{
    const float sc = acc[0] > 0 ? (float)(2.0 * inv_d / acc[0]) : 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float a = 0.f;
        for (int p = rp[i]; p < rp[i + 1]; p++) a += bv[p] * e[ci[p]];
        dc[i] = sc * a;
    }
}

// Decoder backward: dH4 = dc w_out; grad w_out += dc h; grad b_out += dc (warp per node)
__global__ void __launch_bounds__(kThreads)
k_decode_back(const float *H, const float *P, const float *dc, float *dH, float *G, long long n)
{
    __shared__ float gw[kThreads / 32][kHid];
    __shared__ float gb[kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const float w0 = P[kOffWout + 2 * lane], w1 = P[kOffWout + 2 * lane + 1];
    float g0 = 0.f, g1 = 0.f, gbs = 0.f;
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const float2 h = *reinterpret_cast<const float2 *>(H + i * 64 + 2 * lane);
        const float g = dc[i];
        *reinterpret_cast<float2 *>(dH + i * 64 + 2 * lane) = make_float2(g * w0, g * w1);
        g0 += g * h.x;
        g1 += g * h.y;
        gbs += g;
    }
    gw[wid][2 * lane] = g0;
    gw[wid][2 * lane + 1] = g1;
    if (lane == 0) gb[wid] = gbs;
    __syncthreads();
    if (threadIdx.x < kHid) {
        float s = 0;
        for (int w = 0; w < kThreads / 32; w++) s += gw[w][threadIdx.x];
        atomicAdd(G + kOffWout + threadIdx.x, s);
    }
    if (threadIdx.x == 0) {
        float s = 0;
        for (int w = 0; w < kThreads / 32; w++) s += gb[w];
        atomicAdd(G + kOffBout, s);
    }
}

}  // namespace

// ------------------------------------------------------------------ the network

struct Mpnn {
    // parameters and optimiser state (device, FP32)
    DevBuf<float> P, G, M, V;
    DevBuf<bf16> Wb, WTb;  // per layer Theta (128x64) and Theta^T (64x128)
    int step = 0;
    // bound graph
    const void *bound = nullptr;  // the System it was bound to
    long long n = 0;
    float d = 1.f;                // mean diagonal
    DevBuf<int> wr, wc, tr, tcol; // W and W^T (CSR)
    DevBuf<float> wv, tv, fd, fs;
    DevBuf<int> ar, ac, atr, atc; // A and A^T (CSR, FP32 values) for the residual-space loss
    DevBuf<float> av, atv, cbuf, dcb, ebuf;
    DevBuf<double> ailu;          // A ILU(r)
    DevBuf<double> cstep, acstep, alpha;  // scaled correction c, A c, and the step alpha
    int loss_mode = 1;            // 0: error space, 1: residual space
    float clip = 1.0f;            // global gradient-norm clip of the Adam step (<= 0: off)
    int step_mode = 1;            // 0: K = ILU + c, 1: K = ILU + alpha c (least-squares alpha, the default)
    DevBuf<float> gnorm;
    // activations
    DevBuf<bf16> X[kLayers], Z[kLayers], dZ;
    DevBuf<float> H[kLayers + 1], dH, dH2, dM, t;
    DevBuf<float> rms;            // rms, 1/rms
    DevBuf<double> red, acc;
    DevBuf<unsigned> ticket;
    DevBuf<int> status;

    void init(const float *host_params)
    {
        P.alloc(kParams);
        G.alloc(kParams);
        M.alloc(kParams);
        V.alloc(kParams);
        Wb.alloc((size_t)kLayers * 128 * 64);
        WTb.alloc((size_t)kLayers * 128 * 64);
        SENK_CUDA(cudaMemcpy(P.p, host_params, sizeof(float) * kParams, cudaMemcpyHostToDevice));
        SENK_CUDA(cudaMemset(M.p, 0, M.bytes()));
        SENK_CUDA(cudaMemset(V.p, 0, V.bytes()));
        status.alloc(1);
        SENK_CUDA(cudaMemset(status.p, 0, sizeof(int)));
        gnorm.alloc(1);
        rms.alloc(2);
        red.alloc(sm_count() * 8);  // two partials per CTA for k_step_alpha
        acc.alloc(2);
        ticket.alloc(1);
        SENK_CUDA(cudaMemset(ticket.p, 0, sizeof(unsigned)));
        refresh_weights(nullptr);
        SENK_CUDA(cudaDeviceSynchronize());
    }

    void refresh_weights(cudaStream_t s)
    {
        k_weights_bf16<<<ceil_div(kLayers * 128 * 64, kThreads), kThreads, 0, s>>>(P.p, Wb.p, WTb.p);
        SENK_LAUNCH_CHECK();
    }

    // Graph data of a CSR matrix (host copy): W, W^T, diagonal and |row| sums.
    void bind_matrix(const double *val, const int *cind, const int *rptr, int N, cudaStream_t s)
    {
        std::vector<int> r(N + 1, 0), c, tr_(N + 1, 0), tc_;
        std::vector<float> w, tw, hd(N), hs(N);
        double dsum = 0;
        for (int i = 0; i < N; i++) {
            double diag = 0, off = 0;
            for (int p = rptr[i]; p < rptr[i + 1]; p++) {
                if (cind[p] == i) diag = val[p];
                else off += std::fabs(val[p]);
            }
            hd[i] = (float)diag;
            hs[i] = (float)(off + std::fabs(diag));
            dsum += diag;
            for (int p = rptr[i]; p < rptr[i + 1]; p++) {
                if (cind[p] == i) continue;
                c.push_back(cind[p]);
                w.push_back(off > 0 ? (float)(std::fabs(val[p]) / off) : 0.f);
                tr_[cind[p] + 1]++;
            }
            r[i + 1] = (int)c.size();
        }
        d = (float)(dsum / N);
        SENK_REQUIRE(d > 0, "the learned preconditioner needs a positive mean diagonal");
        for (int i = 0; i < N; i++) {
            hd[i] /= d;
            hs[i] /= d;
        }
        for (int i = 0; i < N; i++) tr_[i + 1] += tr_[i];
        tc_.resize(c.size());
        tw.resize(c.size());
        std::vector<int> fill(tr_.begin(), tr_.end() - 1);
        for (int i = 0; i < N; i++)
            for (int p = r[i]; p < r[i + 1]; p++) {
                const int q = fill[c[p]]++;
                tc_[q] = i;
                tw[q] = w[p];
            }
        // A and A^T with FP32 values
        std::vector<int> atr_(N + 1, 0), atc_(rptr[N]), fill2;
        std::vector<float> av_(rptr[N]), atv_(rptr[N]);
        for (int p = 0; p < rptr[N]; p++) {
            av_[p] = (float)val[p];
            atr_[cind[p] + 1]++;
        }
        for (int i = 0; i < N; i++) atr_[i + 1] += atr_[i];
        fill2.assign(atr_.begin(), atr_.end() - 1);
        for (int i = 0; i < N; i++)
            for (int p = rptr[i]; p < rptr[i + 1]; p++) {
                const int q = fill2[cind[p]]++;
                atc_[q] = i;
                atv_[q] = av_[p];
            }
        auto put = [s](auto &buf, const auto &h) {
            buf.alloc(h.size());
            buf.upload(h.data(), h.size(), s);
        };
        put(ar, std::vector<int>(rptr, rptr + N + 1));
        put(ac, std::vector<int>(cind, cind + rptr[N]));
        put(av, av_);
        put(atr, atr_);
        put(atc, atc_);
        put(atv, atv_);
        put(wr, r);
        put(wc, c);
        put(wv, w);
        put(tr, tr_);
        put(tcol, tc_);
        put(tv, tw);
        put(fd, hd);
        put(fs, hs);
        if (n != N) {
            n = N;
            for (int l = 0; l < kLayers; l++) {
                X[l].alloc((size_t)N * 128);
                Z[l].alloc((size_t)N * 64);
            }
            for (int l = 0; l <= kLayers; l++) H[l].alloc((size_t)N * 64);
            dZ.alloc((size_t)N * 64);
            dH.alloc((size_t)N * 64);
            dH2.alloc((size_t)N * 64);
            dM.alloc((size_t)N * 64);
            t.alloc(N);
            cbuf.alloc(N);
            dcb.alloc(N);
            ebuf.alloc(N);
            ailu.alloc(N);
            cstep.alloc(N);
            acstep.alloc(N);
            alpha.alloc(1);
        }
        SENK_CUDA(cudaStreamSynchronize(s));
    }

    template <typename T>
    void forward(const T *r, cudaStream_t s, bool keep_z)
    {
        const int rg = std::min(ceil_div(n, kThreads), sm_count() * 4);
        k_rms<T><<<rg, kThreads, 0, s>>>(r, n, red.p, ticket.p, rms.p);
        k_encode<T><<<ceil_div(n * kHid, kThreads), kThreads, 0, s>>>(fd.p, fs.p, r, rms.p, P.p, H[0].p, X[0].p, n);
        const int tiles = ceil_div(n, 128);
        for (int l = 0; l < kLayers; l++) {
            k_aggregate<<<ceil_div(n * 8, kThreads), kThreads, 0, s>>>(wr.p, wc.p, wv.p, X[l].p, n);
            TcArgs a;
            a.bias = P.p + kOffLayer + l * kLayerSize + 2 * kHid * kHid;
            a.hin = H[l].p;
            a.hout = H[l + 1].p;
            a.xout = l + 1 < kLayers ? X[l + 1].p : nullptr;  // the last layer's bf16 copy is not read
            a.xld = 128;
            a.zout = keep_z ? Z[l].p : nullptr;
            k_tc_gemm<128, 64, kTcLayerFwd><<<tiles, 128, kSmemFwd, s>>>(
                X[l].p, 128, WTb.p + (size_t)l * 64 * 128, (int)n, a, status.p);
        }
        SENK_LAUNCH_CHECK();
    }

    // out += (rms / d) * net(r): out already holds ILU(r)
    template <typename T>
    void apply(const T *r, T *out, cudaStream_t s)
    {
        forward<T>(r, s, false);
        k_decode_apply<T><<<ceil_div(n * 32, kThreads), kThreads, 0, s>>>(H[kLayers].p, P.p, rms.p, 1.f / d, out, n);
        SENK_LAUNCH_CHECK();
    }

    // The GCR hook: out holds u = ILU(r) on entry; with step_mode 1,
    // out = u + alpha c where c = (rms / d) net(r) and alpha minimises
    // |r - A(u + alpha c)| (two SpMVs with the system's A and one reduction, no
    // host synchronisation, so it stays inside a captured graph).
    void apply_step(const SpmvOp<double> &A, const double *r, double *out, cudaStream_t s)
    {
        if (step_mode == 0) {
            apply<double>(r, out, s);
            return;
        }
        forward<double>(r, s, false);
        SENK_CUDA(cudaMemsetAsync(cstep.p, 0, sizeof(double) * n, s));
        k_decode_apply<double><<<ceil_div(n * 32, kThreads), kThreads, 0, s>>>(H[kLayers].p, P.p, rms.p, 1.f / d,
                                                                               cstep.p, n);
        SENK_LAUNCH_CHECK();
        A.apply(out, ailu.p, s, nullptr);
        A.apply(cstep.p, acstep.p, s, nullptr);
        const int rg = std::min(ceil_div(n, kThreads), sm_count() * 4);
        k_step_alpha<<<rg, kThreads, 0, s>>>(r, ailu.p, acstep.p, n, red.p, ticket.p, alpha.p);
        k_add_step<<<rg, kThreads, 0, s>>>(out, cstep.p, alpha.p, n);
        SENK_LAUNCH_CHECK();
    }

    // Loss and gradient of one residual/error pair into G (zeroed first).
    //  loss_mode 0 (error space):    t = (e - ILU(r)) d / rms, loss = |c - t|^2 / |t|^2
    //  loss_mode 1 (residual space): q = (r - A ILU(r)) / rms,
    //                                loss = |A c / d - q|^2 / |q|^2
    // `ailu_dev` holds A ILU(r) (mode 1).
    template <typename T>
    void loss_grad(const T *r, const T *ilu, const T *e, const T *ailu_dev, cudaStream_t s)
    {
        SENK_CUDA(cudaMemsetAsync(G.p, 0, G.bytes(), s));
        SENK_CUDA(cudaMemsetAsync(acc.p, 0, acc.bytes(), s));
        forward<T>(r, s, true);
        const int rg = std::min(ceil_div(n, kThreads), sm_count() * 4);
        k_decode_c<<<ceil_div(n * 32, kThreads), kThreads, 0, s>>>(H[kLayers].p, P.p, cbuf.p, n);
        if (loss_mode == 0) {
            k_target<T><<<rg, kThreads, 0, s>>>(e, ilu, rms.p, d, t.p, n, red.p, ticket.p, acc.p);
            k_loss_error<<<rg, kThreads, 0, s>>>(cbuf.p, t.p, dcb.p, acc.p, n);
        } else {
            k_resid_target<T><<<rg, kThreads, 0, s>>>(r, ailu_dev, rms.p, t.p, acc.p, n);
            k_spmv_loss<<<rg, kThreads, 0, s>>>(ar.p, ac.p, av.p, cbuf.p, ebuf.p, n, 1.f / d, t.p, acc.p);
            k_spmv_grad<<<rg, kThreads, 0, s>>>(atr.p, atc.p, atv.p, ebuf.p, dcb.p, n, 1.f / d, acc.p);
        }
        k_decode_back<<<sm_count() * 4, kThreads, 0, s>>>(H[kLayers].p, P.p, dcb.p, dH.p, G.p, n);
        float *dh = dH.p, *dh2 = dH2.p;
        const int tiles = ceil_div(n, 128);
        for (int l = kLayers - 1; l >= 0; l--) {
            float *gl = G.p + kOffLayer + l * kLayerSize;
            k_relu_back<<<sm_count() * 8, kThreads, 0, s>>>(dh, Z[l].p, dZ.p, gl + 2 * kHid * kHid, n);
            k_tc_gemm_tn<64><<<sm_count() * 2, 128, kSmemTn, s>>>(X[l].p, 128, dZ.p, (int)n, gl, status.p);
            TcArgs a;
            a.hin = dh;
            a.hout = dh2;
            a.dm = dM.p;
            k_tc_gemm<64, 128, kTcDx><<<tiles, 128, kSmemDx, s>>>(
                dZ.p, 64, Wb.p + (size_t)l * 128 * 64, (int)n, a, status.p);
            k_aggregate_back<<<ceil_div(n * 8, kThreads), kThreads, 0, s>>>(tr.p, tcol.p, tv.p, dM.p, dh2, n);
            std::swap(dh, dh2);
        }
        k_encode_back<T><<<sm_count() * 8, kThreads, 0, s>>>(fd.p, fs.p, r, rms.p, P.p, dh, G.p, n);
        SENK_LAUNCH_CHECK();
    }

    void adam(float lr, cudaStream_t s)
    {
        step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f / (1.f - std::pow(b1, (float)step)), c2 = 1.f / (1.f - std::pow(b2, (float)step));
        k_grad_norm2<<<1, 1024, 0, s>>>(G.p, kParams, gnorm.p);
        k_adam<<<ceil_div(kParams, kThreads), kThreads, 0, s>>>(P.p, G.p, M.p, V.p, kParams, lr, b1, b2, 1e-8f, c1, c2,
                                                                gnorm.p, clip);
        refresh_weights(s);
    }

    void check_status(cudaStream_t s)
    {
        int h = 0;
        SENK_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        SENK_CUDA(cudaStreamSynchronize(s));
        if (h) throw CudaError{cudaErrorLaunchTimeout, "tensor-core MMA completion wait ran out", __FILE__, __LINE__};
    }
};

static void set_smem_limits()
{
    static bool done = false;
    if (done) return;
    SENK_CUDA(cudaFuncSetAttribute(k_tc_gemm<128, 64, kTcLayerFwd>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   kSmemFwd));
    SENK_CUDA(cudaFuncSetAttribute(k_tc_gemm<128, 64, kTcPlain>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   kSmemFwd));
    SENK_CUDA(cudaFuncSetAttribute(k_tc_gemm<64, 128, kTcDx>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemDx));
    SENK_CUDA(cudaFuncSetAttribute(k_tc_gemm<64, 128, kTcPlain>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   kSmemDx));
    SENK_CUDA(cudaFuncSetAttribute(k_tc_gemm_tn<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTn));
    done = true;
}

// The learned correction hook of System<double>::precondition.
void learned_apply(void *net, const void *sys, const double *v, double *out, cudaStream_t s)
{
    Mpnn *m = static_cast<Mpnn *>(net);
    SENK_REQUIRE(m->bound == sys, "the network is bound to another system");
    m->apply_step(static_cast<const System<double> *>(sys)->A, v, out, s);
}

}  // namespace senkgpu

using namespace senkgpu;

struct senk_mpnn {
    Mpnn net;
};

extern "C" {

int senk_mpnn_num_params(void) { return kParams; }

int senk_mpnn_create(senk_mpnn **out, const float *params, int nparams)
{
    return guarded("senk_mpnn_create", [&] {
        SENK_REQUIRE(out && params && nparams == kParams, "params must hold senk_mpnn_num_params() floats");
        set_smem_limits();
        auto h = std::make_unique<senk_mpnn>();
        h->net.init(params);
        *out = h.release();
        return (int)kOk;
    });
}

int senk_mpnn_destroy(senk_mpnn *net)
{
    return guarded("senk_mpnn_destroy", [&] {
        delete net;
        return (int)kOk;
    });
}

int senk_mpnn_get_params(senk_mpnn *net, float *host, int nparams)
{
    return guarded("senk_mpnn_get_params", [&] {
        SENK_REQUIRE(net && host && nparams == kParams, "bad arguments");
        SENK_CUDA(cudaDeviceSynchronize());
        SENK_CUDA(cudaMemcpy(host, net->net.P.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
        return (int)kOk;
    });
}

int senk_mpnn_set_params(senk_mpnn *net, const float *host, int nparams)
{
    return guarded("senk_mpnn_set_params", [&] {
        SENK_REQUIRE(net && host && nparams == kParams, "bad arguments");
        SENK_CUDA(cudaDeviceSynchronize());
        SENK_CUDA(cudaMemcpy(net->net.P.p, host, sizeof(float) * kParams, cudaMemcpyHostToDevice));
        net->net.refresh_weights(nullptr);
        SENK_CUDA(cudaDeviceSynchronize());
        return (int)kOk;
    });
}

// Training objective: 0 = error space, 1 = residual space (default).
int senk_mpnn_set_loss(senk_mpnn *net, int mode)
{
    return guarded("senk_mpnn_set_loss", [&] {
        SENK_REQUIRE(net && (mode == 0 || mode == 1), "mode must be 0 or 1");
        net->net.loss_mode = mode;
        return (int)kOk;
    });
}

// Global gradient-norm clip of the Adam steps (default 1; <= 0 turns it off).
int senk_mpnn_set_clip(senk_mpnn *net, float clip)
{
    return guarded("senk_mpnn_set_clip", [&] {
        SENK_REQUIRE(net, "null network");
        net->net.clip = clip;
        return (int)kOk;
    });
}

// Step of the correction inside the GCR: 0 = K(r) = ILU(r) + c (default),
// 1 = K(r) = ILU(r) + alpha c with the least-squares alpha.
int senk_mpnn_set_step(senk_mpnn *net, int mode)
{
    return guarded("senk_mpnn_set_step", [&] {
        SENK_REQUIRE(net && (mode == 0 || mode == 1), "mode must be 0 or 1");
        net->net.step_mode = mode;
        return (int)kOk;
    });
}

int senk_mpnn_bind(senk_mpnn *net, senk_system *sys)
{
    return guarded("senk_mpnn_bind", [&] {
        SENK_REQUIRE(net && sys && sys->d, "needs an FP64 system");
        System<double> &S = *sys->d;
        SENK_REQUIRE(S.has_pc(), "the learned correction needs the system's ILU preconditioner");
        SENK_REQUIRE(S.A.has_csr, "the system keeps no CSR copy of A");
        const int N = S.n, nnz = S.A.nnz;
        std::vector<double> v(nnz);
        std::vector<int> c(nnz), r(N + 1);
        SENK_CUDA(cudaStreamSynchronize(S.stream));
        SENK_CUDA(cudaMemcpy(v.data(), S.A.val.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
        SENK_CUDA(cudaMemcpy(c.data(), S.A.cind.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
        SENK_CUDA(cudaMemcpy(r.data(), S.A.rptr.p, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost));
        net->net.bind_matrix(v.data(), c.data(), r.data(), N, S.stream);
        net->net.bound = &S;
        return (int)kOk;
    });
}

// loss of one residual/error pair (device vectors of the bound system); the
// gradient goes to grad (host, may be NULL) and stays on the device for a step.
int senk_mpnn_loss_grad(senk_mpnn *net, senk_system *sys, const double *r, const double *e, double *loss,
                        float *grad)
{
    return guarded("senk_mpnn_loss_grad", [&] {
        SENK_REQUIRE(net && sys && sys->d && r && e, "null argument");
        System<double> &S = *sys->d;
        Mpnn &m = net->net;
        SENK_REQUIRE(m.bound == &S, "bind the network to this system first");
        S.precondition_base(r, S.t.p, nullptr);  // ILU(r) alone
        if (m.loss_mode == 1) S.A.apply(S.t.p, m.ailu.p, S.stream, nullptr);
        m.loss_grad<double>(r, S.t.p, e, m.ailu.p, S.stream);
        double a[2];
        SENK_CUDA(cudaMemcpyAsync(a, m.acc.p, sizeof(a), cudaMemcpyDeviceToHost, S.stream));
        if (grad) SENK_CUDA(cudaMemcpyAsync(grad, m.G.p, sizeof(float) * kParams, cudaMemcpyDeviceToHost, S.stream));
        m.check_status(S.stream);
        if (loss) *loss = a[0] > 0 ? a[1] / a[0] : 0.0;
        return (int)kOk;
    });
}

int senk_mpnn_train_step(senk_mpnn *net, senk_system *sys, const double *r, const double *e, float lr, double *loss)
{
    return guarded("senk_mpnn_train_step", [&] {
        const int rc = senk_mpnn_loss_grad(net, sys, r, e, loss, nullptr);
        if (rc != kOk) return rc;
        net->net.adam(lr, sys->d->stream);
        return (int)kOk;
    });
}

// out = K(r) = ILU(r) + correction, device vectors of the bound system
int senk_mpnn_apply(senk_mpnn *net, senk_system *sys, const double *r, double *out)
{
    return guarded("senk_mpnn_apply", [&] {
        SENK_REQUIRE(net && sys && sys->d && r && out, "null argument");
        System<double> &S = *sys->d;
        SENK_REQUIRE(net->net.bound == &S, "bind the network to this system first");
        S.precondition_base(r, out, nullptr);
        net->net.apply_step(S.A, r, out, S.stream);
        net->net.check_status(S.stream);
        return (int)kOk;
    });
}

// Attach a bound network to the system's GCR as K(r) = ILU(r) + correction
// (net NULL: detach). stall: the GCR falls back to plain ILU for the rest of a
// solve once a restart cycle reduces the residual by less than this factor.
int senk_system_set_learned(senk_system *sys, senk_mpnn *net, double stall)
{
    return guarded("senk_system_set_learned", [&] {
        SENK_REQUIRE(sys && sys->d, "needs an FP64 system");
        SENK_REQUIRE(stall > 0 && stall <= 1, "stall must be in (0, 1]");
        if (net) SENK_REQUIRE(net->net.bound == sys->d.get(), "bind the network to this system first");
        sys->d->learned = net ? &net->net : nullptr;
        sys->d->learned_stall = stall;
        return (int)kOk;
    });
}

// Restart cycle at which the last GCR solve fell back to plain ILU (-1: never).
int senk_system_learned_fallback(senk_system *sys) { return sys && sys->d ? sys->d->learned_fallback : -1; }

// C (n x NO, fp32) = A (n x K, bf16) * Bt (NO x K, bf16)^T, for tests of the
// tensor-core path. K in {64, 128}, NO in {64, 128} (K = 128 needs NO = 64).
int senk_dev_gemm_bf16(const void *A, const void *Bt, float *C, int n, int K, int NO, void *stream)
{
    return guarded("senk_dev_gemm_bf16", [&] {
        SENK_REQUIRE(A && Bt && C && n > 0, "null argument");
        SENK_REQUIRE(((uintptr_t)A & 15) == 0 && ((uintptr_t)Bt & 15) == 0 && ((uintptr_t)C & 15) == 0,
                     "operands and result must be 16-byte aligned");
        set_smem_limits();
        static DevBuf<int> st;
        if (!st.p) {
            st.alloc(1);
            SENK_CUDA(cudaMemset(st.p, 0, sizeof(int)));
        }
        cudaStream_t s = (cudaStream_t)stream;
        TcArgs a;
        a.c = C;
        const int tiles = ceil_div(n, 128);
        const bf16 *a16 = (const bf16 *)A, *b16 = (const bf16 *)Bt;
        if (K == 128 && NO == 64)
            k_tc_gemm<128, 64, kTcPlain><<<tiles, 128, kSmemFwd, s>>>(a16, 128, b16, n, a, st.p);
        else if (K == 64 && NO == 128)
            k_tc_gemm<64, 128, kTcPlain><<<tiles, 128, kSmemDx, s>>>(a16, 64, b16, n, a, st.p);
        else
            throw ArgError("supported shapes: K=128 NO=64, K=64 NO=128");
        SENK_LAUNCH_CHECK();
        int h = 0;
        SENK_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        SENK_CUDA(cudaStreamSynchronize(s));
        SENK_REQUIRE(h == 0, "tensor-core MMA completion wait ran out");
        return (int)kOk;
    });
}

// out (128 x 64, fp32) = X^T dZ, X n x 128 and dZ n x 64 (bf16): the weight
// gradient product, for tests.
int senk_dev_gemm_tn_bf16(const void *X, const void *dZ, float *out, int n, void *stream)
{
    return guarded("senk_dev_gemm_tn_bf16", [&] {
        SENK_REQUIRE(X && dZ && out && n > 0, "null argument");
        SENK_REQUIRE(((uintptr_t)X & 15) == 0 && ((uintptr_t)dZ & 15) == 0, "operands must be 16-byte aligned");
        set_smem_limits();
        static DevBuf<int> st;
        if (!st.p) {
            st.alloc(1);
            SENK_CUDA(cudaMemset(st.p, 0, sizeof(int)));
        }
        cudaStream_t s = (cudaStream_t)stream;
        SENK_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * 128 * 64, s));
        k_tc_gemm_tn<64><<<std::min(ceil_div(n, 64), sm_count() * 2), 128, kSmemTn, s>>>((const bf16 *)X, 128,
                                                                                (const bf16 *)dZ, n, out, st.p);
        SENK_LAUNCH_CHECK();
        int h = 0;
        SENK_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        SENK_CUDA(cudaStreamSynchronize(s));
        SENK_REQUIRE(h == 0, "tensor-core MMA completion wait ran out");
        return (int)kOk;
    });
}

}  // extern "C"
