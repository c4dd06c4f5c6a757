// sm_103a kernels of the SenK Krylov path: SpMV, blas1 reductions, the
// Arnoldi Gram-Schmidt step and the colour-by-colour ILU sweeps.
//
// Conventions:
//  * `gate`: optional device flag; a kernel whose gate is non-zero returns at once.
//    A restart cycle is captured once in a CUDA graph; after convergence the
//    remaining inner iterations of that cycle see the flag and do nothing.
//  * Reductions write one partial per CTA and the last CTA to arrive sums the
//    partials in a fixed order, so results do not depend on scheduling.
#pragma once

#include "common.cuh"
#include "wf_layout.hpp"

namespace senkgpu {

template <typename T> struct Acc { using type = T; };  // accumulation type

// Per-solve device scalars of a Krylov engine.
struct KrylovState {
    double nrm_b;      // ||b|| as passed by the caller
    double eps;        // relative tolerance
    double scale;      // 1/h_{j+1,j} (GMRES) or 1/||r|| of the last normalisation
    double res;        // |e_{j+1}|/nrm_b at convergence
    int done;          // 1 once converged (gates the rest of the cycle)
    int jconv;         // number of basis vectors of the converged cycle
    int breakdown;     // a pivot scalar was zero or not finite
    int count;         // BiCGStab: iterations completed
    int maxit;         // BiCGStab: iteration limit (done = 2 when reached)
    int pad;
    double s[8];       // scratch scalars (BiCGStab/GCR coefficients)
};

__device__ __forceinline__ bool gated(const int *gate) { return gate != nullptr && *(volatile const int *)gate != 0; }

// ------------------------------------------------------------------- SpMV

// CSR SpMV, G lanes per row (G a power of two <= 32). MODE 0: y = A x;
// MODE 1: y = b - A x. NORM: also reduce ||y||^2 and, in the last CTA, store
// sqrt into *norm_out and its inverse into *inv_out (used for r0 / ||r0||).
template <typename MT, typename XT, int G, int MODE, bool NORM>
__global__ void __launch_bounds__(kThreads)
k_spmv_csr(const MT *__restrict__ val, const int *__restrict__ cind, const int *__restrict__ rptr,
           const XT *__restrict__ x, const XT *__restrict__ b, XT *__restrict__ y, int n,
           double *part, unsigned *ticket, double *norm_out, double *inv_out, const int *gate)
{
    if (gated(gate)) return;
    using A = typename Acc<XT>::type;
    constexpr int RPW = 32 / G;  // rows per warp per step
    const int lane = threadIdx.x & 31, sub = lane / G, l = lane % G;
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    double nacc = 0;
    for (long long base = warp * RPW; base < n; base += nwarps * RPW) {
        const long long row = base + sub;
        A sum = 0;
        if (row < n) {
            const int s = __ldg(rptr + row), e = __ldg(rptr + row + 1);
            for (int j = s + l; j < e; j += G) sum += (A)ld_stream(val + j) * (A)__ldg(x + ld_stream(cind + j));
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (row < n && l == 0) {
            XT v = MODE == 1 ? (XT)((A)b[row] - sum) : (XT)sum;
            y[row] = v;
            if (NORM) nacc += (double)v * (double)v;
        }
    }
    if (NORM) {
        __shared__ double sh[32];
        double t = block_sum(nacc, sh);
        if (threadIdx.x == 0) part[blockIdx.x] = t;
        if (last_cta_arrives(ticket, gridDim.x)) {
            __shared__ double shp[32];
            const double s = cta_sum_partials(part, gridDim.x, shp);
            if (threadIdx.x == 0) {
                double r = sqrt(s);
                *norm_out = r;
                if (inv_out) *inv_out = 1.0 / r;
            }
        }
    }
}

// Row sum of one SELL-32 row (lane r of the slice at element offset o, w
// columns): sum over k of val * x[col] in column order. The entries are taken
// eight at a time with every load of a batch issued before the first product
// (values and columns, then the x gathers), so a stencil row of seven entries
// costs two dependent memory latencies instead of one per entry.
template <typename MT, typename XT, typename A>
__device__ __forceinline__ A sell_row_sum(const MT *__restrict__ val, const int *__restrict__ col,
                                          const XT *__restrict__ x, int o, int w, int r)
{
    constexpr int B = 8;
    A sum = 0;
    for (int k = 0; k < w; k += B) {
        MT v[B];
        int c[B];
        XT xv[B];
#pragma unroll
        for (int u = 0; u < B; u++) {
            const int i0 = o + (k + u) * 32 + r;
            v[u] = k + u < w ? ld_stream(val + i0) : MT(0);
            c[u] = k + u < w ? ld_stream(col + i0) : 0;
        }
#pragma unroll
        for (int u = 0; u < B; u++) xv[u] = k + u < w ? __ldg(x + c[u]) : XT(0);
#pragma unroll
        for (int u = 0; u < B; u++)
            if (k + u < w) sum += (A)v[u] * (A)xv[u];
    }
    return sum;
}

// SELL-C SpMV, one thread per row, C = 32 rows per slice, slice-major columns:
// element (slice s, column k, lane r) at off[s] + k*32 + r. `perm` (optional)
// maps slice position -> row for sigma-sorted layouts.
template <typename MT, typename XT, int MODE>
__global__ void __launch_bounds__(kThreads)
k_spmv_sell32(const MT *__restrict__ val, const int *__restrict__ col, const int *__restrict__ off,
              const int *__restrict__ perm, const XT *__restrict__ x, const XT *__restrict__ b,
              XT *__restrict__ y, int n, const int *gate)
{
    if (gated(gate)) return;
    using A = typename Acc<XT>::type;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ((long long)n + 31) / 32 * 32) return;
    const int s = (int)(p >> 5), r = (int)(p & 31);
    const int o = __ldg(off + s), w = (__ldg(off + s + 1) - o) >> 5;
    const A sum = sell_row_sum<MT, XT, A>(val, col, x, o, w, r);
    const long long row = perm ? (long long)__ldg(perm + p) : p;
    if (row < n && row >= 0) y[row] = MODE == 1 ? (XT)((A)b[row] - sum) : (XT)sum;
}

// r = b - A x on the SELL-32 copy, with ||r||^2 reduced to the last CTA, which
// stores ||r|| in *norm_out and 1/||r|| in *inv_out.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_residual_sell32(const T *__restrict__ val, const int *__restrict__ col, const int *__restrict__ off,
                  const int *__restrict__ perm, const T *__restrict__ x, const T *__restrict__ b,
                  T *__restrict__ r, int n, double *part, unsigned *ticket, double *norm_out, double *inv_out)
{
    using A = typename Acc<T>::type;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double nacc = 0;
    if (p < n) {  // positions below n hold rows (sigma windows lie within the rows)
        const int s = (int)(p >> 5), lane = (int)(p & 31);
        const int o = __ldg(off + s), w = (__ldg(off + s + 1) - o) >> 5;
        const A sum = sell_row_sum<T, T, A>(val, col, x, o, w, lane);
        const long long row = perm ? (long long)__ldg(perm + p) : p;
        const T v = (T)((A)b[row] - sum);
        r[row] = v;
        nacc = (double)v * (double)v;
    }
    __shared__ double sh[32];
    const double t = block_sum(nacc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    if (last_cta_arrives(ticket, gridDim.x)) {
        const double s = cta_sum_partials(part, gridDim.x, sh);
        if (threadIdx.x == 0) {
            const double nr = sqrt(s);
            *norm_out = nr;
            if (inv_out) *inv_out = 1.0 / nr;
        }
    }
}

// Iterative refinement glue: r32 = (float)(r * (*inv)); x += (*norm) * d32.
static __global__ void __launch_bounds__(kThreads)
k_ir_demote(const double *__restrict__ r, const double *inv, float *__restrict__ r32, long long n)
{
    const double s = *inv;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        r32[i] = (float)(r[i] * s);
}

static __global__ void __launch_bounds__(kThreads)
k_ir_correct(double *__restrict__ x, const double *norm, const float *__restrict__ d32, long long n)
{
    const double s = *norm;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] += s * (double)d32[i];
}

// CSR SpMV with a separately stored diagonal (reference SpmvCsr with diag).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_spmv_csr_diag(const T *__restrict__ val, const int *__restrict__ cind, const int *__restrict__ rptr,
                const T *__restrict__ diag, const T *__restrict__ x, T *__restrict__ y, int n)
{
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    T sum = x[row] * diag[row];
    for (int j = rptr[row]; j < rptr[row + 1]; j++) sum += val[j] * __ldg(x + cind[j]);
    y[row] = sum;
}

// BCSR SpMV, one thread per block row; BNL x BNW blocks stored column-major.
template <typename MT, typename XT, int BNL, int BNW, int MODE>
__global__ void __launch_bounds__(kThreads)
k_spmv_bcsr(const MT *__restrict__ bval, const int *__restrict__ bcind, const int *__restrict__ brptr,
            const XT *__restrict__ x, const XT *__restrict__ b, XT *__restrict__ y, int nb, const int *gate)
{
    if (gated(gate)) return;
    using A = typename Acc<XT>::type;
    const long long br = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (br >= nb) return;
    A acc[BNL];
#pragma unroll
    for (int r = 0; r < BNL; r++) acc[r] = 0;
    for (int blk = __ldg(brptr + br); blk < __ldg(brptr + br + 1); blk++) {
        const MT *bv = bval + (long long)blk * (BNL * BNW);
        const int xc = __ldg(bcind + blk) * BNW;
#pragma unroll
        for (int c = 0; c < BNW; c++) {
            const A xv = (A)__ldg(x + xc + c);
#pragma unroll
            for (int r = 0; r < BNL; r++) acc[r] += (A)ld_stream(bv + c * BNL + r) * xv;
        }
    }
#pragma unroll
    for (int r = 0; r < BNL; r++) {
        const long long i = br * BNL + r;
        y[i] = MODE == 1 ? (XT)((A)b[i] - acc[r]) : (XT)acc[r];
    }
}

// Reference SELL-c layout SpMV (include/senk_sparse.hpp:103-121): slice s holds
// wid[s+1]-wid[s] columns of `len` rows, column-major, rows = len except a short
// last slice (stride = its row count, as Csr2Sell lays it out).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_spmv_sell_ref(const T *__restrict__ val, const int *__restrict__ cind, const int *__restrict__ wid,
                int len, const T *__restrict__ x, T *__restrict__ y, int n)
{
    const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    const int s = (int)(row / len), j = (int)(row % len);
    const int nslice = (n + len - 1) / len;
    const int rows = (s == nslice - 1 && n % len) ? n % len : len;
    const long long start = (long long)wid[s] * len;
    T sum = 0;
    for (int c = 0; c < wid[s + 1] - wid[s]; c++) {
        const long long i = start + (long long)c * rows + j;
        sum += val[i] * __ldg(x + cind[i]);
    }
    y[row] = sum;
}

// ----------------------------------------------------------------- blas1

// Element-wise ops. OP: 0 y=a*x+y, 1 y=a*x+b*y, 2 z=a*x+y, 3 x=a*x, 4 y=x,
// 5 y*=x, 6 y/=x.  Scalars may come from device memory (a_dev/b_dev, optional).
template <typename T, int OP>
__global__ void __launch_bounds__(kThreads)
k_elementwise(T a, const double *a_dev, double a_dev_mul, T b, const T *__restrict__ x,
              T *__restrict__ y, T *__restrict__ z, long long n, const int *gate)
{
    if (gated(gate)) return;
    if (a_dev) a = (T)(a_dev_mul * *a_dev);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (OP == 0) y[i] += a * x[i];
        else if (OP == 1) y[i] = a * x[i] + b * y[i];
        else if (OP == 2) z[i] = a * x[i] + y[i];
        else if (OP == 3) y[i] *= a;
        else if (OP == 4) y[i] = x[i];
        else if (OP == 5) y[i] *= x[i];
        else y[i] /= x[i];
    }
}

// Dot products of w against nv vectors V_k (V_k = V + k*ldv), computed in
// chunks of 8 columns per CTA column (blockIdx.y). The last CTA writes
// coef[k] = sum and, if hcol is given, hcol[k] = sum (ACCUM=false) or
// hcol[k] += sum (ACCUM=true).
template <typename XT, bool ACCUM>
__global__ void __launch_bounds__(kThreads)
k_multidot(const XT *__restrict__ V, long long ldv, int nv, const XT *__restrict__ w, long long n,
           double *part, unsigned *ticket, double *coef, double *hcol, const int *gate)
{
    if (gated(gate)) return;
    constexpr int CH = 8;
    const int c0 = blockIdx.y * CH;
    const int nc = min(CH, nv - c0);
    // Per-thread partial sums in the vector type (FP32 vectors stay on the FP32
    // pipe), combined across threads and CTAs in FP64; four independent
    // elements per step keep enough loads in flight.
    using A = typename Acc<XT>::type;
    A acc[CH];
#pragma unroll
    for (int q = 0; q < CH; q++) acc[q] = 0;
    const long long S = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * S < n; i += 4 * S) {
        const A w0 = (A)w[i], w1 = (A)w[i + S], w2 = (A)w[i + 2 * S], w3 = (A)w[i + 3 * S];
#pragma unroll
        for (int q = 0; q < CH; q++) {
            if (q < nc) {
                const XT *vq = V + (long long)(c0 + q) * ldv + i;
                const A a0 = (A)ld_stream(vq), a1 = (A)ld_stream(vq + S), a2 = (A)ld_stream(vq + 2 * S),
                        a3 = (A)ld_stream(vq + 3 * S);
                acc[q] += a0 * w0;
                acc[q] += a1 * w1;
                acc[q] += a2 * w2;
                acc[q] += a3 * w3;
            }
        }
    }
    for (; i < n; i += S) {
        const A wi = (A)w[i];
#pragma unroll
        for (int q = 0; q < CH; q++)
            if (q < nc) acc[q] += (A)ld_stream(V + (long long)(c0 + q) * ldv + i) * wi;
    }
    // columns this CTA holds only (nc is the same in all its warps)
    __shared__ double sh[CH][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < CH; q++) {
        if (q < nc) {
            const double v = warp_sum((double)acc[q]);
            if (lane == 0) sh[q][wid] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < CH * 32 && (int)(threadIdx.x >> 5) < nc) {
        const int q = threadIdx.x >> 5;
        double v = lane < (int)(blockDim.x >> 5) ? sh[q][lane] : 0.0;
        v = warp_sum(v);
        if (lane == 0) part[(long long)(c0 + q) * gridDim.x + blockIdx.x] = v;
    }
    const unsigned total = gridDim.x * gridDim.y;
    if (last_cta_arrives(ticket, total)) {
        __shared__ double shp[32];
        cta_sum_columns(part, gridDim.x, nv, shp, [&](int k, double s) {
            coef[k] = s;
            if (hcol) hcol[k] = ACCUM ? hcol[k] + s : s;
        });
    }
}

// 16-byte vectors of the Krylov kernels: float4 / double2.
template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec16<double> { using type = double2; static constexpr int n = 2; };

__device__ __forceinline__ float vdot(const float4 &a, const float4 &b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ double vdot(const double2 &a, const double2 &b) { return a.x * b.x + a.y * b.y; }
__device__ __forceinline__ void vaxpy(float4 &y, float a, const float4 &x) { y.x -= a * x.x; y.y -= a * x.y; y.z -= a * x.z; y.w -= a * x.w; }
__device__ __forceinline__ void vaxpy(double2 &y, double a, const double2 &x) { y.x -= a * x.x; y.y -= a * x.y; }

// k_multidot with 16-byte loads: n and ldv are multiples of the vector width
// and V, w are 16-byte aligned (the launcher checks). Each thread keeps CH
// column sums over two vectors per step; the combination across threads and
// CTAs is k_multidot's.
template <typename XT, bool ACCUM>
__global__ void __launch_bounds__(kThreads)
k_multidot_v(const XT *__restrict__ V, long long ldv, int nv, const XT *__restrict__ w, long long n,
             double *part, unsigned *ticket, double *coef, double *hcol, const int *gate)
{
    if (gated(gate)) return;
    using VT = typename Vec16<XT>::type;
    constexpr int W = Vec16<XT>::n;
    constexpr int CH = 8;
    const int c0 = blockIdx.y * CH;
    const int nc = min(CH, nv - c0);
    XT acc[CH];
#pragma unroll
    for (int q = 0; q < CH; q++) acc[q] = 0;
    const long long nvec = n / W, ldvec = ldv / W;
    const VT *wv = reinterpret_cast<const VT *>(w);
    const VT *Vv = reinterpret_cast<const VT *>(V) + (long long)c0 * ldvec;
    const long long S = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + S < nvec; i += 2 * S) {
        const VT w0 = wv[i], w1 = wv[i + S];
#pragma unroll
        for (int q = 0; q < CH; q++) {
            if (q < nc) {
                const VT a0 = ld_stream(Vv + q * ldvec + i), a1 = ld_stream(Vv + q * ldvec + i + S);
                acc[q] += vdot(a0, w0);
                acc[q] += vdot(a1, w1);
            }
        }
    }
    for (; i < nvec; i += S) {
        const VT w0 = wv[i];
#pragma unroll
        for (int q = 0; q < CH; q++)
            if (q < nc) acc[q] += vdot(ld_stream(Vv + q * ldvec + i), w0);
    }
    // columns this CTA holds only (nc is the same in all its warps); each
    // warp adds its lanes' sums in XT (FP64 shuffles and adds are slow on
    // this GPU), then the CTA's warps and the grid's CTAs in FP64
    __shared__ double sh[CH][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < CH; q++) {
        if (q < nc) {
            const XT v = warp_sum(acc[q]);
            if (lane == 0) sh[q][wid] = (double)v;
        }
    }
    __syncthreads();
    if (threadIdx.x < CH * 32 && (int)(threadIdx.x >> 5) < nc) {
        const int q = threadIdx.x >> 5;
        double v = lane < (int)(blockDim.x >> 5) ? sh[q][lane] : 0.0;
        v = warp_sum(v);
        if (lane == 0) part[(long long)(c0 + q) * gridDim.x + blockIdx.x] = v;
    }
    const unsigned total = gridDim.x * gridDim.y;
    if (last_cta_arrives(ticket, total)) {
        __shared__ double shp[32];
        cta_sum_columns(part, gridDim.x, nv, shp, [&](int k, double s) {
            coef[k] = s;
            if (hcol) hcol[k] = ACCUM ? hcol[k] + s : s;
        });
    }
}

// Epilogues run by one thread of the last CTA of k_update, after ||w|| is known.
enum UpdateEpilogue : int {
    kEpiNone = 0,      // store sqrt(sum) into *norm_out, 1/sqrt into st->scale
    kEpiGmres = 1,     // GMRES: H column j, Givens rotations, convergence test
};

struct GmresEpi {
    double *H;   // (m+1) x m column-major Hessenberg, ld = m+1
    double *cs;  // Givens cosines [m]
    double *sn;  // Givens sines [m]
    double *e;   // rhs of the least squares problem [m+1]
    int j;       // iteration inside the cycle
    int m;
};

__device__ __forceinline__ void gmres_givens_step(KrylovState *st, const GmresEpi &g, double hn)
{
    const int ld = g.m + 1, j = g.j;
    double *h = g.H + (long long)j * ld;
    h[j + 1] = hn;
    st->scale = 1.0 / hn;
    // include/senk_gmres.hpp:230-236 / senk_blas1.hpp:145-168
    for (int k = 0; k < j; k++) {
        const double t = h[k];
        h[k] = g.cs[k] * t - g.sn[k] * h[k + 1];
        h[k + 1] = g.sn[k] * t + g.cs[k] * h[k + 1];
    }
    const double a = h[j], b = h[j + 1];
    const double r = sqrt(a * a + b * b);
    g.cs[j] = a / r;
    g.sn[j] = -b / r;
    h[j] = r;
    h[j + 1] = 0;
    g.e[j + 1] = g.sn[j] * g.e[j];
    g.e[j] = g.cs[j] * g.e[j];
    if (!(r == r) || r == 0.0) st->breakdown = 1;
    if (fabs(g.e[j + 1]) <= st->nrm_b * st->eps) {
        st->done = 1;
        st->jconv = j + 1;
        st->res = fabs(g.e[j + 1]) / st->nrm_b;
    }
}

// w -= sum_k coef[k] V_k, and ||w||^2 reduced to the last CTA, which runs the
// epilogue.  nv <= 64.
template <typename XT, int EPI>
__global__ void __launch_bounds__(kThreads)
k_update(const XT *__restrict__ V, long long ldv, int nv, const double *__restrict__ coef,
         XT *__restrict__ w, long long n, double *part, unsigned *ticket, double *norm_out,
         KrylovState *st, GmresEpi g, const int *gate)
{
    if (gated(gate)) return;
    using A = typename Acc<XT>::type;  // FP32 vectors are updated on the FP32 pipe
    __shared__ A sc[64];
    if (threadIdx.x < nv) sc[threadIdx.x] = (A)coef[threadIdx.x];
    __syncthreads();
    A nacc = 0;
    const long long S = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * S < n; i += 4 * S) {  // four independent elements per step
        A v0 = (A)w[i], v1 = (A)w[i + S], v2 = (A)w[i + 2 * S], v3 = (A)w[i + 3 * S];
#pragma unroll 2
        for (int k = 0; k < nv; k++) {
            const XT *vk = V + (long long)k * ldv + i;
            const A c = sc[k];
            const A a0 = (A)ld_stream(vk), a1 = (A)ld_stream(vk + S), a2 = (A)ld_stream(vk + 2 * S),
                    a3 = (A)ld_stream(vk + 3 * S);
            v0 -= c * a0;
            v1 -= c * a1;
            v2 -= c * a2;
            v3 -= c * a3;
        }
        const XT t0 = (XT)v0, t1 = (XT)v1, t2 = (XT)v2, t3 = (XT)v3;
        w[i] = t0;
        w[i + S] = t1;
        w[i + 2 * S] = t2;
        w[i + 3 * S] = t3;
        nacc += (A)t0 * (A)t0;
        nacc += (A)t1 * (A)t1;
        nacc += (A)t2 * (A)t2;
        nacc += (A)t3 * (A)t3;
    }
    for (; i < n; i += S) {
        A v = (A)w[i];
        for (int k = 0; k < nv; k++) v -= sc[k] * (A)ld_stream(V + (long long)k * ldv + i);
        const XT vt = (XT)v;
        w[i] = vt;
        nacc += (A)vt * (A)vt;
    }
    __shared__ double sh[32];
    double t = block_sum((double)nacc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    if (last_cta_arrives(ticket, gridDim.x)) {
        __shared__ double shp[32];
        const double s = cta_sum_partials(part, gridDim.x, shp);
        if (threadIdx.x == 0) {
            const double hn = sqrt(s);
            if (norm_out) *norm_out = hn;
            if (EPI == kEpiGmres) gmres_givens_step(st, g, hn);
            else st->scale = 1.0 / hn;
        }
    }
}

// k_update with 16-byte loads and stores (same conditions as k_multidot_v).
template <typename XT, int EPI>
__global__ void __launch_bounds__(kThreads)
k_update_v(const XT *__restrict__ V, long long ldv, int nv, const double *__restrict__ coef,
           XT *__restrict__ w, long long n, double *part, unsigned *ticket, double *norm_out,
           KrylovState *st, GmresEpi g, const int *gate)
{
    if (gated(gate)) return;
    using VT = typename Vec16<XT>::type;
    constexpr int W = Vec16<XT>::n;
    __shared__ XT sc[64];
    if (threadIdx.x < nv) sc[threadIdx.x] = (XT)coef[threadIdx.x];
    __syncthreads();
    XT nacc = 0;
    const long long nvec = n / W, ldvec = ldv / W;
    VT *wv = reinterpret_cast<VT *>(w);
    const VT *Vv = reinterpret_cast<const VT *>(V);
    const long long S = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + S < nvec; i += 2 * S) {
        VT v0 = wv[i], v1 = wv[i + S];
#pragma unroll 4
        for (int k = 0; k < nv; k++) {
            const VT a0 = ld_stream(Vv + k * ldvec + i), a1 = ld_stream(Vv + k * ldvec + i + S);
            vaxpy(v0, sc[k], a0);
            vaxpy(v1, sc[k], a1);
        }
        wv[i] = v0;
        wv[i + S] = v1;
        nacc += vdot(v0, v0);
        nacc += vdot(v1, v1);
    }
    for (; i < nvec; i += S) {
        VT v0 = wv[i];
        for (int k = 0; k < nv; k++) vaxpy(v0, sc[k], ld_stream(Vv + k * ldvec + i));
        wv[i] = v0;
        nacc += vdot(v0, v0);
    }
    __shared__ double sh[32];
    // lanes in XT, then the warps in FP64 (as in k_multidot_v)
    const XT wsum = warp_sum(nacc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = (double)wsum;
    __syncthreads();
    double t = 0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        t = warp_sum(t);
    }
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    if (last_cta_arrives(ticket, gridDim.x)) {
        __shared__ double shp[32];
        const double s = cta_sum_partials(part, gridDim.x, shp);
        if (threadIdx.x == 0) {
            const double hn = sqrt(s);
            if (norm_out) *norm_out = hn;
            if (EPI == kEpiGmres) gmres_givens_step(st, g, hn);
            else st->scale = 1.0 / hn;
        }
    }
}

// Whether the Krylov kernels take 16-byte vectors for these operands: FP32
// vectors only (measured: the FP64 form of the dot product stalls on the
// texture pipe and runs at less than half the scalar kernel's rate).
template <typename XT>
inline bool vec16_ok(const void *a, const void *b, long long n, long long ld)
{
    constexpr int W = 16 / sizeof(XT);
    return sizeof(XT) == 4 && n % W == 0 && ld % W == 0 && ((uintptr_t)a & 15) == 0 && ((uintptr_t)b & 15) == 0;
}

// Launchers that take the 16-byte kernels when the operands allow.
template <typename XT, bool ACCUM>
inline void launch_multidot(dim3 grid, cudaStream_t s, const XT *V, long long ldv, int nv, const XT *w, long long n,
                            double *part, unsigned *ticket, double *coef, double *hcol, const int *gate)
{
    if (vec16_ok<XT>(V, w, n, ldv)) {
        // the same number of CTAs in all: column blocks share the row slices
        grid.x = max(1u, grid.x / grid.y);
        k_multidot_v<XT, ACCUM><<<grid, kThreads, 0, s>>>(V, ldv, nv, w, n, part, ticket, coef, hcol, gate);
    } else {
        k_multidot<XT, ACCUM><<<grid, kThreads, 0, s>>>(V, ldv, nv, w, n, part, ticket, coef, hcol, gate);
    }
}

template <typename XT, int EPI>
inline void launch_update(int grid, cudaStream_t s, const XT *V, long long ldv, int nv, const double *coef, XT *w,
                          long long n, double *part, unsigned *ticket, double *norm_out, KrylovState *st, GmresEpi g,
                          const int *gate)
{
    if (vec16_ok<XT>(V, w, n, ldv))
        k_update_v<XT, EPI><<<grid, kThreads, 0, s>>>(V, ldv, nv, coef, w, n, part, ticket, norm_out, st, g, gate);
    else
        k_update<XT, EPI><<<grid, kThreads, 0, s>>>(V, ldv, nv, coef, w, n, part, ticket, norm_out, st, g, gate);
}

// Back-solve of the Hessenberg least squares (include/senk_blas2.hpp:24-34) for
// the J = (converged ? jconv : m) columns of this cycle; one thread.
static __global__ void k_gmres_trsv(KrylovState *st, const double *H, const double *e, double *y, int m)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int ld = m + 1;
    const int J = st->done ? st->jconv : m;
    for (int i = J - 1; i >= 0; i--) {
        double t = e[i];
        for (int k = J - 1; k > i; k--) t -= H[(long long)k * ld + i] * y[k];
        y[i] = t / H[(long long)i * ld + i];
    }
    for (int i = J; i < m; i++) y[i] = 0;
}

// Solution update of a cycle. PRE: V0 = y0*V0 + sum_{k<J} y_k V_k (then the
// caller applies the preconditioner and adds it to x), as
// include/senk_gmres.hpp:249-252; otherwise x += sum_k y_k V_k (:80-82).
template <typename XT, bool PRE>
__global__ void __launch_bounds__(kThreads)
k_gmres_combine(XT *__restrict__ V, long long ldv, const double *__restrict__ y, const KrylovState *st,
                XT *__restrict__ x, long long n, int m)
{
    using A = typename Acc<XT>::type;
    __shared__ A sy[64];
    const int J = st->done ? st->jconv : m;
    if (threadIdx.x < J) sy[threadIdx.x] = (A)y[threadIdx.x];
    __syncthreads();
    const long long S = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * S < n; i += 4 * S) {  // four independent elements per step
        A v[4];
#pragma unroll
        for (int u = 0; u < 4; u++) v[u] = PRE ? sy[0] * (A)V[i + u * S] : (A)x[i + u * S];
        for (int k = PRE ? 1 : 0; k < J; k++) {
            const XT *vk = V + (long long)k * ldv + i;
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] += sy[k] * (A)vk[u * S];
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (PRE) V[i + u * S] = (XT)v[u];
            else x[i + u * S] = (XT)v[u];
        }
    }
    for (; i < n; i += S) {
        if (PRE) {
            A v = sy[0] * (A)V[i];
            for (int k = 1; k < J; k++) v += sy[k] * (A)V[(long long)k * ldv + i];
            V[i] = (XT)v;
        } else {
            A v = (A)x[i];
            for (int k = 0; k < J; k++) v += sy[k] * (A)V[(long long)k * ldv + i];
            x[i] = (XT)v;
        }
    }
}

// --------------------------------------------------------------- ILU sweep

// One group of the chain-major factor layout: up to 32 chains of one colour (a
// chain = bsize consecutive schedule positions solved in order, one ABMC block),
// one chain per lane. Row l of a group has we[l] external slots followed, after
// all rows' external slots, by wi[l] in-chain slots; slot k of row l of the
// chain in `lane` sits at off + (slot_index)*32 + lane, so a warp's loads of one
// slot coalesce. In-chain slots hold chain-local row numbers; unused slots hold
// column -1. The widths (uint8 we[BS], wi[BS]) are at widths + widx.
struct GroupDesc {
    int pos0;       // schedule position of chain 0, row 0
    int off;        // element offset of the group's first slot
    int nchains;    // chains in this group (<= 32)
    int widx;       // byte offset of this group's widths
};
static_assert(sizeof(GroupDesc) == 16, "GroupDesc is one 16-byte load");

constexpr unsigned kWaitLimit = 1u << 24;  // polls of a TMA wait before it is declared failed

// Sweep of one colour: L (forward, unit diagonal) or U (backward, inverted
// diagonal in dinv). One CTA of BS warps solves one group of up to 32 chains:
//  * phase 1 (all warps): warp l takes row l of every chain (lane = chain) and
//    subtracts that row's external entries (columns of other colours, already
//    final); the warp reads slot k of row l as one 32-wide row of the staged
//    block, so shared-memory reads are conflict-free and every lane of an FP64
//    instruction is useful;
//  * phase 2 (warp 0, one lane per chain): the chain's rows in solve order with
//    their in-chain entries, all operands on chip;
//  * all warps store the finished rows.
// Per row the subtraction order is the reference's: external entries, then
// in-chain ones, each in the reference's column order.
//
// STAGED: the group's factor block (values and columns, contiguous in the
// layout) is copied to shared memory by two TMA bulk copies issued before the
// kernel waits for the previous colour (programmatic dependent launch), so the
// loads of colour k+1 overlap the tail of colour k. A TMA wait that does not end
// within kWaitLimit polls sets *status; the CTA then waits once more (bounded)
// for its copies and leaves.
template <typename VT, typename XT, int BS, bool UPPER, bool MAPPED, bool STAGED>
__global__ void __launch_bounds__(BS * 32)
k_sweep(const GroupDesc *__restrict__ groups, int g_begin, const unsigned char *__restrict__ widths,
        const VT *__restrict__ val, const int *__restrict__ col, const VT *__restrict__ dinv,
        const int *__restrict__ rowmap, const XT *x, XT *y, const int *gate, int *status)
{
    extern __shared__ __align__(128) unsigned char dsm[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ XT tsh[BS][32];    // row l of chain q
    __shared__ XT dsh[UPPER ? BS : 1][32];
    __shared__ int wsh[2 * BS];   // we[BS], wi[BS]
    const int g = g_begin + blockIdx.x;
    const int l = threadIdx.x >> 5, q = threadIdx.x & 31;
    const GroupDesc d = groups[g];
    if (threadIdx.x < 2 * BS) wsh[threadIdx.x] = widths[d.widx + threadIdx.x];
    __syncthreads();
    int eo = 0, etot = 0;
#pragma unroll
    for (int r = 0; r < BS; r++) {
        if (r < l) eo += wsh[r];
        etot += wsh[r];
    }
    int itot = 0;
#pragma unroll
    for (int r = 0; r < BS; r++) itot += wsh[BS + r];
    const int slots = etot + itot;
    const unsigned vbytes = (unsigned)slots * 32u * sizeof(VT), cbytes = (unsigned)slots * 32u * 4u;
    const VT *vb;
    const int *cb;
    if (STAGED) {
        VT *sv = reinterpret_cast<VT *>(dsm);
        int *sc = reinterpret_cast<int *>(dsm + vbytes);
        if (threadIdx.x == 0) {
            mbar_init(&bar, 1);
            if (slots > 0) {
                mbar_expect_tx(&bar, vbytes + cbytes);
                bulk_g2s(sv, val + d.off, vbytes, &bar);
                bulk_g2s(sc, col + d.off, cbytes, &bar);
            }
        }
        __syncthreads();
        vb = sv;
        cb = sc;
    } else {
        vb = val + d.off;
        cb = col + d.off;
    }
    pdl_launch_dependents();
    pdl_wait();  // the previous colour (or the producer of x) has finished
    const bool skip = gated(gate);
    bool ok = true;
    if (STAGED && slots > 0) ok = mbar_wait_bounded(&bar, 0, kWaitLimit);
    if (__syncthreads_or(!ok)) {  // leave together: no thread may wait at a later barrier alone
        if (threadIdx.x == 0) atomicExch(status, 1);
        if (!ok) mbar_wait_bounded(&bar, 0, kWaitLimit);
        return;
    }
    if (skip) return;
    const bool live = q < d.nchains;
    const int pos = d.pos0 + q * BS + l;
    const int row = live ? (MAPPED ? __ldg(rowmap + pos) : pos) : 0;
    XT t = live ? x[row] : XT(0);
    // Phase 1: row l's external entries.
    const int we = wsh[l];
    for (int k = 0; k < we; k++) {
        const int at = (eo + k) * 32 + q;
        const int c = STAGED ? cb[at] : ld_stream(cb + at);
        const VT v = STAGED ? vb[at] : ld_stream(vb + at);
        if (c >= 0) t -= (XT)v * y[c];
    }
    if (BS == 1) {
        if (UPPER && live) t *= (XT)__ldg(dinv + pos);
        if (live) y[row] = t;
        return;
    }
    tsh[l][q] = t;
    if (UPPER) dsh[l][q] = live ? (XT)__ldg(dinv + pos) : XT(0);
    __syncthreads();
    // Phase 2: one lane per chain, rows in solve order.
    if (l == 0) {
        // slot offset of row r's in-chain entries: etot + sum of wi over rows < r,
        // walked upwards for L and downwards for U
        int io = etot;
        if (UPPER) {
            for (int r = 0; r < BS; r++) io += wsh[BS + r];
        }
#pragma unroll 4
        for (int s = 0; s < BS; s++) {
            const int r = UPPER ? BS - 1 - s : s;
            XT tt = tsh[r][q];
            const int wi = wsh[BS + r];
            if (UPPER) io -= wi;
            const int ro = io;
            if (!UPPER) io += wi;
            for (int k = 0; k < wi; k++) {
                const int at = (ro + k) * 32 + q;
                const int c = cb[at];
                const VT v = vb[at];
                if (c >= 0) tt -= (XT)v * tsh[c][q];
            }
            if (UPPER) tt *= dsh[r][q];
            tsh[r][q] = tt;
        }
    }
    __syncthreads();
    if (live) y[row] = tsh[l][q];
}

// ------------------------------------------------- small systems, one CTA
// One triangular factor in the compact chain layout, chains of one row (level
// sets of the natural order, or AMC colours), for k_ilu_small.
template <typename VT>
struct SmallFactor {
    const WfGroup *groups;
    const int2 *chains;
    const VT *val;
    const int *col;
    const VT *cdinv;        // U: inverted diagonal per chain
    const int4 *levels;     // per colour (level set), processing order: {first group, groups, first slot, slots}
    int ncolours;
};

// Stages the data of one level (colour) lv into buf with bulk copies counted on
// bar: group descriptors, chain descriptors, the groups' blocks (columns, then
// values) and, for U, the chains' inverted diagonals. One thread; no global
// loads, so a stage costs the issuing thread a few instructions.
template <typename VT>
__device__ __forceinline__ void small_stage(const SmallFactor<VT> &F, bool upper, int4 lv, unsigned char *buf,
                                            unsigned long long *bar)
{
    const int g0 = lv.x, G = lv.y, e0 = lv.z, ne = lv.w;
    const unsigned bytes = G > 0 ? (unsigned)G * 16u + (unsigned)G * 256u + (unsigned)ne * (4u + (unsigned)sizeof(VT)) +
                                       (upper ? (unsigned)G * 32u * (unsigned)sizeof(VT) : 0u)
                                 : 0u;
    // earlier generic accesses to this buffer come before the async writes
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(bar, bytes);
    if (G == 0) return;
    unsigned char *p = buf;
    bulk_g2s(p, F.groups + g0, (unsigned)G * 16u, bar);
    p += G * 16;
    bulk_g2s(p, F.chains + (size_t)g0 * 32, (unsigned)G * 256u, bar);
    p += G * 256;
    if (ne > 0) {
        bulk_g2s(p, F.col + e0, (unsigned)ne * 4u, bar);
        p += (size_t)ne * 4;
        bulk_g2s(p, F.val + e0, (unsigned)ne * (unsigned)sizeof(VT), bar);
        p += (size_t)ne * sizeof(VT);
    }
    if (upper) bulk_g2s(p, F.cdinv + (size_t)g0 * 32, (unsigned)G * 32u * (unsigned)sizeof(VT), bar);
}

// Both triangular sweeps of one ILU application y = U^-1 L^-1 x for a system
// whose vector fits in shared memory, in one CTA (which: bit 0 L, bit 1 U;
// x == y allowed). The levels (colours) run in order, one consumer thread per
// row, with a barrier among the consumers between levels. The last warp stages:
// its first lane copies each level's data by TMA into one of nbuf buffers (2 to
// 8) as soon as the consumers have released that buffer (full / empty
// mbarriers per buffer), so up to nbuf levels are in flight ahead of the one
// being solved and no staging work lies on the consumers' path. A wait that
// runs out sets *status = 2 and a shared abort flag; the other side stops at
// its next wait, and the stager waits (bounded) for every copy it issued
// before it leaves.
constexpr int kSmallMaxBufs = 8;

template <typename VT, typename XT>
__global__ void __launch_bounds__(1024)
k_ilu_small(SmallFactor<VT> Lf, SmallFactor<VT> Uf, int which, const XT *x, XT *y, int n, const int *gate,
            int *status, int buf_bytes, int nbuf)
{
    extern __shared__ __align__(128) unsigned char sms[];
    __shared__ __align__(8) unsigned long long full[kSmallMaxBufs], empty[kSmallMaxBufs];
    __shared__ int abort_flag;
    if (gated(gate)) return;
    const int nl = (which & 1) ? Lf.ncolours : 0, nu = (which & 2) ? Uf.ncolours : 0, steps = nl + nu;
    // shared memory: the vector, the descriptors of all levels in processing
    // order (copied once, so the stager reads no global memory between levels),
    // then the staging buffers (small_smem_bytes)
    XT *ysh = reinterpret_cast<XT *>(sms);
    int4 *lvs = reinterpret_cast<int4 *>(sms + ((size_t)n * sizeof(XT) + 127) / 128 * 128);
    unsigned char *bufs = reinterpret_cast<unsigned char *>(lvs) + ((size_t)steps * 16 + 127) / 128 * 128;
    const int ncons = (int)blockDim.x - 32;  // consumer threads; the last warp stages
    if (threadIdx.x == 0) {
        for (int b = 0; b < nbuf; b++) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        abort_flag = 0;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) ysh[i] = x[i];
    for (int j = threadIdx.x; j < steps; j += blockDim.x)
        lvs[j] = j < nl ? __ldg(Lf.levels + j) : __ldg(Uf.levels + (j - nl));
    __syncthreads();
    if ((int)threadIdx.x >= ncons) {
        if ((int)threadIdx.x != ncons) return;
        // stager: step j fills buffer b = j % nbuf for its (j / nbuf)-th time
        int issued = 0;
        unsigned epar = 0u;  // bit b: parity of buffer b's next release
        for (int j = 0, b = 0; j < steps; j++, b = b + 1 == nbuf ? 0 : b + 1) {
            if (j >= nbuf) {  // released by the consumers after step j - nbuf
                const unsigned par = (epar >> b) & 1u;
                epar ^= 1u << b;
                bool got = false;
                for (unsigned i = 0; i < kWaitLimit && !got; i++) {
                    got = mbar_try_wait(&empty[b], par);
                    if (!got && *(volatile int *)&abort_flag) break;
                }
                if (!got) {
                    if (!*(volatile int *)&abort_flag) {
                        atomicExch(status, 2);
                        *(volatile int *)&abort_flag = 1;
                    }
                    break;
                }
            }
            unsigned char *buf = bufs + (size_t)b * buf_bytes;
            if (j < nl) small_stage(Lf, false, lvs[j], buf, &full[b]);
            else small_stage(Uf, true, lvs[j], buf, &full[b]);
            issued = j + 1;
        }
        // the last use of each buffer: complete (consumed or not) before the CTA leaves
        for (int j = issued > nbuf ? issued - nbuf : 0; j < issued; j++)
            mbar_wait_bounded(&full[j % nbuf], (unsigned)(j / nbuf) & 1u, kWaitLimit);
        return;
    }
    // consumers: one barrier per level. A wait that runs out sets the abort
    // flag (and *status = 2) before the level's barrier; after it every
    // consumer sees the flag and all leave together.
    unsigned fpar = 0u;  // bit b: parity of buffer b's next fill
    for (int k = 0, b = 0; k < steps; k++, b = b + 1 == nbuf ? 0 : b + 1) {
        const bool upper = k >= nl;
        const bool ok = mbar_wait_bounded(&full[b], (fpar >> b) & 1u, kWaitLimit);
        fpar ^= 1u << b;
        if (!ok) {
            atomicExch(status, 2);
            *(volatile int *)&abort_flag = 1;
        }
        if (ok && !*(volatile int *)&abort_flag) {
            const int4 lv = lvs[k];
            const int G = lv.y, e0 = lv.z, ne = lv.w;
            const unsigned char *sb = bufs + (size_t)b * buf_bytes;
            const WfGroup *sd = reinterpret_cast<const WfGroup *>(sb);
            const int2 *sc = reinterpret_cast<const int2 *>(sb + G * 16);
            const int *scol = reinterpret_cast<const int *>(sb + G * 16 + G * 256);
            const VT *sval = reinterpret_cast<const VT *>(sb + G * 16 + G * 256 + (size_t)ne * 4);
            const VT *sdinv = reinterpret_cast<const VT *>(sb + G * 16 + G * 256 + (size_t)ne * (4 + sizeof(VT)));
            for (int t = threadIdx.x; t < G * 32; t += ncons) {
                const int gi = t >> 5, lane = t & 31;
                const WfGroup d = sd[gi];
                if (lane >= d.nchains) continue;
                const int2 ch = sc[t];
                const int row = ch.x, E = ch.y & 0xffff;
                const int base = d.off - e0 + lane;
                XT tt = ysh[row];
                for (int e = 0; e < E; e++) tt -= (XT)sval[base + e * 32] * ysh[scol[base + e * 32] & kColMask];
                if (upper) tt *= (XT)sdinv[t];
                ysh[row] = tt;
            }
        }
        named_bar(1, ncons);  // the level's rows are final and buffer b is free
        if (*(volatile int *)&abort_flag) return;
        if (threadIdx.x == 0) mbar_arrive(&empty[b]);
    }
    for (int i = threadIdx.x; i < n; i += ncons) y[i] = ysh[i];
}

// Dynamic shared memory of k_ilu_small: vector, level descriptors, buffers.
inline size_t small_smem_bytes(size_t n, size_t xt_bytes, int steps, size_t buf_bytes, int nbuf)
{
    return (n * xt_bytes + 127) / 128 * 128 + ((size_t)steps * 16 + 127) / 128 * 128 + (size_t)nbuf * buf_bytes;
}

// ------------------------------------------------------ dataflow sweeps
// One launch per triangular sweep, one group of up to 32 chains per warp.
//
// Layout ("compact chains"): the chains of a colour are sorted by their entry
// counts and taken 32 at a time; chain q of group g is lane q. Its external
// entries (columns of other chains, all in earlier colours) are packed one
// after another, entry k at off + k*32 + q, followed after the group's widest
// chain by its in-chain entries, so a group pads only to its widest chain
// (chains of similar counts are grouped). Both parts list rows in solve order
// and each row's entries in the reference's subtraction order. Column words:
// external (row << 27) | column, in-chain (row << 8) | chain-local column,
// rows chain-local. Per chain: int2 {first row, E | I << 16}, E and I its
// external and in-chain entry counts.
//
// Schedule: warps take groups in processing order from a counter, stage the
// group's block into their shared memory with two TMA bulk copies, read x of
// their chains' rows, and wait until every group their external columns belong
// to has published its flag for this sweep (flags hold the sweep's epoch;
// acquire/release at GPU scope). A group only reads groups taken before it by
// running warps, so every wait ends. Then, per lane: the external entries'
// products are gathered (all loads of a batch in flight together) and
// subtracted row by row; the in-chain recurrence runs on chip in shared memory;
// the rows are stored and the group's flag is published. The last warp to
// finish resets the counter and starts the next epoch.
//
// ctrl = {counter, epoch, abort, warps finished}. A wait that runs out of polls
// sets abort and *status; later waits give up at once; the launch then drains
// and the last warp clears abort (the status stays set for the host).
constexpr unsigned kFlagPolls = 1u << 21;  // polls of a dependency flag (64 ns back-off each) before giving up

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_release_add(int *p, int v)
{
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
__device__ __forceinline__ T ld_l2(const T *p) { return __ldcg(p); }

// Shared memory of one warp: the staged block (columns, then values) of
// slots_max slots, the chain rows tsh[BS][32] and, for U, the inverted diagonal
// dsh[BS][32], then the warp's mbarrier (wf_bytes_for in wf_layout.hpp).
template <typename VT, typename XT, int BS, bool UPPER>
__host__ __device__ constexpr size_t wf_warp_bytes(int slots_max)
{
    return ((size_t)slots_max * 32 * (4 + sizeof(VT)) + (size_t)BS * 32 * sizeof(XT) * (UPPER ? 2 : 1) + 8 + 15) /
           16 * 16;
}

// Solves one staged group (compact chain layout) for lane `lane` = chain:
// tsh[BS][32] holds x of the chain's rows on entry and the solved rows on exit
// (dsh: U's inverted diagonal). Products of the external entries are gathered
// G at a time (all loads of a batch in flight together) and subtracted row by
// row; then the in-chain recurrence, rows in solve order, on chip.
template <typename VT, typename XT, int BS, bool UPPER>
__device__ __forceinline__ void wf_solve_group(const WfGroup &d, int E, int I, const int *cw, const VT *vw, XT *tsh,
                                               const XT *dsh, const XT *y, int lane)
{
    constexpr int G = sizeof(XT) == 4 ? 16 : 8;
    XT t = XT(0);
    int cur = -1;
    for (int b = 0; b < d.emax; b += G) {
        XT gv[G];
#pragma unroll
        for (int u = 0; u < G; u++) {
            const int e = b + u;
            gv[u] = XT(0);
            if (e < E) gv[u] = ld_l2(y + (cw[e * 32 + lane] & kColMask));
        }
#pragma unroll
        for (int u = 0; u < G; u++) {
            const int e = b + u;
            if (e < E) {
                const int r = (int)((unsigned)cw[e * 32 + lane] >> kColBits);
                if (r != cur) {
                    if (cur >= 0) tsh[cur * 32 + lane] = t;
                    cur = r;
                    t = tsh[r * 32 + lane];
                }
                t -= (XT)vw[e * 32 + lane] * gv[u];
            }
        }
    }
    if (cur >= 0) tsh[cur * 32 + lane] = t;
    // this chain's in-chain entries follow those of the lanes before it
    int ibase = I;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, ibase, o);
        if (lane >= o) ibase += v;
    }
    ibase -= I;
    const int *iw = cw + d.emax * 32 + ibase;
    const VT *iv = vw + d.emax * 32 + ibase;
    int e = 0;
#pragma unroll
    for (int s = 0; s < BS; s++) {
        const int r = UPPER ? BS - 1 - s : s;
        XT tt = tsh[r * 32 + lane];
        while (e < I) {
            const int w = iw[e];
            if ((w >> 8) != r) break;
            tt -= (XT)iv[e] * tsh[(w & 255) * 32 + lane];
            e++;
        }
        if (UPPER) tt *= dsh[r * 32 + lane];
        tsh[r * 32 + lane] = tt;
    }
}

template <typename VT, typename XT, int BS, bool UPPER>
__global__ void __launch_bounds__(256)
k_sweep_wf(const WfGroup *__restrict__ groups, int g0, int ng, const int2 *__restrict__ chains,
           const VT *__restrict__ val, const int *__restrict__ col, const VT *__restrict__ dinv,
           const int *__restrict__ dep_ptr, const int *__restrict__ dep_idx, int *flags, int *ctrl, const XT *x,
           XT *y, const int *gate, int *status, int slots_max)
{
    extern __shared__ __align__(128) unsigned char wfs[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const size_t per_warp = wf_warp_bytes<VT, XT, BS, UPPER>(slots_max);
    unsigned char *base = wfs + (size_t)wib * per_warp;
    int *cw = reinterpret_cast<int *>(base);
    VT *vw = reinterpret_cast<VT *>(base + (size_t)slots_max * 32 * 4);
    XT *tsh = reinterpret_cast<XT *>(base + (size_t)slots_max * 32 * (4 + sizeof(VT)));
    XT *dsh = tsh + BS * 32;
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(base + per_warp - 16);
    pdl_wait();  // the previous kernel (e.g. the other sweep) has finished
    if (gated(gate)) return;
    if (lane == 0) mbar_init(bar, 1);
    __syncwarp();
    const int epoch = *(volatile const int *)(ctrl + 1);
    unsigned phase = 0;
    for (;;) {
        int g = 0;
        if (lane == 0) g = g0 + atomicAdd(ctrl, 1);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ng) break;
        const WfGroup d = groups[g];
        const int slots = d.emax + d.imax;
        // one read of the abort flag for the whole warp
        bool ok = __shfl_sync(0xffffffffu, lane == 0 ? (int)(*(volatile const int *)(ctrl + 2) == 0) : 0, 0) != 0;
        const bool staged = ok && slots > 0;
        if (staged && lane == 0) {
            mbar_expect_tx(bar, (unsigned)slots * 32u * (4u + (unsigned)sizeof(VT)));
            bulk_g2s(cw, col + d.off, (unsigned)slots * 32u * 4u, bar);
            bulk_g2s(vw, val + d.off, (unsigned)slots * 32u * (unsigned)sizeof(VT), bar);
        }
        const bool live = lane < d.nchains;
        const int2 ch = live ? __ldg(chains + (size_t)g * 32 + lane) : make_int2(0, 0);
        const int r0 = ch.x, E = ch.y & 0xffff, I = (int)((unsigned)ch.y >> 16);
        // x of the chain's rows (and U's inverted diagonal) while the block arrives
#pragma unroll
        for (int l = 0; l < BS; l++) {
            tsh[l * 32 + lane] = live ? x[r0 + l] : XT(0);
            if (UPPER) dsh[l * 32 + lane] = live ? (XT)__ldg(dinv + r0 + l) : XT(0);
        }
        // the groups this one reads from
        for (int i = dep_ptr[g] + lane; ok && i < dep_ptr[g + 1]; i += 32) {
            const int *f = flags + __ldg(dep_idx + i);
            unsigned k = 0;
            while (ld_acquire(f) != epoch) {
                __nanosleep(64);
                if (++k > kFlagPolls || *(volatile const int *)(ctrl + 2)) {
                    atomicExch(ctrl + 2, 1);
                    atomicExch(status, 1);
                    ok = false;
                    break;
                }
            }
        }
        ok = __all_sync(0xffffffffu, ok);
        if (staged) {
            const bool arrived = __all_sync(0xffffffffu, mbar_wait_bounded(bar, phase, kWaitLimit));
            phase ^= 1u;
            if (!arrived) {
                // the copy did not complete: report, wait once more for it, and
                // stop using this buffer (this warp takes no more groups)
                if (lane == 0) {
                    atomicExch(ctrl + 2, 1);
                    atomicExch(status, 2);
                }
                mbar_wait_bounded(bar, phase ^ 1u, kWaitLimit);
                __syncwarp();
                if (lane == 0) st_release(flags + g, epoch);
                break;
            }
        }
        if (ok) {
            wf_solve_group<VT, XT, BS, UPPER>(d, E, I, cw, vw, tsh, dsh, y, lane);
            if (live) {
#pragma unroll
                for (int l = 0; l < BS; l++) y[r0 + l] = tsh[l * 32 + lane];
            }
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(flags + g, epoch);
    }
    // the last warp to finish starts the next sweep's epoch
    if (lane == 0) {
        __threadfence();
        const unsigned total = gridDim.x * (blockDim.x >> 5);
        if ((unsigned)atomicAdd(ctrl + 3, 1) == total - 1) {
            ctrl[0] = 0;
            ctrl[2] = 0;
            ctrl[3] = 0;
            __threadfence();
            atomicExch(ctrl + 1, epoch + 1);
        }
    }
}

// Row l's place in one of its chain's count arrays (BS bytes, one per row;
// rows come in solve order, i.e. descending for U): eo = the sum over the rows
// solved before l, ne = row l's own count. With BS >= 8 the counts are read as
// 32-bit words and summed four bytes at a time (__dp4a) under a byte mask of
// the rows that come first.
template <int BS, bool UPPER>
__device__ __forceinline__ void cc_row_counts(const unsigned char *cq, int l, int &eo, int &ne)
{
    eo = 0;
    ne = 0;
    if constexpr (BS >= 8) {
        // the words before (L) or after (U) row l's word count whole; row l's
        // own word counts its bytes below (L) or above (U) row l's
        const uint32_t *cw = reinterpret_cast<const uint32_t *>(cq);
        const int k = l >> 2, b = 8 * (l & 3);
        uint32_t mine = 0;
#pragma unroll
        for (int j = 0; j < BS / 4; j++) {
            const uint32_t v = cw[j];
            if (UPPER ? j > k : j < k) eo += (int)__dp4a(v, 0x01010101u, 0u);
            if (j == k) mine = v;
        }
        const uint32_t m = UPPER ? (b == 24 ? 0u : ~0u << (b + 8)) : (1u << b) - 1u;
        eo += (int)__dp4a(mine & m, 0x01010101u, 0u);
        ne = (int)((mine >> b) & 255u);
    } else {
#pragma unroll
        for (int r = 0; r < BS; r++)
            if (UPPER ? r > l : r < l) eo += cq[r];
        ne = cq[l];
    }
}

// In-chain recurrence of one chain qc in the BS lanes [BS*k, BS*k+BS) of a warp
// (lane = row rr): the rows are finished in solve order; the lane of the row
// finished at step s (U: after its inverted diagonal) broadcasts it by a
// shuffle within the chain's lanes, and every lane that has an in-chain entry
// in that column subtracts it. A lane's entries come in the same order as the
// steps (the reference's column order): `mask` holds their columns and `at`
// the next one's place in the block. Every lane of the warp calls step(s) for
// every s.
//
// U: `sc` keeps the row's value times its inverted diagonal, recomputed after
// every step, so the lane of column c broadcasts sc (its final value once the
// columns after c are done) and no step selects which lane scales.
template <typename VT, typename XT, int BS, bool UPPER>
struct ChainRec {
    const VT *iv;
    int at, rr;
    uint32_t mask;
    XT tt, di, sc;

    // iw, iv0: the chain's in-chain entries in the block; cc: its 2*BS row
    // counts; t: the row's value after its external entries; d_inv: U's
    // inverted diagonal of the row
    __device__ __forceinline__ void init_at(const int *iw, const VT *iv0, const unsigned char *cc, int row, XT t,
                                            XT d_inv)
    {
        int at0, left;
        cc_row_counts<BS, UPPER>(cc + BS, row, at0, left);
        init_with(iw, iv0, at0, left, row, t, d_inv);
    }

    // as init_at, with the row's first in-chain entry (at0) and their number
    // (left) already known
    __device__ __forceinline__ void init_with(const int *iw, const VT *iv0, int at0, int left, int row, XT t,
                                              XT d_inv)
    {
        rr = row;
        iv = iv0;
        at = at0;
        mask = 0;
#pragma unroll
        for (int k = 0; k < 3; k++)  // a 7-point row's in-chain entries, predicated
            if (k < left) mask |= 1u << (iw[at + k] & 255);
        for (int k = 3; k < left; k++) mask |= 1u << (iw[at + k] & 255);
        tt = t;
        di = d_inv;
        if (UPPER) sc = tt * di;
    }

    // the solved row: U's scaled by its inverted diagonal
    __device__ __forceinline__ XT out() const { return UPPER ? sc : tt; }

    __device__ __forceinline__ void init(const WfGroup &d, const int *cw, const VT *vw, const unsigned char *cnt,
                                         const XT (*tsh)[BS + 1], const XT (*dsh)[BS + 1], const int *ibase, int qc,
                                         int row)
    {
        init_at(cw + d.emax * 32 + ibase[qc], vw + d.emax * 32 + ibase[qc], cnt + qc * 2 * BS, row, tsh[qc][row],
                UPPER ? dsh[qc][row] : XT(1));
    }

    // Each step's subtraction, increment and rescale are predicated on the
    // lane's bit for the step's column.
    __device__ __forceinline__ void step(int s)
    {
        const int c = UPPER ? BS - 1 - s : s;
        const XT yc = __shfl_sync(0xffffffffu, UPPER ? sc : tt, c, BS);
        if (mask & (1u << c)) {  // predicated, no branch
            tt -= (XT)iv[at] * yc;
            at++;
            if (UPPER) sc = tt * di;
        }
    }
};

// One group of the compact chain layout, staged in shared memory (cw, vw: its
// block; cnt: its per-chain row counts), for the thread of row l of chain q
// (t: x of that row on entry): subtracts the row's external entries, then runs
// the in-chain recurrence; the solved rows are in tsh on return (all threads
// past a CTA barrier). NC reads y through the non-coherent path, for kernels in
// which y's earlier rows were written by earlier kernels.
template <typename VT, typename XT, int BS, bool UPPER, bool NC>
__device__ __forceinline__ void cc_solve(const WfGroup &d, const int *cw, const VT *vw, const unsigned char *cnt,
                                         XT (*tsh)[BS + 1], const XT (*dsh)[BS + 1], const int *ibase, XT t,
                                         const XT *y, int l, int q)
{
    int eo, ne;
    cc_row_counts<BS, UPPER>(cnt + q * 2 * BS, l, eo, ne);
    // up to 6 entries at a time (a 7-point stencil row's external entries in
    // one batch; 6 keeps the kernel within 32 registers), all their gathers
    // issued before the first subtraction (one memory latency per batch); the
    // second half of a batch only where a lane of the warp needs it. The
    // subtractions keep the entries' order.
    constexpr int B = 6, H = 3;
    for (int k0 = 0; __any_sync(0xffffffffu, k0 < ne); k0 += B) {  // warp-uniform
        VT vv[B];
        XT yy[B];
        const bool more = __any_sync(0xffffffffu, k0 + H < ne);
#pragma unroll
        for (int u = 0; u < B; u++) {
            if (u >= H && !more) break;
            const bool in = k0 + u < ne;
            const int at = (eo + k0 + u) * 32 + q;
            const int c = in ? (cw[at] & kColMask) : 0;
            vv[u] = in ? vw[at] : VT(0);
            yy[u] = in ? (NC ? __ldg(y + c) : y[c]) : XT(0);
        }
#pragma unroll
        for (int u = 0; u < B; u++) {
            if (u >= H && !more) break;
            if (k0 + u < ne) t -= (XT)vv[u] * yy[u];
        }
    }
    tsh[q][l] = t;
    __syncthreads();
    // In-chain recurrence, BS lanes per chain (lane = row), 32 / BS chains
    // per warp, all warps busy.
    if (BS > 1 || UPPER) {
        constexpr int CPW = 32 / BS;  // chains per warp
        const int lane = threadIdx.x & 31;
        const int qc = l * CPW + lane / BS;
        ChainRec<VT, XT, BS, UPPER> a;
        a.init(d, cw, vw, cnt, tsh, dsh, ibase, qc, lane % BS);
#pragma unroll
        for (int s = 0; s < BS; s++) a.step(s);
        tsh[qc][a.rr] = a.out();
    }
    __syncthreads();
}

// cc_solve with two rows per thread, for a CTA of BS/2 warps (BS >= 4): the
// thread of warp w, lane q takes rows w and w + BS/2 of chain q (t0, t1: x of
// those rows on entry). The external entries of both rows are gathered
// together, up to 4 of each at a time; the in-chain recurrence runs the
// group's 32 chains as two interleaved halves of 16 (2 * 32 / BS chains per
// warp and half). Same subtractions, in the same order, as cc_solve.
template <typename VT, typename XT, int BS, bool UPPER>
__device__ __forceinline__ void cc_solve2(const WfGroup &d, const int *cw, const VT *vw, const unsigned char *cnt,
                                          XT (*tsh)[BS + 1], const XT (*dsh)[BS + 1], const int *ibase, XT t0, XT t1,
                                          const XT *y, int w, int q)
{
    static_assert(BS >= 4, "two rows per thread need at least two warps");
    constexpr int W = BS / 2;
    const int l0 = w, l1 = w + W;
    int eo0, ne0, eo1, ne1;
    cc_row_counts<BS, UPPER>(cnt + q * 2 * BS, l0, eo0, ne0);
    cc_row_counts<BS, UPPER>(cnt + q * 2 * BS, l1, eo1, ne1);
    const int nmax = max(ne0, ne1);
    for (int k0 = 0; k0 < nmax; k0 += 4) {
        VT va[4], vb[4];
        XT ya[4], yb[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const bool ia = k0 + u < ne0, ib = k0 + u < ne1;
            const int aa = (eo0 + k0 + u) * 32 + q, ab = (eo1 + k0 + u) * 32 + q;
            const int ca = ia ? (cw[aa] & kColMask) : 0, cb = ib ? (cw[ab] & kColMask) : 0;
            va[u] = ia ? vw[aa] : VT(0);
            vb[u] = ib ? vw[ab] : VT(0);
            ya[u] = ia ? __ldg(y + ca) : XT(0);
            yb[u] = ib ? __ldg(y + cb) : XT(0);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (k0 + u < ne0) t0 -= (XT)va[u] * ya[u];
            if (k0 + u < ne1) t1 -= (XT)vb[u] * yb[u];
        }
    }
    tsh[q][l0] = t0;
    tsh[q][l1] = t1;
    __syncthreads();
    {
        constexpr int CPW = 32 / BS;  // chains per warp in each half
        const int lane = threadIdx.x & 31;
        const int qa = w * CPW + lane / BS, qb = qa + 16;
        ChainRec<VT, XT, BS, UPPER> a, b;
        a.init(d, cw, vw, cnt, tsh, dsh, ibase, qa, lane % BS);
        b.init(d, cw, vw, cnt, tsh, dsh, ibase, qb, lane % BS);
#pragma unroll
        for (int s = 0; s < BS; s++) {
            a.step(s);
            b.step(s);
        }
        tsh[qa][a.rr] = a.out();
        tsh[qb][b.rr] = b.out();
    }
    __syncthreads();
}

// Resident CTAs per SM that k_sweep_cc is compiled for: 2,048 threads (the
// SM's limit), i.e. at most 32 registers a thread.
constexpr int cc_min_blocks(int bs) { return 2048 / (bs * 32) < 32 ? 2048 / (bs * 32) : 32; }

// One colour per launch on the compact chain layout, one CTA of BS warps per
// group: warp l takes row l of every chain (lane q = chain q) and subtracts
// that row's external entries, read from the staged block at lane q's offset
// for row l (the per-chain row counts give it; reads of slot e*32+q hit bank q
// whatever e is, so they are conflict-free), gathering y through L1 (earlier
// colours were written by earlier kernels); then the in-chain recurrence with
// one lane per row (below); all warps store the finished rows.
//
// The group's block, its row counts (TMA) and U's inverted diagonal are read
// before the kernel waits for the previous kernel (programmatic dependent
// launch). With early_x, x and the gate are read before the wait too and the
// next kernel may start its prologue only once this one has passed its wait;
// the host sets it only where the kernels still running cannot be writing
// these rows (not for the first colour of a sweep; only the sweeps use
// programmatic launches, so the kernel before a sweep, and every writer of the
// gate, has completed before its second colour starts). A TMA wait that runs
// out sets *status = 2.
template <typename VT, typename XT, int BS, bool UPPER>
__global__ void __launch_bounds__(BS * 32, cc_min_blocks(BS))
k_sweep_cc(const WfGroup *__restrict__ groups, int g0, const int2 *__restrict__ chains,
           const unsigned char *__restrict__ counts, const VT *__restrict__ val, const int *__restrict__ col,
           const VT *__restrict__ dinv, const XT *x, XT *y, const int *gate, int *status, int early_x)
{
    extern __shared__ __align__(128) unsigned char ccs[];
    __shared__ __align__(8) unsigned long long bar;
    // rows of chain q at tsh[q][r]: stride BS + 1 is odd, so both the
    // row-per-warp accesses (lane = chain) and the row-per-lane ones (16 lanes
    // of one chain) fall in different banks
    __shared__ XT tsh[32][BS + 1];
    __shared__ XT dsh[UPPER ? 32 : 1][BS + 1];
    __shared__ int ibase[32];
    const int g = g0 + blockIdx.x;
    const int l = threadIdx.x >> 5, q = threadIdx.x & 31;
    const WfGroup d = groups[g];
    const int slots = d.emax + d.imax;
    const unsigned cbytes = (unsigned)slots * 32u * 4u, vbytes = (unsigned)slots * 32u * (unsigned)sizeof(VT);
    constexpr unsigned nbytes = 32u * 2u * BS;
    int *cw = reinterpret_cast<int *>(ccs);
    VT *vw = reinterpret_cast<VT *>(ccs + cbytes);
    unsigned char *cnt = ccs + cbytes + vbytes;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_expect_tx(&bar, cbytes + vbytes + nbytes);
        if (slots > 0) {
            bulk_g2s(cw, col + d.off, cbytes, &bar);
            bulk_g2s(vw, val + d.off, vbytes, &bar);
        }
        bulk_g2s(cnt, counts + (size_t)g * nbytes, nbytes, &bar);
    }
    __syncthreads();
    const bool live = q < d.nchains;
    const int2 ch = live ? __ldg(chains + (size_t)g * 32 + q) : make_int2(0, 0);
    const int row = ch.x + l;
    if (UPPER) dsh[q][l] = live ? (XT)__ldg(dinv + row) : XT(0);
    if (l == 0) {  // where each chain's in-chain entries start in the block
        const int I = (int)((unsigned)ch.y >> 16);
        int v = I;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (q >= o) v += u;
        }
        ibase[q] = v - I;
    }
    // x and the gate: before the wait where early_x allows it (the gate's
    // writer precedes the sweep), else right after it, so that their loads
    // overlap the staging wait
    XT t = XT(0);
    bool skip = false;
    if (early_x) {
        if (live) t = x[row];
        skip = gated(gate);
    }
    if (!early_x) pdl_launch_dependents();
    pdl_wait();  // the previous colour (or the producer of x) has finished
    if (early_x) pdl_launch_dependents();
    else {
        skip = gated(gate);
        if (live) t = x[row];
    }
    const bool ok = mbar_wait_bounded(&bar, 0, kWaitLimit);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(status, 2);
        if (!ok) mbar_wait_bounded(&bar, 0, kWaitLimit);
        return;
    }
    if (skip) return;
    cc_solve<VT, XT, BS, UPPER, true>(d, cw, vw, cnt, tsh, dsh, ibase, t, y, l, q);
    if (live) y[row] = tsh[q][l];
}

// Resident CTAs per SM that k_sweep_cc2 is compiled for: 1,280 threads, i.e.
// at most 51 registers a thread (BS = 32: 1,024 threads, 64 registers, still
// twice the groups of k_sweep_cc's one 1,024-thread CTA), at most the SM's 32
// CTAs.
constexpr int cc2_min_blocks(int bs) { return bs == 32 ? 2 : 1280 / (bs * 16) < 32 ? 1280 / (bs * 16) : 32; }

// k_sweep_cc with two rows per thread: one CTA of BS/2 warps per group, warp w
// taking rows w and w + BS/2 of every chain (cc_solve2). Half the threads and,
// at up to 48 registers, five CTAs per SM instead of four (BS = 16), so a
// colour with more groups than k_sweep_cc keeps resident runs in one wave
// (the 128^3 system's widest colours have 630-689 groups against 608 resident
// CTAs of k_sweep_cc on 152 SMs). Same prologue, waits and error handling.
template <typename VT, typename XT, int BS, bool UPPER>
__global__ void __launch_bounds__(BS * 16, cc2_min_blocks(BS))
k_sweep_cc2(const WfGroup *__restrict__ groups, int g0, const int2 *__restrict__ chains,
            const unsigned char *__restrict__ counts, const VT *__restrict__ val, const int *__restrict__ col,
            const VT *__restrict__ dinv, const XT *x, XT *y, const int *gate, int *status, int early_x)
{
    static_assert(BS >= 4, "two rows per thread need at least two warps");
    constexpr int W = BS / 2;
    extern __shared__ __align__(128) unsigned char ccs[];
    __shared__ __align__(8) unsigned long long bar;
    __shared__ XT tsh[32][BS + 1];
    __shared__ XT dsh[UPPER ? 32 : 1][BS + 1];
    __shared__ int ibase[32];
    const int g = g0 + blockIdx.x;
    const int w = threadIdx.x >> 5, q = threadIdx.x & 31;
    const WfGroup d = groups[g];
    const int slots = d.emax + d.imax;
    const unsigned cbytes = (unsigned)slots * 32u * 4u, vbytes = (unsigned)slots * 32u * (unsigned)sizeof(VT);
    constexpr unsigned nbytes = 32u * 2u * BS;
    int *cw = reinterpret_cast<int *>(ccs);
    VT *vw = reinterpret_cast<VT *>(ccs + cbytes);
    unsigned char *cnt = ccs + cbytes + vbytes;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_expect_tx(&bar, cbytes + vbytes + nbytes);
        if (slots > 0) {
            bulk_g2s(cw, col + d.off, cbytes, &bar);
            bulk_g2s(vw, val + d.off, vbytes, &bar);
        }
        bulk_g2s(cnt, counts + (size_t)g * nbytes, nbytes, &bar);
    }
    __syncthreads();
    const bool live = q < d.nchains;
    const int2 ch = live ? __ldg(chains + (size_t)g * 32 + q) : make_int2(0, 0);
    const int row0 = ch.x + w, row1 = ch.x + w + W;
    if (UPPER) {
        dsh[q][w] = live ? (XT)__ldg(dinv + row0) : XT(0);
        dsh[q][w + W] = live ? (XT)__ldg(dinv + row1) : XT(0);
    }
    if (w == 0) {  // where each chain's in-chain entries start in the block
        const int I = (int)((unsigned)ch.y >> 16);
        int v = I;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (q >= o) v += u;
        }
        ibase[q] = v - I;
    }
    XT t0 = XT(0), t1 = XT(0);
    bool skip = false;
    if (early_x) {
        if (live) {
            t0 = x[row0];
            t1 = x[row1];
        }
        skip = gated(gate);
    }
    if (!early_x) pdl_launch_dependents();
    pdl_wait();  // the previous colour (or the producer of x) has finished
    if (early_x) pdl_launch_dependents();
    else {
        skip = gated(gate);
        if (live) {
            t0 = x[row0];
            t1 = x[row1];
        }
    }
    const bool ok = mbar_wait_bounded(&bar, 0, kWaitLimit);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(status, 2);
        if (!ok) mbar_wait_bounded(&bar, 0, kWaitLimit);
        return;
    }
    if (skip) return;
    cc_solve2<VT, XT, BS, UPPER>(d, cw, vw, cnt, tsh, dsh, ibase, t0, t1, y, w, q);
    if (live) {
        y[row0] = tsh[q][w];
        y[row1] = tsh[q][w + W];
    }
}

// Resident CTAs per SM that k_sweep_rl is compiled for: one chain per lane as
// k_sweep_cc (2,048 threads), two as k_sweep_cc2 (1,280 threads); with 8-byte
// values a quarter (one chain) or one CTA (two chains) fewer, so that the
// doubles fit the registers without spilling.
constexpr int rl_min_blocks(int bs, int r, int vbytes)
{
    return r == 1 ? (vbytes == 8 && cc_min_blocks(bs) >= 2 ? cc_min_blocks(bs) * 3 / 4 : cc_min_blocks(bs))
                  : (vbytes == 8 && cc2_min_blocks(bs) >= 2 ? cc2_min_blocks(bs) - 1 : cc2_min_blocks(bs));
}

// One colour per launch on the compact chain layout with the external part
// chain-major (make_wf_layout with chain_major), one CTA per group of 32
// chains. Every thread holds row rr = lane % BS of R chains (chain
// w * 32/BS + lane / BS, plus 32/R * r for the r-th), so the lanes of a chain
// are its rows throughout: a chain's x loads and y stores are consecutive
// words, and its rows' gathers of earlier colours fall in a few neighbouring
// chains. Each row subtracts its external entries (the chain's stream at
// qc * emax in the staged block, the rows of one chain in different banks),
// then the chain's in-chain recurrence runs in the same lanes (ChainRec) with
// the row's value already in a register, and each lane stores its row; after
// the staging wait no CTA barrier is needed. R = 2 (BS >= 2) halves the
// threads of a group, for colours with more groups than one wave of R = 1
// holds. Each lane reads its chains' descriptors itself (the chain-major
// layout stores the chain's in-chain offset there) and finds its row's
// offsets by one shuffle scan of the chain's counts. Prologue, programmatic
// launch, early_x and gate as in k_sweep_cc; a staging wait that runs out sets
// *status = 2 and its warp leaves (after a second bounded wait for the copy).
template <typename VT, typename XT, int BS, bool UPPER, int R>
__global__ void __launch_bounds__(BS * 32 / R,
                                  rl_min_blocks(BS, R, (int)(sizeof(VT) > sizeof(XT) ? sizeof(VT) : sizeof(XT))))
k_sweep_rl(const WfGroup *__restrict__ groups, int g0, const int2 *__restrict__ chains,
           const unsigned char *__restrict__ counts, const VT *__restrict__ val, const int *__restrict__ col,
           const VT *__restrict__ dinv, const XT *x, XT *y, const int *gate, int *status, int early_x)
{
    static_assert(R == 1 || (R == 2 && BS >= 2), "two chains per lane need chains of at least two rows");
    constexpr int CPW = 32 / BS;  // chains per warp, per r
    extern __shared__ __align__(128) unsigned char ccs[];
    __shared__ __align__(8) unsigned long long bar;
    const int g = g0 + blockIdx.x;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, rr = lane % BS;
    const WfGroup d = groups[g];
    const int slots = d.emax + d.imax;
    const unsigned cbytes = (unsigned)slots * 32u * 4u, vbytes = (unsigned)slots * 32u * (unsigned)sizeof(VT);
    constexpr unsigned nbytes = 32u * 2u * BS;
    const int *cw = reinterpret_cast<const int *>(ccs);
    const VT *vw = reinterpret_cast<const VT *>(ccs + cbytes);
    const unsigned char *cnt = ccs + cbytes + vbytes;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_expect_tx(&bar, cbytes + vbytes + nbytes);
        if (slots > 0) {
            bulk_g2s(ccs, col + d.off, cbytes, &bar);
            bulk_g2s(ccs + cbytes, val + d.off, vbytes, &bar);
        }
        bulk_g2s(ccs + cbytes + vbytes, counts + (size_t)g * nbytes, nbytes, &bar);
    }
    __syncthreads();
    // each lane reads its chains' descriptors: first row, and where the
    // chain's in-chain entries start in the block (the chain-major layout
    // keeps that offset in the descriptor)
    int qc[R], row[R], ib[R];
    bool live[R];
    XT t[R], di[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        qc[r] = w * CPW + lane / BS + (32 / R) * r;
        const int2 cd = __ldg(chains + (size_t)g * 32 + qc[r]);
        row[r] = cd.x + rr;
        ib[r] = (int)((unsigned)cd.y >> 16);
        live[r] = qc[r] < d.nchains;
        di[r] = UPPER && live[r] ? (XT)__ldg(dinv + row[r]) : XT(1);
        t[r] = XT(0);
    }
    bool skip = false;
    if (early_x) {
#pragma unroll
        for (int r = 0; r < R; r++)
            if (live[r]) t[r] = x[row[r]];
        skip = gated(gate);
    }
    if (!early_x) pdl_launch_dependents();
    pdl_wait();  // the previous colour (or the producer of x) has finished
    if (early_x) pdl_launch_dependents();
    else {
        skip = gated(gate);
#pragma unroll
        for (int r = 0; r < R; r++)
            if (live[r]) t[r] = x[row[r]];
    }
    // each warp leaves together (its lanes shuffle below), and no CTA barrier
    // follows: a warp that saw the staging complete may use the block
    const bool ok = mbar_wait_bounded(&bar, 0, kWaitLimit);
    if (__any_sync(0xffffffffu, !ok)) {
        if (!ok) {
            atomicExch(status, 2);
            mbar_wait_bounded(&bar, 0, kWaitLimit);
        }
        return;
    }
    if (skip) return;
    // the row's external entries (ne, from eo on in the chain's stream) and
    // in-chain entries (left, from at on): the counts of the chain's rows
    // before it (L) or after it (U), one scan of both counts over the chain's
    // lanes (16 bits each)
    int eo[R], ne[R], at[R], left[R], nmax = 0;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const unsigned char *cq = cnt + qc[r] * 2 * BS;
        ne[r] = cq[rr];
        left[r] = cq[BS + rr];
        const int own = ne[r] | (left[r] << 16);
        int v = own;
#pragma unroll
        for (int o = 1; o < BS; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o, BS);
            if (rr >= o) v += u;
        }
        if (UPPER) v = __shfl_sync(0xffffffffu, v, BS - 1, BS) - v;  // rows after this one
        else v -= own;                                                 // rows before it
        eo[r] = v & 0xffff;
        at[r] = v >> 16;
        nmax = max(nmax, ne[r]);
    }
    // external entries, B at a time per chain with all gathers of a batch
    // issued before its first subtraction (R = 1: the second half of a batch
    // only where a lane of the warp needs it); each row's subtractions keep
    // its entries' order
    constexpr int B = R == 1 ? 6 : 3, H = R == 1 ? 3 : B;
    for (int k0 = 0; __any_sync(0xffffffffu, k0 < nmax); k0 += B) {  // warp-uniform
        VT vv[R][B];
        XT yy[R][B];
        const bool more = H == B || __any_sync(0xffffffffu, k0 + H < nmax);
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int u = 0; u < B; u++) {
                if (u >= H && !more) break;
                if (k0 + u < ne[r]) {  // predicated loads, nothing selected
                    const int at = qc[r] * d.emax + eo[r] + k0 + u;
                    vv[r][u] = vw[at];
                    yy[r][u] = __ldg(y + (cw[at] & kColMask));
                }
            }
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int u = 0; u < B; u++) {
                if (u >= H && !more) break;
                if (k0 + u < ne[r]) t[r] -= (XT)vv[r][u] * yy[r][u];
            }
    }
    // in-chain recurrence in the chain's own lanes
    ChainRec<VT, XT, BS, UPPER> a[R];
#pragma unroll
    for (int r = 0; r < R; r++)
        a[r].init_with(cw + d.emax * 32 + ib[r], vw + d.emax * 32 + ib[r], at[r], left[r], rr, t[r], di[r]);
    // the last step's column (L: BS - 1, U: 0) is no row's in-chain entry
#pragma unroll
    for (int s = 0; s < BS - 1; s++)
#pragma unroll
        for (int r = 0; r < R; r++) a[r].step(s);
#pragma unroll
    for (int r = 0; r < R; r++)
        if (live[r]) y[row[r]] = a[r].out();
}

// Colours [cbeg, cend) of one sweep in one cooperative launch, on the
// compact chain layout (all of them, or a run of small colours between
// per-colour launches): CTA b takes groups b, b + gridDim.x, ... of each colour (the group
// body of k_sweep_cc), and a grid barrier separates the colours. Each group's
// block and row counts are staged by TMA into one of two buffers while the
// group before it is solved, across the barrier too (the blocks are read-only).
// Rows of earlier colours were written in this launch, so y (and x, which may
// be y) are read through the coherent path: the acquire at the barrier drops
// L1 lines cached before it.
//
// ctrl = {arrivals, departures, abort}. Barrier k waits for k * gridDim.x
// arrivals. A barrier wait that runs out of polls sets abort and *status = 1, a
// TMA wait that runs out abort and *status = 2; after an abort every CTA stops
// taking groups, waits (bounded) for its copies in flight and leaves, and the
// last CTA to leave resets ctrl for the next launch.
template <typename VT, typename XT, int BS, bool UPPER>
__global__ void __launch_bounds__(BS * 32)
k_sweep_cp(const WfGroup *__restrict__ groups, const int *__restrict__ cgroups, int cbeg, int cend,
           const int2 *__restrict__ chains, const unsigned char *__restrict__ counts, const VT *__restrict__ val,
           const int *__restrict__ col, const VT *__restrict__ dinv, const XT *x, XT *y, const int *gate,
           int *status, int *ctrl, unsigned buf_bytes)
{
    extern __shared__ __align__(128) unsigned char cps[];
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ XT tsh[32][BS + 1];
    __shared__ XT dsh[UPPER ? 32 : 1][BS + 1];
    __shared__ int ibase[32];
    __shared__ int s_ok;
    constexpr unsigned nbytes = 32u * 2u * BS;
    const int l = threadIdx.x >> 5, q = threadIdx.x & 31;
    if (gated(gate)) return;  // every CTA alike, before any control word is touched
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
    }
    __syncthreads();
    auto stage = [&](int g, int k) {  // thread 0: group g's block and counts into buffer k
        const WfGroup d = groups[g];
        const int slots = d.emax + d.imax;
        const unsigned cbytes = (unsigned)slots * 32u * 4u, vbytes = (unsigned)slots * 32u * (unsigned)sizeof(VT);
        unsigned char *b = cps + (size_t)k * buf_bytes;
        // the generic reads of this buffer (two groups back) come before the async writes
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[k], cbytes + vbytes + nbytes);
        if (slots > 0) {
            bulk_g2s(b, col + d.off, cbytes, &bar[k]);
            bulk_g2s(b + cbytes, val + d.off, vbytes, &bar[k]);
        }
        bulk_g2s(b + cbytes + vbytes, counts + (size_t)g * nbytes, nbytes, &bar[k]);
    };
    // this CTA's first group in colour c or a later one (-1: none); its colour in *cc
    auto first_from = [&](int c, int *cc) {
        for (; c < cend; c++) {
            const int g = __ldg(cgroups + c) + (int)blockIdx.x;
            if (g < __ldg(cgroups + c + 1)) {
                *cc = c;
                return g;
            }
        }
        return -1;
    };
    // per buffer b: bit b of ph = parity of its next completion, bit b of pend = a copy in flight
    unsigned ph = 0u, pend = 0u;
    int k = 0, cdummy = 0;
    {
        const int g = first_from(cbeg, &cdummy);
        if (g >= 0) {
            if (threadIdx.x == 0) stage(g, 0);
            pend = 1u;
        }
    }
    bool ok = true;
    for (int c = cbeg; c < cend && ok; c++) {
        const int ge = __ldg(cgroups + c + 1);
        for (int g = __ldg(cgroups + c) + (int)blockIdx.x; g < ge; g += (int)gridDim.x) {
            int cn = c, gn = g + (int)gridDim.x;
            if (gn >= ge) gn = first_from(c + 1, &cn);
            const bool arrived = mbar_wait_bounded(&bar[k], (ph >> k) & 1u, kWaitLimit);
            if (__syncthreads_or(!arrived)) {
                if (threadIdx.x == 0) {
                    atomicExch(status, 2);
                    atomicExch(ctrl + 2, 1);
                }
                ok = false;
                break;
            }
            ph ^= 1u << k;
            pend &= ~(1u << k);
            if (gn >= 0) {
                if (threadIdx.x == 0) stage(gn, k ^ 1);
                pend |= 1u << (k ^ 1);
            }
            const WfGroup d = groups[g];
            const int slots = d.emax + d.imax;
            const unsigned char *b = cps + (size_t)k * buf_bytes;
            const int *cw = reinterpret_cast<const int *>(b);
            const VT *vw = reinterpret_cast<const VT *>(b + (size_t)slots * 32 * 4);
            const unsigned char *cnt = b + (size_t)slots * 32 * (4 + sizeof(VT));
            const bool live = q < d.nchains;
            const int2 ch = live ? __ldg(chains + (size_t)g * 32 + q) : make_int2(0, 0);
            const int row = ch.x + l;
            if (UPPER) dsh[q][l] = live ? (XT)__ldg(dinv + row) : XT(0);
            if (l == 0) {
                const int I = (int)((unsigned)ch.y >> 16);
                int v = I;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(0xffffffffu, v, o);
                    if (q >= o) v += u;
                }
                ibase[q] = v - I;
            }
            const XT t = live ? x[row] : XT(0);
            cc_solve<VT, XT, BS, UPPER, false>(d, cw, vw, cnt, tsh, dsh, ibase, t, y, l, q);
            if (live) y[row] = tsh[q][l];
            k ^= 1;
        }
        if (!ok || c + 1 == cend) break;
        // grid barrier: this CTA's rows of colour c are written (ordered before
        // thread 0's release by the CTA barrier); the acquire that sees the
        // last arrival orders the next colour's reads after every CTA's rows
        __syncthreads();
        if (threadIdx.x == 0) {
            red_release_add(ctrl, 1);
            const int target = (c - cbeg + 1) * (int)gridDim.x;
            int good = 1;
            unsigned polls = 0;
            while (ld_acquire(ctrl) < target) {
                if ((++polls & 63u) == 0 && *(volatile const int *)(ctrl + 2)) {
                    good = 0;
                    break;
                }
                if (polls > 1024u) __nanosleep(32);
                if (polls > kFlagPolls) {
                    atomicExch(ctrl + 2, 1);
                    atomicExch(status, 1);
                    good = 0;
                    break;
                }
            }
            s_ok = good;
        }
        __syncthreads();
        ok = s_ok != 0;
    }
    // copies still in flight (after an abort) land before the CTA leaves
    if (threadIdx.x == 0) {
        for (int b = 0; b < 2; b++)
            if ((pend >> b) & 1u) mbar_wait_bounded(&bar[b], (ph >> b) & 1u, kWaitLimit);
        __threadfence();
        if (atomicAdd(ctrl + 1, 1) == (int)gridDim.x - 1) {
            ctrl[0] = 0;
            ctrl[2] = 0;
            __threadfence();
            atomicExch(ctrl + 1, 0);
        }
    }
    __syncthreads();
}

}  // namespace senkgpu
