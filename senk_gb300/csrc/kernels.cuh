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
            double s = 0;
            if (threadIdx.x < 32) {
                for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) s += part[i];
                s = warp_sum(s);
            }
            if (threadIdx.x == 0) {
                double r = sqrt(s);
                *norm_out = r;
                if (inv_out) *inv_out = 1.0 / r;
            }
        }
    }
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
    A sum = 0;
    int k = 0;
    for (; k + 4 <= w; k += 4) {
        const int i0 = o + k * 32 + r;
        const MT v0 = ld_stream(val + i0), v1 = ld_stream(val + i0 + 32), v2 = ld_stream(val + i0 + 64), v3 = ld_stream(val + i0 + 96);
        const int c0 = ld_stream(col + i0), c1 = ld_stream(col + i0 + 32), c2 = ld_stream(col + i0 + 64), c3 = ld_stream(col + i0 + 96);
        const XT x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
        sum += (A)v0 * (A)x0;
        sum += (A)v1 * (A)x1;
        sum += (A)v2 * (A)x2;
        sum += (A)v3 * (A)x3;
    }
    for (; k < w; k++) {
        const int i0 = o + k * 32 + r;
        sum += (A)ld_stream(val + i0) * (A)__ldg(x + ld_stream(col + i0));
    }
    const long long row = perm ? (long long)__ldg(perm + p) : p;
    if (row < n && row >= 0) y[row] = MODE == 1 ? (XT)((A)b[row] - sum) : (XT)sum;
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
    double acc[CH];
#pragma unroll
    for (int q = 0; q < CH; q++) acc[q] = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double wi = (double)w[i];
#pragma unroll
        for (int q = 0; q < CH; q++)
            if (q < nc) acc[q] += (double)ld_stream(V + (long long)(c0 + q) * ldv + i) * wi;
    }
    __shared__ double sh[CH][kThreads / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < CH; q++) {
        double v = warp_sum(acc[q]);
        if (lane == 0) sh[q][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < CH * 32) {
        const int q = threadIdx.x >> 5;
        double v = lane < (int)(blockDim.x >> 5) ? sh[q][lane] : 0.0;
        v = warp_sum(v);
        if (lane == 0 && q < nc) part[(long long)(c0 + q) * gridDim.x + blockIdx.x] = v;
    }
    const unsigned total = gridDim.x * gridDim.y;
    if (last_cta_arrives(ticket, total)) {
        const int P = gridDim.x;
        for (int k = wid; k < nv; k += blockDim.x >> 5) {
            double s = 0;
            for (int p = lane; p < P; p += 32) s += part[(long long)k * P + p];
            s = warp_sum(s);
            if (lane == 0) {
                coef[k] = s;
                if (hcol) hcol[k] = ACCUM ? hcol[k] + s : s;
            }
        }
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
    __shared__ double sc[64];
    if (threadIdx.x < nv) sc[threadIdx.x] = coef[threadIdx.x];
    __syncthreads();
    double nacc = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = (double)w[i];
        for (int k = 0; k < nv; k++) v -= sc[k] * (double)ld_stream(V + (long long)k * ldv + i);
        const XT vt = (XT)v;
        w[i] = vt;
        nacc += (double)vt * (double)vt;
    }
    __shared__ double sh[32];
    double t = block_sum(nacc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    if (last_cta_arrives(ticket, gridDim.x)) {
        double s = 0;
        if (threadIdx.x < 32) {
            for (int i = threadIdx.x; i < (int)gridDim.x; i += 32) s += part[i];
            s = warp_sum(s);
        }
        if (threadIdx.x == 0) {
            const double hn = sqrt(s);
            if (norm_out) *norm_out = hn;
            if (EPI == kEpiGmres) gmres_givens_step(st, g, hn);
            else st->scale = 1.0 / hn;
        }
    }
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
    __shared__ double sy[64];
    const int J = st->done ? st->jconv : m;
    if (threadIdx.x < J) sy[threadIdx.x] = y[threadIdx.x];
    __syncthreads();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (PRE) {
            double v = sy[0] * (double)V[i];
            for (int k = 1; k < J; k++) v += sy[k] * (double)V[(long long)k * ldv + i];
            V[i] = (XT)v;
        } else {
            double v = (double)x[i];
            for (int k = 0; k < J; k++) v += sy[k] * (double)V[(long long)k * ldv + i];
            x[i] = (XT)v;
        }
    }
}

// --------------------------------------------------------------- ILU sweep

// One slice of the chain-sliced factor layout: up to 32 consecutive schedule
// positions of one colour (whole chains of bsize rows). Entries of slot k of the
// slice's row `lane` sit at off + k*32 + lane; slots [0, we) hold entries whose
// column lies outside the row's chain, slots [we, we+wi) hold in-chain entries
// as chain-local column indices. Unused slots have column -1.
struct SliceDesc {
    int pos0;       // first schedule position
    int off;        // element offset of slot 0 (multiple of 32)
    short nrows;    // rows in this slice (<= 32)
    short we;       // external slots
    short wi;       // in-chain slots
    short pad;
};
static_assert(sizeof(SliceDesc) == 16, "SliceDesc is one 16-byte load");

// Sweep of one colour: L (forward, unit diagonal) or U (backward, inverted
// diagonal in dinv). Each warp solves one slice; the rows of a chain are
// finished in order by broadcasting each finished value to the chain's lanes.
// Per row the subtraction order is the reference's: external entries (columns
// of other, already solved colours) first, then in-chain entries, each in the
// reference's column order (ascending for L, descending for U).
template <typename VT, typename XT, int BS, bool UPPER, bool MAPPED>
__global__ void __launch_bounds__(kThreads)
k_sweep(const SliceDesc *__restrict__ slices, int s_begin, int s_end,
        const VT *__restrict__ val, const int *__restrict__ col, const VT *__restrict__ dinv,
        const int *__restrict__ rowmap, const XT *x, XT *y, const int *gate)
{
    if (gated(gate)) return;
    const int s = s_begin + (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (s >= s_end) return;  // warp-uniform
    const int lane = threadIdx.x & 31;
    const SliceDesc d = slices[s];
    const int pos = d.pos0 + lane;
    const bool live = lane < d.nrows;
    const int row = live ? (MAPPED ? __ldg(rowmap + pos) : pos) : 0;
    XT t = live ? x[row] : XT(0);
    // Phase 1: entries outside the chain (other colours, already final).
    const int *cb = col + d.off + lane;
    const VT *vb = val + d.off + lane;
    int k = 0;
    for (; k + 2 <= d.we; k += 2) {
        const int c0 = ld_stream(cb + k * 32), c1 = ld_stream(cb + (k + 1) * 32);
        const VT v0 = ld_stream(vb + k * 32), v1 = ld_stream(vb + (k + 1) * 32);
        const XT y0 = c0 >= 0 ? y[c0] : XT(0);
        const XT y1 = c1 >= 0 ? y[c1] : XT(0);
        if (c0 >= 0) t -= (XT)v0 * y0;
        if (c1 >= 0) t -= (XT)v1 * y1;
    }
    if (k < d.we) {
        const int c0 = ld_stream(cb + k * 32);
        const VT v0 = ld_stream(vb + k * 32);
        if (c0 >= 0) t -= (XT)v0 * y[c0];
    }
    if (BS > 1) {
        // Phase 2: in-chain entries, column by column in solve order.
        const int r = lane % BS, base = lane - r;
        const int kend = d.we + d.wi;
        int kk = d.we;
        int ic0 = -1, ic1 = -1, ic2 = -1, ic3 = -1;
        VT iv0 = 0, iv1 = 0, iv2 = 0, iv3 = 0;
        if (kk < kend) { ic0 = ld_stream(cb + kk * 32); iv0 = ld_stream(vb + kk * 32); }
        if (kk + 1 < kend) { ic1 = ld_stream(cb + (kk + 1) * 32); iv1 = ld_stream(vb + (kk + 1) * 32); }
        if (kk + 2 < kend) { ic2 = ld_stream(cb + (kk + 2) * 32); iv2 = ld_stream(vb + (kk + 2) * 32); }
        if (kk + 3 < kend) { ic3 = ld_stream(cb + (kk + 3) * 32); iv3 = ld_stream(vb + (kk + 3) * 32); }
        kk += 4;
#pragma unroll
        for (int step = 0; step < BS; step++) {
            const int sc = UPPER ? BS - 1 - step : step;
            if (UPPER && r == sc && live) t *= (XT)__ldg(dinv + pos);
            const XT yv = __shfl_sync(0xffffffffu, t, base + sc);
            if (ic0 == sc) {
                t -= (XT)iv0 * yv;
                ic0 = ic1; iv0 = iv1; ic1 = ic2; iv1 = iv2; ic2 = ic3; iv2 = iv3;
                if (kk < kend) { ic3 = ld_stream(cb + kk * 32); iv3 = ld_stream(vb + kk * 32); }
                else ic3 = -1;
                kk++;
            }
        }
    } else if (UPPER) {
        if (live) t *= (XT)__ldg(dinv + pos);
    }
    if (live) y[row] = t;
}

}  // namespace senkgpu
