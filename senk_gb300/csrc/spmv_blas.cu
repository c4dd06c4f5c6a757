// SpMV operators and the single-operation device entry points (SpMV, blas1).
#include <algorithm>
#include <climits>
#include <mutex>

#include "device.hpp"

namespace senkgpu {

int csr_lanes(long long nnz, int n)
{
    const double mean = n > 0 ? (double)nnz / n : 1.0;
    int g = 2;
    while (g < 32 && g < mean) g *= 2;
    return g;
}

namespace {

template <typename MT, typename XT, int MODE>
void spmv_csr_dispatch(const MT *v, const int *c, const int *r, const XT *x, const XT *b, XT *y, int n, int lanes,
                       cudaStream_t s, const int *gate)
{
    if (n <= 0) return;
    const int rows_per_cta_step = kThreads / lanes;
    const int grid = stream_grid(n, rows_per_cta_step, 8);
#define SENK_CSR_CASE(G) \
    case G: k_spmv_csr<MT, XT, G, MODE, false><<<grid, kThreads, 0, s>>>(v, c, r, x, b, y, n, nullptr, nullptr, nullptr, nullptr, gate); break;
    switch (lanes) {
        SENK_CSR_CASE(2) SENK_CSR_CASE(4) SENK_CSR_CASE(8) SENK_CSR_CASE(16) SENK_CSR_CASE(32)
    default: throw ArgError("bad lane count");
    }
#undef SENK_CSR_CASE
    SENK_LAUNCH_CHECK();
}

}  // namespace

void launch_spmv_csr_d(const double *v, const int *c, const int *r, const double *x, const double *b, double *y,
                       int n, int lanes, int mode, cudaStream_t s, const int *gate)
{
    if (mode) spmv_csr_dispatch<double, double, 1>(v, c, r, x, b, y, n, lanes, s, gate);
    else spmv_csr_dispatch<double, double, 0>(v, c, r, x, b, y, n, lanes, s, gate);
}

void launch_spmv_csr_s(const float *v, const int *c, const int *r, const float *x, const float *b, float *y, int n,
                       int lanes, int mode, cudaStream_t s, const int *gate)
{
    if (mode) spmv_csr_dispatch<float, float, 1>(v, c, r, x, b, y, n, lanes, s, gate);
    else spmv_csr_dispatch<float, float, 0>(v, c, r, x, b, y, n, lanes, s, gate);
}

// CSR -> SELL-32 on the device: one warp per slice of 32 rows, lane = slice
// position; slot k of position q's row is element off[slice] + 32 k + lane.
// perm (optional, SELL-32-sigma) maps position -> row (-1 past the last row).
// Padding reads a valid x entry (column 0) times 0. Values are converted to TD.
template <typename TS, typename TD>
__global__ void __launch_bounds__(kThreads)
k_csr_to_sell(const TS *__restrict__ v, const int *__restrict__ c, const int *__restrict__ r,
              const int *__restrict__ off, const int *__restrict__ perm, TD *__restrict__ sv, int *__restrict__ sc,
              int n)
{
    const long long slice = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long q = slice * 32 + lane;
    if (slice * 32 >= n) return;
    const int o = off[slice], w = (off[slice + 1] - o) / 32;
    const long long row = perm ? (long long)perm[q] : (q < n ? q : -1);
    const bool live = row >= 0 && row < n;
    const int b = live ? r[row] : 0, len = live ? r[row + 1] - b : 0;
    for (int k = 0; k < w; k++) {
        const long long at = o + (long long)k * 32 + lane;
        if (k < len) {
            sv[at] = (TD)v[b + k];
            sc[at] = c[b + k];
        } else {
            sv[at] = TD(0);
            sc[at] = live ? (int)row : 0;
        }
    }
}

template <typename TS, typename TD>
__global__ void __launch_bounds__(kThreads) k_cast(const TS *__restrict__ a, TD *__restrict__ b, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (TD)a[i];
}

// Slice offsets of SELL-32 from a host row pointer: slice width = longest row
// of the slice. sigma > 1 (SELL-32-sigma): within each window of sigma rows
// the rows are taken longest first (stable, so equal rows keep their order);
// perm receives position -> row (-1 past the last row, size a multiple of 32).
static std::vector<int> sell_offsets(const int *r, int N, int sigma = 0, std::vector<int> *perm = nullptr)
{
    const int ns = (N + 31) / 32;
    std::vector<int> pos;  // position -> row
    if (sigma > 1) {
        pos.assign((size_t)ns * 32, -1);
        for (int w0 = 0; w0 < N; w0 += sigma) {
            const int w1 = std::min(N, w0 + sigma);
            for (int i = w0; i < w1; i++) pos[i] = i;
            std::stable_sort(pos.begin() + w0, pos.begin() + w1,
                             [&](int a, int b) { return r[a + 1] - r[a] > r[b + 1] - r[b]; });
        }
    }
    std::vector<int> off(ns + 1, 0);
    long long acc = 0;
    for (int i = 0; i < ns; i++) {
        int w = 0;
        const int e = std::min(N, i * 32 + 32);
        for (int q = i * 32; q < e; q++) {
            const int row = pos.empty() ? q : pos[q];
            w = std::max(w, r[row + 1] - r[row]);
        }
        acc += 32LL * w;
        SENK_REQUIRE(acc < INT_MAX, "matrix too large for SELL-32 offsets");
        off[i + 1] = (int)acc;
    }
    if (perm) *perm = std::move(pos);
    return off;
}

template <typename T>
template <typename S>
void SpmvOp<T>::sell_from_device(const S *dv, const int *dc, const int *dr, const std::vector<int> &off,
                                 const std::vector<int> &perm, cudaStream_t s)
{
    sell_off = off;
    sell_perm = perm;
    h2d += (long long)sizeof(int) * (off.size() + perm.size());
    const int ns = (int)off.size() - 1;
    sval.alloc(std::max(off[ns], 1));
    scol.alloc(std::max(off[ns], 1));
    soff.alloc(off.size());
    soff.upload(off.data(), off.size(), s);
    if (!perm.empty()) {
        sperm.alloc(perm.size());
        sperm.upload(perm.data(), perm.size(), s);
    } else {
        sperm.release();
    }
    k_csr_to_sell<S, T><<<ceil_div((long long)ns * 32, kThreads), kThreads, 0, s>>>(
        dv, dc, dr, soff.p, perm.empty() ? nullptr : sperm.p, sval.p, scol.p, n);
    SENK_LAUNCH_CHECK();
    if (!perm.empty()) SENK_CUDA(cudaStreamSynchronize(s));  // the host copy of perm may go away
}

template <typename T>
void SpmvOp<T>::upload(const T *v, const int *c, const int *r, int N, int format, cudaStream_t s, bool keep_csr)
{
    SENK_REQUIRE(N > 0 && v && c && r, "empty or null matrix");
    n = N;
    nnz = r[N];
    SENK_REQUIRE(r[0] == 0 && nnz >= 0, "rptr must start at 0");
    lanes = csr_lanes(nnz, N);
    // The inner SpMV defaults to SELL-32: one thread per row keeps every lane of
    // every FP64 instruction useful (GB300's FP64 pipe, not HBM, limits the
    // CSR-vector kernel). The CSR arrays go up as they are and the SELL copy is
    // built from them on the device.
    use_sell = format == SENK_SPMV_SELL || format == SENK_SPMV_SELL_SIGMA || format == SENK_SPMV_AUTO;
    const int sigma = format == SENK_SPMV_SELL ? 0 : kSellSigma;
    val.alloc(std::max(nnz, 1));
    cind.alloc(std::max(nnz, 1));
    rptr.alloc(N + 1);
    val.upload(v, nnz, s);
    cind.upload(c, nnz, s);
    rptr.upload(r, N + 1, s);
    has_csr = true;
    h2d = (long long)(sizeof(T) + sizeof(int)) * nnz + sizeof(int) * (N + 1LL);
    if (use_sell) {
        std::vector<int> perm;
        const std::vector<int> off = sell_offsets(r, N, sigma, &perm);
        sell_from_device<T>(val.p, cind.p, rptr.p, off, perm, s);
    }
    if (!keep_csr) drop_csr(s);
}

// The same matrix in another precision, converted on the device from `src`,
// which must still hold its CSR arrays.
template <typename T>
template <typename S>
void SpmvOp<T>::convert_from(const SpmvOp<S> &src, int format, cudaStream_t s, bool keep_csr)
{
    SENK_REQUIRE(src.has_csr, "the source operator keeps no CSR copy");
    n = src.n;
    nnz = src.nnz;
    lanes = src.lanes;
    use_sell = format == SENK_SPMV_SELL || format == SENK_SPMV_SELL_SIGMA || format == SENK_SPMV_AUTO;
    if (use_sell) {
        SENK_REQUIRE(!src.sell_off.empty() || !src.use_sell, "source SELL offsets missing");
        std::vector<int> off = src.sell_off, perm = src.sell_perm;
        if (off.empty()) {
            std::vector<int> hr(n + 1);
            SENK_CUDA(cudaMemcpyAsync(hr.data(), src.rptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
            SENK_CUDA(cudaStreamSynchronize(s));
            off = sell_offsets(hr.data(), n, format == SENK_SPMV_SELL ? 0 : kSellSigma, &perm);
        }
        sell_from_device<S>(src.val.p, src.cind.p, src.rptr.p, off, perm, s);
    }
    has_csr = keep_csr || !use_sell;
    if (has_csr) {
        val.alloc(std::max(nnz, 1));
        cind.alloc(std::max(nnz, 1));
        rptr.alloc(n + 1);
        k_cast<S, T><<<stream_grid(nnz, kThreads, 8), kThreads, 0, s>>>(src.val.p, val.p, nnz);
        SENK_CUDA(cudaMemcpyAsync(cind.p, src.cind.p, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, s));
        SENK_CUDA(cudaMemcpyAsync(rptr.p, src.rptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, s));
        SENK_LAUNCH_CHECK();
    }
}

template <typename T>
void SpmvOp<T>::drop_csr(cudaStream_t s)
{
    if (!use_sell || !has_csr) return;
    SENK_CUDA(cudaStreamSynchronize(s));  // the SELL build may still read them
    val.release();
    cind.release();
    rptr.release();
    has_csr = false;
}

template void SpmvOp<float>::convert_from<double>(const SpmvOp<double> &, int, cudaStream_t, bool);
template void SpmvOp<double>::convert_from<double>(const SpmvOp<double> &, int, cudaStream_t, bool);

template <typename T>
void SpmvOp<T>::apply(const T *x, T *y, cudaStream_t s, const int *gate) const
{
    if (use_sell) {
        const long long nthreads = ((long long)n + 31) / 32 * 32;
        k_spmv_sell32<T, T, 0><<<ceil_div(nthreads, kThreads), kThreads, 0, s>>>(
            sval.p, scol.p, soff.p, sell_perm.empty() ? nullptr : sperm.p, x, nullptr, y, n, gate);
        SENK_LAUNCH_CHECK();
        return;
    }
    spmv_csr_dispatch<T, T, 0>(val.p, cind.p, rptr.p, x, nullptr, y, n, lanes, s, gate);
}

template <typename T>
void SpmvOp<T>::residual(const T *x, const T *b, T *y, ReduceScratch &red, double *norm_out, double *inv_out,
                         cudaStream_t s) const
{
    red.ensure(s);
    if (use_sell) {
        const int grid = ceil_div(n, kThreads);
        SENK_REQUIRE(grid <= red.ctas * ReduceScratch::kMaxCols, "N too large for the reduction scratch");
        k_residual_sell32<T><<<grid, kThreads, 0, s>>>(sval.p, scol.p, soff.p, sell_perm.empty() ? nullptr : sperm.p,
                                                       x, b, y, n, red.part.p, red.ticket.p,
                                                       norm_out, inv_out);
        SENK_LAUNCH_CHECK();
        return;
    }
    const int grid = std::min(stream_grid(n, kThreads / lanes, 8), red.ctas * ReduceScratch::kMaxCols);
#define SENK_RES_CASE(G) \
    case G: k_spmv_csr<T, T, G, 1, true><<<grid, kThreads, 0, s>>>(val.p, cind.p, rptr.p, x, b, y, n, red.part.p, red.ticket.p, norm_out, inv_out, nullptr); break;
    switch (lanes) {
        SENK_RES_CASE(2) SENK_RES_CASE(4) SENK_RES_CASE(8) SENK_RES_CASE(16) SENK_RES_CASE(32)
    default: throw ArgError("bad lane count");
    }
#undef SENK_RES_CASE
    SENK_LAUNCH_CHECK();
}

template struct SpmvOp<double>;
template struct SpmvOp<float>;

// Scratch for the one-shot reductions of the device entry points, per device.
namespace {
std::mutex g_red_mu;
ReduceScratch g_red[64];
DevBuf<double> g_red_out[64];

template <typename T, int OP>
void elementwise(T a, T b, const T *x, T *y, T *z, int n, cudaStream_t s)
{
    if (n <= 0) return;
    k_elementwise<T, OP><<<stream_grid(n, kThreads, 8), kThreads, 0, s>>>(a, nullptr, 1.0, b, x, y, z, n, nullptr);
    SENK_LAUNCH_CHECK();
}
}  // namespace

}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_dev_spmv_csr_d(const double *val, const int *cind, const int *rptr, const double *x, double *y, int N,
                        int nnz, void *stream)
{
    return guarded("senk_dev_spmv_csr_d", [&] {
        SENK_REQUIRE(N >= 0 && nnz >= 0, "negative size");
        launch_spmv_csr_d(val, cind, rptr, x, nullptr, y, N, csr_lanes(nnz, N), 0, (cudaStream_t)stream, nullptr);
        return (int)kOk;
    });
}

int senk_dev_spmv_csr_s(const float *val, const int *cind, const int *rptr, const float *x, float *y, int N,
                        int nnz, void *stream)
{
    return guarded("senk_dev_spmv_csr_s", [&] {
        SENK_REQUIRE(N >= 0 && nnz >= 0, "negative size");
        launch_spmv_csr_s(val, cind, rptr, x, nullptr, y, N, csr_lanes(nnz, N), 0, (cudaStream_t)stream, nullptr);
        return (int)kOk;
    });
}

int senk_dev_spmv_csr_diag_d(const double *val, const int *cind, const int *rptr, const double *diag,
                             const double *x, double *y, int N, void *stream)
{
    return guarded("senk_dev_spmv_csr_diag_d", [&] {
        if (N <= 0) return (int)kOk;
        k_spmv_csr_diag<double><<<ceil_div(N, kThreads), kThreads, 0, (cudaStream_t)stream>>>(val, cind, rptr, diag,
                                                                                             x, y, N);
        SENK_LAUNCH_CHECK();
        return (int)kOk;
    });
}

int senk_dev_spmv_bcsr_d(const double *bval, const int *bcind, const int *brptr, const double *x, double *y, int N,
                         int bnl, int bnw, void *stream)
{
    return guarded("senk_dev_spmv_bcsr_d", [&] {
        SENK_REQUIRE(bnl > 0 && bnw > 0 && N % bnl == 0, "N must be a multiple of bnl");
        const int nb = N / bnl;
        if (nb == 0) return (int)kOk;
        cudaStream_t s = (cudaStream_t)stream;
        const int grid = ceil_div(nb, kThreads);
#define SENK_BCSR_CASE(R, C) \
        if (bnl == R && bnw == C) { k_spmv_bcsr<double, double, R, C, 0><<<grid, kThreads, 0, s>>>(bval, bcind, brptr, x, nullptr, y, nb, nullptr); SENK_LAUNCH_CHECK(); return (int)kOk; }
        SENK_BCSR_CASE(1, 1) SENK_BCSR_CASE(2, 1) SENK_BCSR_CASE(2, 2) SENK_BCSR_CASE(3, 3)
        SENK_BCSR_CASE(4, 1) SENK_BCSR_CASE(4, 4) SENK_BCSR_CASE(8, 1)
#undef SENK_BCSR_CASE
        throw ArgError("unsupported BCSR block shape " + std::to_string(bnl) + "x" + std::to_string(bnw));
    });
}

int senk_dev_spmv_sell_d(const double *val, const int *cind, const int *wid, int len, const double *x, double *y,
                         int N, void *stream)
{
    return guarded("senk_dev_spmv_sell_d", [&] {
        SENK_REQUIRE(len > 0, "slice length must be positive");
        if (N <= 0) return (int)kOk;
        k_spmv_sell_ref<double><<<ceil_div(N, kThreads), kThreads, 0, (cudaStream_t)stream>>>(val, cind, wid, len, x,
                                                                                             y, N);
        SENK_LAUNCH_CHECK();
        return (int)kOk;
    });
}

static int dev_reduce(const char *fn, const double *x, const double *y, int N, double *result, bool norm,
                      void *stream)
{
    return guarded(fn, [&] {
        SENK_REQUIRE(result != nullptr && N >= 0, "bad argument");
        if (N == 0) { *result = 0; return (int)kOk; }
        int dev = 0;
        SENK_CUDA(cudaGetDevice(&dev));
        SENK_REQUIRE(dev < 64, "device index out of range");
        cudaStream_t s = (cudaStream_t)stream;
        std::lock_guard<std::mutex> lk(g_red_mu);
        g_red[dev].ensure(s);
        if (!g_red_out[dev].p) g_red_out[dev].alloc(1);
        const int grid = stream_grid(N, kThreads, 2);
        k_multidot<double, false><<<dim3(grid, 1), kThreads, 0, s>>>(x, 0, 1, y, N, g_red[dev].part.p,
                                                                     g_red[dev].ticket.p, g_red_out[dev].p, nullptr,
                                                                     nullptr);
        SENK_LAUNCH_CHECK();
        double h = 0;
        SENK_CUDA(cudaMemcpyAsync(&h, g_red_out[dev].p, sizeof(double), cudaMemcpyDeviceToHost, s));
        SENK_CUDA(cudaStreamSynchronize(s));
        *result = norm ? sqrt(h) : h;
        return (int)kOk;
    });
}

int senk_dev_dot_d(const double *x, const double *y, int N, double *result, void *stream)
{
    return dev_reduce("senk_dev_dot_d", x, y, N, result, false, stream);
}

int senk_dev_nrm2_d(const double *x, int N, double *result, void *stream)
{
    return dev_reduce("senk_dev_nrm2_d", x, x, N, result, true, stream);
}

int senk_dev_axpy_d(double a, const double *x, double *y, int N, void *stream)
{
    return guarded("senk_dev_axpy_d", [&] { elementwise<double, 0>(a, 0.0, x, y, nullptr, N, (cudaStream_t)stream); return (int)kOk; });
}
int senk_dev_axpby_d(double a, const double *x, double b, double *y, int N, void *stream)
{
    return guarded("senk_dev_axpby_d", [&] { elementwise<double, 1>(a, b, x, y, nullptr, N, (cudaStream_t)stream); return (int)kOk; });
}
int senk_dev_axpyz_d(double a, const double *x, const double *y, double *z, int N, void *stream)
{
    return guarded("senk_dev_axpyz_d", [&] { elementwise<double, 2>(a, 0.0, x, (double *)y, z, N, (cudaStream_t)stream); return (int)kOk; });
}
int senk_dev_scal_d(double a, double *x, int N, void *stream)
{
    return guarded("senk_dev_scal_d", [&] { elementwise<double, 3>(a, 0.0, nullptr, x, nullptr, N, (cudaStream_t)stream); return (int)kOk; });
}
int senk_dev_copy_d(const double *x, double *y, int N, void *stream)
{
    return guarded("senk_dev_copy_d", [&] { elementwise<double, 4>(0.0, 0.0, x, y, nullptr, N, (cudaStream_t)stream); return (int)kOk; });
}

}  // extern "C"
