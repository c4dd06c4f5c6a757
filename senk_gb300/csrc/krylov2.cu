// GCR(m) and BiCGStab engines on a device-resident system, the ILUB
// preconditioner (BCSR factors) and the drop-in entry points of those solvers.
//
// GCR: one restart cycle (residual test, then m steps) is captured as a CUDA
// graph, like GMRES; the residual is tested only at restart boundaries, as the
// reference does (include/senk_gcr.hpp:93-142). BiCGStab: one iteration is
// captured as a graph and launched in chunks; every kernel after the residual
// test is gated by the device `done` flag, so the iteration count is exact
// (include/senk_bicgstab.hpp:107-176).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>

#include "device.hpp"
#include "dropin_cache.hpp"

namespace senkgpu {

namespace {

constexpr int kBicgChunk = 8;        // BiCGStab iterations launched between host checks
constexpr int kHistCap = 1 << 20;    // most residual-history entries kept on the device

// BiCGStab scalar slots in KrylovState::s
enum { kRrs = 0, kDen = 1, kAlpha = 2, kDsa = 3, kDaa = 4, kOmega = 5, kRrsNew = 6, kNorm = 7 };

template <typename T>
using AccT = typename Acc<T>::type;

__device__ __forceinline__ bool finite(double v) { return v == v && fabs(v) <= 1.7976931348623157e308; }

// GCR restart test (include/senk_gcr.hpp:130-132): stop when ||r|| < eps ||b||.
__global__ void k_gcr_check(KrylovState *st, const double *nrm)
{
    if (threadIdx.x || blockIdx.x) return;
    const double r = *nrm;
    st->res = r / st->nrm_b;
    if (!finite(r)) st->breakdown = 1;
    if (r < st->nrm_b * st->eps || st->breakdown) st->done = 1;
}

// alpha = (Ap_j . r) / (Ap_j . Ap_j); x += alpha p_j; r -= alpha Ap_j
// (include/senk_gcr.hpp:135-138). coef = [Ap_j.Ap_j, Ap_j.r].
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_gcr_step(KrylovState *st, const double *coef, double *dAp_j, T *x, T *r, const T *p, const T *Ap, long long n,
           const int *gate)
{
    if (gated(gate)) return;
    const double d = coef[0];
    const double alpha = coef[1] / d;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *dAp_j = d;
        if (!finite(alpha) || d == 0) st->breakdown = 1;
    }
    const AccT<T> a = (AccT<T>)alpha;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        x[i] = (T)((AccT<T>)x[i] + a * (AccT<T>)p[i]);
        r[i] = (T)((AccT<T>)r[i] + (-a) * (AccT<T>)Ap[i]);
    }
}

// New direction (include/senk_gcr.hpp:139-147): beta_k = -(Ap_k . AKr)/dAp_k;
// p_{j+1} = beta_0 p_0 + Kr + sum_{k>=1} beta_k p_k and the same for Ap_{j+1}.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_gcr_dir(const double *coef, const double *dAp, int j, T *P, T *AP, long long ld, const T *Kr, const T *AKr,
          long long n, const int *gate)
{
    if (gated(gate)) return;
    __shared__ AccT<T> beta[64];
    if (threadIdx.x <= j) beta[threadIdx.x] = (AccT<T>)(-coef[threadIdx.x] / dAp[threadIdx.x]);
    __syncthreads();
    T *pn = P + (long long)(j + 1) * ld, *apn = AP + (long long)(j + 1) * ld;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        AccT<T> pv = beta[0] * (AccT<T>)P[i] + (AccT<T>)Kr[i];
        AccT<T> av = beta[0] * (AccT<T>)AP[i] + (AccT<T>)AKr[i];
        for (int k = 1; k <= j; k++) {
            pv += beta[k] * (AccT<T>)P[(long long)k * ld + i];
            av += beta[k] * (AccT<T>)AP[(long long)k * ld + i];
        }
        pn[i] = (T)pv;
        apn[i] = (T)av;
    }
}

// alpha = (r.r*)/(AKp.r*); s = -alpha AKp + r (include/senk_bicgstab.hpp:140-141)
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_bicg_s(KrylovState *st, const T *r, const T *AKp, T *s, long long n, const int *gate)
{
    if (gated(gate)) return;
    const double alpha = st->s[kRrs] / st->s[kDen];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        st->s[kAlpha] = alpha;
        if (!finite(alpha)) st->breakdown = 1;
    }
    const AccT<T> a = (AccT<T>)(-alpha);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        s[i] = (T)(a * (AccT<T>)AKp[i] + (AccT<T>)r[i]);
}

// omega = (AKs.s)/(AKs.AKs); x += alpha Kp; x += omega Ks; r = -omega AKs + s;
// ||r|| and the stopping test (include/senk_bicgstab.hpp:145-156), in the last CTA.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_bicg_xr(KrylovState *st, T *x, const T *Kp, const T *Ks, const T *AKs, const T *s, T *r, long long n,
          double *part, unsigned *ticket, double *hist, int hist_cap, const int *gate)
{
    if (gated(gate)) return;
    const double omega = st->s[kDsa] / st->s[kDaa];
    const AccT<T> a = (AccT<T>)st->s[kAlpha], w = (AccT<T>)omega;
    double nacc = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        AccT<T> xv = (AccT<T>)x[i] + a * (AccT<T>)Kp[i];
        xv = xv + w * (AccT<T>)Ks[i];
        x[i] = (T)xv;
        const T rv = (T)((-w) * (AccT<T>)AKs[i] + (AccT<T>)s[i]);
        r[i] = rv;
        nacc += (double)rv * (double)rv;
    }
    __shared__ double sh[32];
    const double t = block_sum(nacc, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    if (last_cta_arrives(ticket, gridDim.x)) {
        const double sum = cta_sum_partials(part, gridDim.x, sh);
        if (threadIdx.x == 0) {
            const double nr = sqrt(sum);
            st->s[kOmega] = omega;
            st->s[kNorm] = nr;
            const int it = ++st->count;
            st->res = nr / st->nrm_b;
            if (it <= hist_cap) hist[it - 1] = st->res;
            if (!finite(omega) || !finite(nr)) st->breakdown = 1;
            if (nr < st->eps * st->nrm_b) {
                st->done = 1;
                st->jconv = it;
            } else if (it >= st->maxit || st->breakdown) {
                st->done = 2;
            }
        }
    }
}

// beta = alpha/omega * (r.r*)_new/(r.r*)_old; p = beta (-omega AKp + p) + r
// (include/senk_bicgstab.hpp:157-161). The new r.r* replaces the old one in a
// separate one-thread kernel so that no CTA reads a half-updated scalar.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_bicg_p(const KrylovState *st, T *p, const T *AKp, const T *r, long long n, const int *gate)
{
    if (gated(gate)) return;
    const double alpha = st->s[kAlpha], omega = st->s[kOmega];
    const double beta = alpha / omega * st->s[kRrsNew] / st->s[kRrs];
    const AccT<T> b = (AccT<T>)beta, w = (AccT<T>)(-omega);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const AccT<T> tmp = w * (AccT<T>)AKp[i] + (AccT<T>)p[i];
        p[i] = (T)(b * tmp + (AccT<T>)r[i]);
    }
}

__global__ void k_bicg_roll(KrylovState *st, const int *gate)
{
    if (gated(gate) || threadIdx.x || blockIdx.x) return;
    st->s[kRrs] = st->s[kRrsNew];
}

template <typename T>
void copy_vec(const T *x, T *y, long long n, cudaStream_t s, const int *gate)
{
    k_elementwise<T, 4><<<stream_grid(n, kThreads, 8), kThreads, 0, s>>>(T(0), nullptr, 1.0, T(0), x, y, nullptr, n,
                                                                         gate);
}

template <typename T>
void multidot(System<T> &S, const T *V, long long ldv, int nv, const T *w, double *hcol, const int *gate)
{
    launch_multidot<T, false>(dim3(S.red.ctas, (nv + 7) / 8), S.stream, 
        V, ldv, nv, w, S.n, S.red.part.p, S.red.ticket.p, S.coef.p, hcol, gate);
}


template <typename T>
cudaGraphExec_t capture(System<T> &S, long long *nodes, const std::function<void()> &body)
{
    cudaGraph_t g = nullptr;
    SENK_CUDA(cudaStreamBeginCapture(S.stream, cudaStreamCaptureModeThreadLocal));
    try {
        body();
    } catch (...) {
        cudaStreamEndCapture(S.stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    SENK_CUDA(cudaStreamEndCapture(S.stream, &g));
    size_t nn = 0;
    SENK_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
    *nodes = (long long)nn;
    cudaGraphExec_t ex = nullptr;
    const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    SENK_CUDA(e);
    return ex;
}

}  // namespace

template <typename T>
int System<T>::gcr(double nrm_b, int outer, int m, double eps, senk_result *res)
{
    SENK_REQUIRE(!ir_only, "this system was created for GMRES-IR only (mixed = 2)");
    SENK_REQUIRE(outer >= 0 && m >= 1 && m <= 62, "GCR restart length m must be in [1, 62]");
    if (gcr_m != m) {
        if (gcr_cycle) cudaGraphExecDestroy(gcr_cycle);
        gcr_cycle = nullptr;
        P.alloc((size_t)(m + 2) * n);   // p_0..p_m, Kr
        AP.alloc((size_t)(m + 3) * n);  // Ap_0..Ap_m, r, AKr
        dAp.alloc(64);
        if (!coef.p) coef.alloc(64);
        gcr_m = m;
    }
    const long long ld = n;
    T *r = AP.p + (long long)(m + 1) * ld, *AKr = AP.p + (long long)(m + 2) * ld, *Kr = P.p + (long long)(m + 1) * ld;
    // The learned correction (if attached) is part of the captured cycle; after
    // a fall-back the cycle is captured again without it.
    void *const attached = learned;
    learned_fallback = -1;
    auto recapture_if = [&](bool with_learned) {
        if (gcr_cycle && gcr_learned_in_graph != with_learned) {
            cudaGraphExecDestroy(gcr_cycle);
            gcr_cycle = nullptr;
        }
        learned = with_learned ? attached : nullptr;
        gcr_learned_in_graph = with_learned;
    };
    recapture_if(attached != nullptr);
    const std::function<void()> body = [&] {
            const int *gate = &st.p->done;
            A.residual(x.p, b.p, r, red, &st.p->s[0], nullptr, stream);
            k_gcr_check<<<1, 32, 0, stream>>>(st.p, &st.p->s[0]);
            precondition((const T *)r, P.p, gate);
            A.apply(P.p, AP.p, stream, gate);
            const int grid = stream_grid(n, kThreads, 8);
            for (int j = 0; j < m; j++) {
                T *pj = P.p + (long long)j * ld, *apj = AP.p + (long long)j * ld;
                multidot(*this, (const T *)apj, (long long)(m + 1 - j) * ld, 2, (const T *)apj, nullptr, gate);
                k_gcr_step<T><<<grid, kThreads, 0, stream>>>(st.p, coef.p, dAp.p + j, x.p, r, pj, apj, n, gate);
                precondition((const T *)r, Kr, gate);
                A.apply(Kr, AKr, stream, gate);
                multidot(*this, (const T *)AP.p, ld, j + 1, (const T *)AKr, nullptr, gate);
                k_gcr_dir<T><<<grid, kThreads, 0, stream>>>(coef.p, dAp.p, j, P.p, AP.p, ld, Kr, AKr, n, gate);
            }
            SENK_LAUNCH_CHECK();
    };
    if (!gcr_cycle) gcr_cycle = capture<T>(*this, &gcr_nodes, body);
    KrylovState init{};
    init.nrm_b = nrm_b;
    init.eps = eps;
    *st_host = init;
    SENK_CUDA(cudaMemcpyAsync(st.p, st_host, sizeof(KrylovState), cudaMemcpyHostToDevice, stream));
    SENK_CUDA(cudaEventRecord(ev0, stream));
    int cycles = 0, iters = outer * m, conv = 0;
    double resid = -1, prev = -1;
    for (int i = 0; i < outer; i++) {
        SENK_CUDA(cudaGraphLaunch(gcr_cycle, stream));
        SENK_CUDA(cudaMemcpyAsync(st_host, st.p, sizeof(KrylovState), cudaMemcpyDeviceToHost, stream));
        SENK_CUDA(cudaStreamSynchronize(stream));
        cycles++;
        resid = st_host->res;
        if (opt.verbose) printf("%d %e\n", i * m, resid);  // include/senk_gcr.hpp:131
        if (st_host->done) {
            conv = !st_host->breakdown;
            iters = i * m;
            break;
        }
        // stagnation of the learned preconditioner: the residual measured at
        // this restart did not fall below learned_stall times the previous one
        if (learned && prev > 0 && !(resid < learned_stall * prev)) {
            learned_fallback = i;
            recapture_if(false);
            gcr_cycle = capture<T>(*this, &gcr_nodes, body);
        }
        prev = resid;
    }
    learned = attached;
    SENK_CUDA(cudaEventRecord(ev1, stream));
    SENK_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    SENK_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    check_pc();
    if (opt.verbose) fflush(stdout);
    if (res) {
        res->iters = iters;
        res->converged = conv;
        res->res = resid;
        res->solve_ms = ms;
        res->breakdown = st_host->breakdown;
        res->cycles = cycles;
        res->launches = gcr_nodes * cycles;
    }
    return kOk;
}

template <typename T>
int System<T>::bicgstab(double nrm_b, int max_iter, double eps, senk_result *res)
{
    SENK_REQUIRE(!ir_only, "this system was created for GMRES-IR only (mixed = 2)");
    SENK_REQUIRE(max_iter >= 0, "max_iter must be non-negative");
    const long long ld = n;
    if (!BW.p) {
        BW.alloc((size_t)8 * n);
        if (!coef.p) coef.alloc(64);
    }
    T *r = BW.p, *rs = BW.p + ld, *p = BW.p + 2 * ld, *Kp = BW.p + 3 * ld, *AKp = BW.p + 4 * ld;
    T *s = BW.p + 5 * ld, *AKs = BW.p + 6 * ld, *Ks = BW.p + 7 * ld;
    // The residual history (printed by verbose solves) holds at most kHistCap
    // entries; the captured iteration bakes its address in, so growing it means
    // capturing again.
    const int hist_need = std::max(1, std::min(max_iter, kHistCap));
    if ((long long)hist.n < hist_need) {
        hist.alloc(hist_need);
        if (bicg_step) cudaGraphExecDestroy(bicg_step);
        bicg_step = nullptr;
    }
    const int hist_cap = (int)hist.n;
    if (!bicg_step) {
        bicg_step = capture<T>(*this, &bicg_nodes, [&] {
            const int *gate = &st.p->done;
            const int grid = stream_grid(n, kThreads, 8);
            precondition((const T *)p, Kp, gate);
            A.apply(Kp, AKp, stream, gate);
            multidot(*this, (const T *)AKp, ld, 1, (const T *)rs, &st.p->s[kDen], gate);
            k_bicg_s<T><<<grid, kThreads, 0, stream>>>(st.p, r, AKp, s, n, gate);
            precondition((const T *)s, Ks, gate);
            A.apply(Ks, AKs, stream, gate);
            // [AKs.s, AKs.AKs]: s and AKs are adjacent columns
            multidot(*this, (const T *)s, ld, 2, (const T *)AKs, &st.p->s[kDsa], gate);
            k_bicg_xr<T><<<red.ctas, kThreads, 0, stream>>>(st.p, x.p, Kp, Ks, AKs, s, r, n, red.part.p,
                                                            red.ticket.p, hist.p, hist_cap, gate);
            multidot(*this, (const T *)r, ld, 1, (const T *)rs, &st.p->s[kRrsNew], gate);
            k_bicg_p<T><<<grid, kThreads, 0, stream>>>(st.p, p, AKp, r, n, gate);
            k_bicg_roll<<<1, 32, 0, stream>>>(st.p, gate);
            SENK_LAUNCH_CHECK();
        });
    }
    KrylovState init{};
    init.nrm_b = nrm_b;
    init.eps = eps;
    init.maxit = max_iter;
    init.res = 1.0;  // ||r|| starts as nrm_b (include/senk_bicgstab.hpp:129)
    *st_host = init;
    SENK_CUDA(cudaEventRecord(ev0, stream));
    SENK_CUDA(cudaMemcpyAsync(st.p, st_host, sizeof(KrylovState), cudaMemcpyHostToDevice, stream));
    // r = b - A x; r* = r; p = r; (r.r*) (include/senk_bicgstab.hpp:131-135)
    A.residual(x.p, b.p, r, red, &st.p->s[kNorm], nullptr, stream);
    copy_vec((const T *)r, rs, n, stream, nullptr);
    copy_vec((const T *)r, p, n, stream, nullptr);
    multidot(*this, (const T *)r, ld, 1, (const T *)rs, &st.p->s[kRrs], nullptr);
    SENK_LAUNCH_CHECK();
    long long launched = 0;
    while (launched < max_iter) {
        const int chunk = (int)std::min<long long>(kBicgChunk, max_iter - launched);
        for (int c = 0; c < chunk; c++) SENK_CUDA(cudaGraphLaunch(bicg_step, stream));
        launched += chunk;
        SENK_CUDA(cudaMemcpyAsync(st_host, st.p, sizeof(KrylovState), cudaMemcpyDeviceToHost, stream));
        SENK_CUDA(cudaStreamSynchronize(stream));
        if (st_host->done) break;
    }
    SENK_CUDA(cudaEventRecord(ev1, stream));
    SENK_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    SENK_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    check_pc();
    const int done = st_host->done, count = st_host->count;
    const bool conv = done == 1 && !st_host->breakdown;
    if (opt.verbose) {
        const int shown = std::min(count, (int)hist.n);
        std::vector<double> h(shown);
        if (shown) SENK_CUDA(cudaMemcpy(h.data(), hist.p, sizeof(double) * shown, cudaMemcpyDeviceToHost));
        for (int i = 0; i < shown; i++) printf("%d %e\n", i + 1, h[i]);  // include/senk_bicgstab.hpp:150
        if (conv) printf("# iter %d\n", count);
        else printf("# iter %d (max)\n", count);
        printf("# res %e\n", st_host->res);
        fflush(stdout);
    }
    if (res) {
        res->iters = count;
        res->converged = conv;
        res->res = st_host->res;
        res->solve_ms = ms;
        res->breakdown = st_host->breakdown;
        res->cycles = count;
        res->launches = bicg_nodes * launched + 4;
    }
    return kOk;
}

template int System<double>::gcr(double, int, int, double, senk_result *);
template int System<float>::gcr(double, int, int, double, senk_result *);
template int System<double>::bicgstab(double, int, double, senk_result *);
template int System<float>::bicgstab(double, int, double, senk_result *);

namespace {

template <typename T>
void bcsr_to_csr(const T *bval, const int *bcind, const int *brptr, int N, int bnl, int bnw, std::vector<T> &val,
                 std::vector<int> &cind, std::vector<int> &rptr)
{
    SENK_REQUIRE(bnl > 0 && bnw > 0 && N % bnl == 0 && N % bnw == 0, "N must be a multiple of bnl and bnw");
    const int bs = bnl * bnw;
    rptr.assign(N + 1, 0);
    val.clear();
    cind.clear();
    for (int i = 0; i < N; i++) {  // include/senk_matrix.hpp:213-241
        const int br = i / bnl, r = i % bnl;
        for (int blk = brptr[br]; blk < brptr[br + 1]; blk++)
            for (int c = 0; c < bnw; c++) {
                cind.push_back(bcind[blk] * bnw + c);
                val.push_back(bval[(size_t)blk * bs + c * bnl + r]);
            }
        rptr[i + 1] = (int)val.size();
    }
}

enum Method { kGmres = 0, kGcr = 1, kBicgstab = 2 };

// One drop-in call: upload, solve, copy x back.
template <typename T>
int solve_dropin(const char *fn, Method method, const T *val, const int *cind, const int *rptr, const T *lval,
                 const int *lcind, const int *lrptr, const T *uval, const int *ucind, const int *urptr, int precond,
                 const int *cptr, int cnum, int bsize, const T *b, T *x, double nrm_b, int outer_or_maxit, int m,
                 int N, double eps, const senk_options *opt, senk_result *res, int bnl = 1, int bnw = 1)
{
    SENK_REQUIRE(val && cind && rptr && b && x && N > 0, "null argument");
    senk_system_desc d{};
    d.N = N;
    d.dtype = sizeof(T) == 8 ? SENK_F64 : SENK_F32;
    d.val = val;
    d.cind = cind;
    d.rptr = rptr;
    d.precond = precond;
    d.lval = lval; d.lcind = lcind; d.lrptr = lrptr;
    d.uval = uval; d.ucind = ucind; d.urptr = urptr;
    d.cptr = cptr; d.cnum = cnum; d.bsize = bsize;
    d.m_max = method == kGmres ? m : 0;
    d.bnl = bnl;
    d.bnw = bnw;
    senk_options o{};
    if (opt) o = *opt;
    std::lock_guard<std::mutex> lk(dropin_mutex());
    bool built = false;
    auto sp = dropin_system<T>(fn, d, o, &built);
    System<T> &S = *sp;
    S.b.upload(b, N, S.stream);
    S.x.upload(x, N, S.stream);
    senk_result r{};
    if (method == kGmres) S.gmres(nrm_b, outer_or_maxit, m, eps, &r);
    else if (method == kGcr) S.gcr(nrm_b, outer_or_maxit, m, eps, &r);
    else S.bicgstab(nrm_b, outer_or_maxit, eps, &r);
    SENK_CUDA(cudaMemcpyAsync(x, S.x.p, sizeof(T) * N, cudaMemcpyDeviceToHost, S.stream));
    SENK_CUDA(cudaStreamSynchronize(S.stream));
    r.h2d_bytes = (built ? S.h2d_bytes : 0) + 2LL * sizeof(T) * N;
    r.d2h_bytes = (long long)sizeof(T) * N;
    if (res) *res = r;
    return r.breakdown ? (int)kErrBreakdown : (int)kOk;
}

// ILUB drop-in: the BCSR factors swept as BCSR (IlubPlan).
template <typename T>
int solve_ilub(const char *fn, Method method, const T *val, const int *cind, const int *rptr, const T *blval,
               const int *blcind, const int *blrptr, const T *buval, const int *bucind, const int *burptr,
               const int *cptr, int cnum, int bsize, const T *b, T *x, double nrm_b, int outer_or_maxit, int m, int N,
               double eps, int bnl, int bnw, const senk_options *opt, senk_result *res)
{
    return solve_dropin<T>(fn, method, val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr,
                           cptr ? SENK_PC_ILUB_ABMC : SENK_PC_ILUB, cptr, cnum, bsize, b, x, nrm_b, outer_or_maxit, m,
                           N, eps, opt, res, bnl, bnw);
}

// GMRES(m) on a BCSR matrix: SpmvBcsr (include/senk_sparse.hpp:70-91) sums
// every block entry, zeros included, so the CSR form of all block entries
// gives the same products.
template <typename T>
int bcsr_gmres(const char *fn, const T *bval, const int *bcind, const int *brptr, const T *b, T *x, double nrm_b,
               int outer, int m, int N, double epsilon, int bnl, int bnw, const senk_options *opt, senk_result *res)
{
    std::vector<T> v;
    std::vector<int> c, r;
    bcsr_to_csr(bval, bcind, brptr, N, bnl, bnw, v, c, r);
    return solve_dropin<T>(fn, kGmres, v.data(), c.data(), r.data(), nullptr, nullptr, nullptr, nullptr, nullptr,
                           nullptr, SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

// Block-Jacobi ILU GMRES: the block-Jacobi factors (RemoveOffDiagonal pattern)
// have no entries between blocks; their level sets solve every block's rows in
// the sequential sweep's order, which is what the reference's per-block sweeps
// compute.
template <typename T>
int bj_ilu_gmres(const char *fn, const T *val, const int *cind, const int *rptr, const T *lval, const int *lcind,
                 const int *lrptr, const T *uval, const int *ucind, const int *urptr, int bnum, const T *b, T *x,
                 double nrm_b, int outer, int m, int N, double epsilon, const senk_options *opt, senk_result *res)
{
    SENK_REQUIRE(bnum > 0 && N % bnum == 0, "N must be a multiple of bnum");
    const int bs = N / bnum;
    for (int i = 0; i < N; i++) {
        for (int j = lrptr[i]; j < lrptr[i + 1]; j++)
            SENK_REQUIRE(lcind[j] / bs == i / bs, "L factor couples two Jacobi blocks");
        for (int j = urptr[i]; j < urptr[i + 1]; j++)
            SENK_REQUIRE(ucind[j] / bs == i / bs, "U factor couples two Jacobi blocks");
    }
    return solve_dropin<T>(fn, kGmres, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, SENK_PC_ILU, nullptr,
                           0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

}  // namespace

}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_system_gcr(senk_system *sys, double nrm_b, int outer, int m, double epsilon, senk_result *res)
{
    return guarded("senk_system_gcr", [&] {
        SENK_REQUIRE(sys, "null system");
        senk_result r{};
        if (sys->d) sys->d->gcr(nrm_b, outer, m, epsilon, &r);
        else sys->f->gcr(nrm_b, outer, m, epsilon, &r);
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

int senk_system_bicgstab(senk_system *sys, double nrm_b, int max_iter, double epsilon, senk_result *res)
{
    return guarded("senk_system_bicgstab", [&] {
        SENK_REQUIRE(sys, "null system");
        senk_result r{};
        if (sys->d) sys->d->bicgstab(nrm_b, max_iter, epsilon, &r);
        else sys->f->bicgstab(nrm_b, max_iter, epsilon, &r);
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

int senk_gcr_d(const double *val, const int *cind, const int *rptr, const double *b, double *x, double nrm_b,
               int outer, int m, int N, double epsilon, const senk_options *opt, senk_result *res)
{
    return guarded("senk_gcr_d", [&] {
        return solve_dropin<double>("senk_gcr_d", kGcr, val, cind, rptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                    nullptr, SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
    });
}

int senk_ilu_gcr_d(const double *val, const int *cind, const int *rptr, const double *lval, const int *lcind,
                   const int *lrptr, const double *uval, const int *ucind, const int *urptr, const double *b,
                   double *x, double nrm_b, int outer, int m, int N, double epsilon, const senk_options *opt,
                   senk_result *res)
{
    return guarded("senk_ilu_gcr_d", [&] {
        return solve_dropin<double>("senk_ilu_gcr_d", kGcr, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                    SENK_PC_ILU, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
    });
}

int senk_ilub_gcr_d(const double *val, const int *cind, const int *rptr, const double *blval, const int *blcind,
                    const int *blrptr, const double *buval, const int *bucind, const int *burptr, const double *b,
                    double *x, double nrm_b, int outer, int m, int N, double epsilon, int bnl, int bnw,
                    const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilub_gcr_d", [&] {
        return solve_ilub<double>("senk_ilub_gcr_d", kGcr, val, cind, rptr, blval, blcind, blrptr, buval, bucind,
                                  burptr, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, opt, res);
    });
}

int senk_bicgstab_d(const double *val, const int *cind, const int *rptr, const double *b, double *x, double nrm_b,
                    int max_iter, int N, double epsilon, const senk_options *opt, senk_result *res)
{
    return guarded("senk_bicgstab_d", [&] {
        return solve_dropin<double>("senk_bicgstab_d", kBicgstab, val, cind, rptr, nullptr, nullptr, nullptr, nullptr,
                                    nullptr, nullptr, SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, max_iter, 0, N,
                                    epsilon, opt, res);
    });
}

int senk_ilu_bicgstab_d(const double *val, const int *cind, const int *rptr, const double *lval, const int *lcind,
                        const int *lrptr, const double *uval, const int *ucind, const int *urptr, const double *b,
                        double *x, double nrm_b, int max_iter, int N, double epsilon, const senk_options *opt,
                        senk_result *res)
{
    return guarded("senk_ilu_bicgstab_d", [&] {
        return solve_dropin<double>("senk_ilu_bicgstab_d", kBicgstab, val, cind, rptr, lval, lcind, lrptr, uval,
                                    ucind, urptr, SENK_PC_ILU, nullptr, 0, 0, b, x, nrm_b, max_iter, 0, N, epsilon,
                                    opt, res);
    });
}

int senk_gcr_s(const float *val, const int *cind, const int *rptr, const float *b, float *x, float nrm_b, int outer,
               int m, int N, float epsilon, const senk_options *opt, senk_result *res)
{
    return guarded("senk_gcr_s", [&] {
        return solve_dropin<float>("senk_gcr_s", kGcr, val, cind, rptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                   nullptr, SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
    });
}

int senk_ilu_gcr_s(const float *val, const int *cind, const int *rptr, const float *lval, const int *lcind,
                   const int *lrptr, const float *uval, const int *ucind, const int *urptr, const float *b, float *x,
                   float nrm_b, int outer, int m, int N, float epsilon, const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilu_gcr_s", [&] {
        return solve_dropin<float>("senk_ilu_gcr_s", kGcr, val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                   SENK_PC_ILU, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
    });
}

int senk_bicgstab_s(const float *val, const int *cind, const int *rptr, const float *b, float *x, float nrm_b,
                    int max_iter, int N, float epsilon, const senk_options *opt, senk_result *res)
{
    return guarded("senk_bicgstab_s", [&] {
        return solve_dropin<float>("senk_bicgstab_s", kBicgstab, val, cind, rptr, nullptr, nullptr, nullptr, nullptr,
                                   nullptr, nullptr, SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, max_iter, 0, N, epsilon,
                                   opt, res);
    });
}

int senk_ilu_bicgstab_s(const float *val, const int *cind, const int *rptr, const float *lval, const int *lcind,
                        const int *lrptr, const float *uval, const int *ucind, const int *urptr, const float *b,
                        float *x, float nrm_b, int max_iter, int N, float epsilon, const senk_options *opt,
                        senk_result *res)
{
    return guarded("senk_ilu_bicgstab_s", [&] {
        return solve_dropin<float>("senk_ilu_bicgstab_s", kBicgstab, val, cind, rptr, lval, lcind, lrptr, uval, ucind,
                                   urptr, SENK_PC_ILU, nullptr, 0, 0, b, x, nrm_b, max_iter, 0, N, epsilon, opt, res);
    });
}

int senk_abmc_ilu_bicgstab_d(const double *val, const int *cind, const int *rptr, const double *lval,
                             const int *lcind, const int *lrptr, const double *uval, const int *ucind,
                             const int *urptr, const int *cptr, int cnum, int bsize, const double *b, double *x,
                             double nrm_b, int max_iter, int N, double epsilon, const senk_options *opt,
                             senk_result *res)
{
    return guarded("senk_abmc_ilu_bicgstab_d", [&] {
        return solve_dropin<double>("senk_abmc_ilu_bicgstab_d", kBicgstab, val, cind, rptr, lval, lcind, lrptr, uval,
                                    ucind, urptr, SENK_PC_ILU_ABMC, cptr, cnum, bsize, b, x, nrm_b, max_iter, 0, N,
                                    epsilon, opt, res);
    });
}

int senk_ilub_bicgstab_d(const double *val, const int *cind, const int *rptr, const double *blval,
                         const int *blcind, const int *blrptr, const double *buval, const int *bucind,
                         const int *burptr, const double *b, double *x, double nrm_b, int max_iter, int N,
                         double epsilon, int bnl, int bnw, const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilub_bicgstab_d", [&] {
        return solve_ilub<double>("senk_ilub_bicgstab_d", kBicgstab, val, cind, rptr, blval, blcind, blrptr, buval,
                                  bucind, burptr, nullptr, 0, 0, b, x, nrm_b, max_iter, 0, N, epsilon, bnl, bnw, opt,
                                  res);
    });
}

int senk_ilub_gmres_d(const double *val, const int *cind, const int *rptr, const double *blval, const int *blcind,
                      const int *blrptr, const double *buval, const int *bucind, const int *burptr, const double *b,
                      double *x, double nrm_b, int outer, int m, int N, double epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilub_gmres_d", [&] {
        return solve_ilub<double>("senk_ilub_gmres_d", kGmres, val, cind, rptr, blval, blcind, blrptr, buval, bucind,
                                  burptr, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, opt, res);
    });
}

int senk_abmc_ilub_gmres_d(const double *val, const int *cind, const int *rptr, const double *blval,
                           const int *blcind, const int *blrptr, const double *buval, const int *bucind,
                           const int *burptr, const int *cptr, int cnum, int bsize, const double *b, double *x,
                           double nrm_b, int outer, int m, int N, double epsilon, int bnl, int bnw,
                           const senk_options *opt, senk_result *res)
{
    return guarded("senk_abmc_ilub_gmres_d", [&] {
        SENK_REQUIRE(cptr && cnum > 0, "colour pointer missing");
        return solve_ilub<double>("senk_abmc_ilub_gmres_d", kGmres, val, cind, rptr, blval, blcind, blrptr, buval,
                                  bucind, burptr, cptr, cnum, bsize, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, opt,
                                  res);
    });
}

int senk_bj_ilu_gmres_d(const double *val, const int *cind, const int *rptr, const double *lval, const int *lcind,
                        const int *lrptr, const double *uval, const int *ucind, const int *urptr, int bnum,
                        const double *b, double *x, double nrm_b, int outer, int m, int N, double epsilon,
                        const senk_options *opt, senk_result *res)
{
    return guarded("senk_bj_ilu_gmres_d", [&] {
        return bj_ilu_gmres<double>("senk_bj_ilu_gmres_d", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                    bnum, b, x, nrm_b, outer, m, N, epsilon, opt, res);
    });
}

int senk_bcsr_gmres_d(const double *bval, const int *bcind, const int *brptr, const double *b, double *x,
                      double nrm_b, int outer, int m, int N, double epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res)
{
    return guarded("senk_bcsr_gmres_d", [&] {
        return bcsr_gmres<double>("senk_bcsr_gmres_d", bval, bcind, brptr, b, x, nrm_b, outer, m, N, epsilon, bnl,
                                  bnw, opt, res);
    });
}

// FP32 forms of the block, block-Jacobi and ILUB drop-in solvers
// (include/senk_gmres.hpp:113-117, 487-494, 582-588, 679-686;
// include/senk_gcr.hpp:163-169; include/senk_bicgstab.hpp:198-204 at T = float).
int senk_bcsr_gmres_s(const float *bval, const int *bcind, const int *brptr, const float *b, float *x, float nrm_b,
                      int outer, int m, int N, float epsilon, int bnl, int bnw, const senk_options *opt,
                      senk_result *res)
{
    return guarded("senk_bcsr_gmres_s", [&] {
        return bcsr_gmres<float>("senk_bcsr_gmres_s", bval, bcind, brptr, b, x, nrm_b, outer, m, N, epsilon, bnl,
                                 bnw, opt, res);
    });
}

int senk_bj_ilu_gmres_s(const float *val, const int *cind, const int *rptr, const float *lval, const int *lcind,
                        const int *lrptr, const float *uval, const int *ucind, const int *urptr, int bnum,
                        const float *b, float *x, float nrm_b, int outer, int m, int N, float epsilon,
                        const senk_options *opt, senk_result *res)
{
    return guarded("senk_bj_ilu_gmres_s", [&] {
        return bj_ilu_gmres<float>("senk_bj_ilu_gmres_s", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                   bnum, b, x, nrm_b, outer, m, N, epsilon, opt, res);
    });
}

int senk_ilub_gmres_s(const float *val, const int *cind, const int *rptr, const float *blval, const int *blcind,
                      const int *blrptr, const float *buval, const int *bucind, const int *burptr, const float *b,
                      float *x, float nrm_b, int outer, int m, int N, float epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilub_gmres_s", [&] {
        return solve_ilub<float>("senk_ilub_gmres_s", kGmres, val, cind, rptr, blval, blcind, blrptr, buval, bucind,
                                 burptr, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, opt, res);
    });
}

int senk_abmc_ilub_gmres_s(const float *val, const int *cind, const int *rptr, const float *blval,
                           const int *blcind, const int *blrptr, const float *buval, const int *bucind,
                           const int *burptr, const int *cptr, int cnum, int bsize, const float *b, float *x,
                           float nrm_b, int outer, int m, int N, float epsilon, int bnl, int bnw,
                           const senk_options *opt, senk_result *res)
{
    return guarded("senk_abmc_ilub_gmres_s", [&] {
        SENK_REQUIRE(cptr && cnum > 0, "colour pointer missing");
        return solve_ilub<float>("senk_abmc_ilub_gmres_s", kGmres, val, cind, rptr, blval, blcind, blrptr, buval,
                                 bucind, burptr, cptr, cnum, bsize, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, opt,
                                 res);
    });
}

int senk_ilub_gcr_s(const float *val, const int *cind, const int *rptr, const float *blval, const int *blcind,
                    const int *blrptr, const float *buval, const int *bucind, const int *burptr, const float *b,
                    float *x, float nrm_b, int outer, int m, int N, float epsilon, int bnl, int bnw,
                    const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilub_gcr_s", [&] {
        return solve_ilub<float>("senk_ilub_gcr_s", kGcr, val, cind, rptr, blval, blcind, blrptr, buval, bucind,
                                 burptr, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, opt, res);
    });
}

int senk_ilub_bicgstab_s(const float *val, const int *cind, const int *rptr, const float *blval,
                         const int *blcind, const int *blrptr, const float *buval, const int *bucind,
                         const int *burptr, const float *b, float *x, float nrm_b, int max_iter, int N,
                         float epsilon, int bnl, int bnw, const senk_options *opt, senk_result *res)
{
    return guarded("senk_ilub_bicgstab_s", [&] {
        return solve_ilub<float>("senk_ilub_bicgstab_s", kBicgstab, val, cind, rptr, blval, blcind, blrptr, buval,
                                 bucind, burptr, nullptr, 0, 0, b, x, nrm_b, max_iter, 0, N, epsilon, bnl, bnw, opt,
                                 res);
    });
}

}  // extern "C"
