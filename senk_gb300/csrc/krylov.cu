// Krylov engines on a device-resident system. One restart cycle of GMRES(m) is
// captured once as a CUDA graph; every inner-iteration kernel is gated by the
// device `done` flag so the iteration count is exact without a host round trip
// per iteration. The host synchronises once per cycle.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include <chrono>
#include <functional>

#include "device.hpp"
#include "dropin_cache.hpp"

namespace senkgpu {

namespace {

// Wall-clock trace of host-side phases, printed to stderr when verbose >= 2.
struct PhaseClock {
    bool on;
    const char *who;
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    void lap(const char *what)
    {
        if (!on) return;
        const auto n = std::chrono::steady_clock::now();
        std::fprintf(stderr, "# setup %s %s %.2f ms\n", who, what,
                     std::chrono::duration<double, std::milli>(n - t).count());
        t = n;
    }
};

}  // namespace


namespace {


template <typename T, int OP>
void ew(const T *x, T *y, T *z, long long n, T a, T b, const double *a_dev, double a_mul, cudaStream_t s,
        const int *gate)
{
    k_elementwise<T, OP><<<stream_grid(n, kThreads, 8), kThreads, 0, s>>>(a, a_dev, a_mul, b, x, y, z, n, gate);
}

}  // namespace

template <typename T>
System<T>::~System()
{
    inner.reset();
    if (cycle) cudaGraphExecDestroy(cycle);
    if (gcr_cycle) cudaGraphExecDestroy(gcr_cycle);
    if (bicg_step) cudaGraphExecDestroy(bicg_step);
    if (st_host) cudaFreeHost(st_host);
    if (ir_host) cudaFreeHost(ir_host);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream && own_stream) cudaStreamDestroy(stream);
}

template <typename T>
void System<T>::create(const senk_system_desc &d, const senk_options *o, cudaStream_t shared, bool sell_only,
                       const SpmvOp<double> *csr_src)
{
    SENK_REQUIRE(d.N > 0, "N must be positive");
    SENK_REQUIRE(d.mixed >= 0 && d.mixed <= 2, "mixed must be 0, 1 or 2");
    n = d.N;
    ir_only = d.mixed == 2;
    if (o) opt = *o;
    PhaseClock clk{opt.verbose >= 2, sizeof(T) == 8 ? "fp64" : "fp32"};
    if (shared) {
        stream = shared;
        own_stream = false;
    } else {
        SENK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    }
    SENK_CUDA(cudaEventCreate(&ev0));
    SENK_CUDA(cudaEventCreate(&ev1));
    SENK_CUDA(cudaMallocHost((void **)&st_host, sizeof(KrylovState)));
    clk.lap("stream+events");
    // GMRES-IR only: the FP64 system computes residuals and updates x; the
    // preconditioner and the Krylov basis live in the FP32 copy.
    if (csr_src) {
        // FP32 copy of an FP64 system: converted on the device
        A.convert_from(*csr_src, opt.spmv, stream, !sell_only);
    } else {
        // an FP32 copy still needs the CSR arrays (dropped once it is built)
        A.upload((const T *)d.val, d.cind, d.rptr, n, opt.spmv, stream, !(sell_only || ir_only) || d.mixed);
    }
    clk.lap("A upload (+SELL build)");
    if (ir_only) {
        // nothing to build here for the preconditioner
    } else if (d.precond == SENK_PC_ILUB || d.precond == SENK_PC_ILUB_ABMC) {
        SENK_REQUIRE((d.precond == SENK_PC_ILUB_ABMC) == (d.cptr != nullptr),
                     "SENK_PC_ILUB_ABMC needs cptr; SENK_PC_ILUB takes none");
        pcb = std::make_unique<IlubPlan<T>>();
        pcb->build(n, d.bnl, d.bnw, (const T *)d.lval, d.lcind, d.lrptr, (const T *)d.uval, d.ucind, d.urptr, d.cptr,
                   d.cnum, d.bsize, stream);
    } else if (d.precond != SENK_PC_NONE) {
        pc = std::make_unique<IluPlan<T>>();
        pc->build(n, (const T *)d.lval, d.lcind, d.lrptr, (const T *)d.uval, d.ucind, d.urptr, d.precond, d.cptr,
                  d.cnum, d.bsize, stream, opt.sweep);
    }
    clk.lap("preconditioner plan");
    b.alloc(n);
    x.alloc(n);
    t.alloc(n);
    SENK_CUDA(cudaMemsetAsync(b.p, 0, b.bytes(), stream));
    SENK_CUDA(cudaMemsetAsync(x.p, 0, x.bytes(), stream));
    st.alloc(1);
    red.ensure(stream);
    if (d.m_max > 0 && !ir_only) ensure_gmres(d.m_max);
    SENK_CUDA(cudaStreamSynchronize(stream));
    clk.lap("vectors + Krylov workspace");
    h2d_bytes = A.h2d;
    if (pcb) h2d_bytes += pcb->h2d_bytes();
    if (pc) {
        for (const SweepFactor<T> *F : {&pc->L, &pc->U})
            h2d_bytes += (long long)(F->val.bytes() + F->col.bytes() + F->dinv.bytes() + F->rowmap.bytes() +
                                     F->groups.bytes() + F->widths.bytes());
    }
    if (d.mixed) {
        SENK_REQUIRE(sizeof(T) == sizeof(double), "mixed precision needs an FP64 system");
        // FP32 copies of A and the factors, as senk::utils::Convert makes them
        // (include/senk_utils.hpp:103-110).
        auto demote = [](const void *src, int cnt) {
            std::vector<float> v(cnt);
            const double *p = static_cast<const double *>(src);
#pragma omp parallel for schedule(static)
            for (int i = 0; i < cnt; i++) v[i] = (float)p[i];
            return v;
        };
        std::vector<float> l32, u32;
        senk_system_desc di = d;
        di.dtype = SENK_F32;
        di.mixed = 0;
        di.val = nullptr;  // A comes from this system's device copy
        if (d.precond == SENK_PC_ILUB || d.precond == SENK_PC_ILUB_ABMC) {
            // BCSR factors: block row pointers of N / bnl block rows
            SENK_REQUIRE(d.bnl > 0 && d.bnw > 0 && n % d.bnl == 0, "bad ILUB block shape");
            const int nbr = n / d.bnl, bsz = d.bnl * d.bnw;
            l32 = demote(d.lval, d.lrptr[nbr] * bsz);
            u32 = demote(d.uval, d.urptr[nbr] * bsz);
            di.lval = l32.data();
            di.uval = u32.data();
        } else if (d.precond != SENK_PC_NONE) {
            l32 = demote(d.lval, d.lrptr[n]);
            u32 = demote(d.uval, d.urptr[n]);
            di.lval = l32.data();
            di.uval = u32.data();
        }
        clk.lap("demote factors");
        inner = std::make_unique<System<float>>();
        if constexpr (std::is_same<T, double>::value) inner->create(di, &opt, stream, ir_only, &A);
        if (ir_only) A.drop_csr(stream);
        clk.lap("FP32 system");
        h2d_bytes += inner->h2d_bytes;
        irs.alloc(2);
        SENK_CUDA(cudaMallocHost((void **)&ir_host, 2 * sizeof(double)));
    }
}

template <typename T>
void System<T>::ensure_gmres(int m)
{
    SENK_REQUIRE(m >= 1 && m <= 63, "restart length m must be in [1, 63]");
    if (m <= m_alloc) return;
    V.alloc((size_t)(m + 1) * n);
    H.alloc((size_t)(m + 1) * m);
    cs.alloc(m);
    sn.alloc(m);
    e.alloc(m + 1);
    y.alloc(m);
    coef.alloc(64);
    m_alloc = m;
    if (cycle) {
        cudaGraphExecDestroy(cycle);
        cycle = nullptr;
        cycle_m = -1;
    }
}

// Arnoldi step j: w = V_{j+1} against V_0..V_j, H column j, Givens, test.
template <typename T>
static void enqueue_orth(System<T> &S, int j, int m, int orth, const int *gate)
{
    const long long ld = S.n;
    T *w = S.V.p + (long long)(j + 1) * ld;
    double *hcol = S.H.p + (long long)j * (m + 1);
    GmresEpi g{S.H.p, S.cs.p, S.sn.p, S.e.p, j, m};
    GmresEpi none{};
    const int nv = j + 1;
    const int kRedCtas = S.red.ctas;  // CTAs of the multi-dot / update kernels
    const dim3 gdot(kRedCtas, (nv + 7) / 8);
    cudaStream_t s = S.stream;
    if (orth == SENK_ORTH_MGS) {
        for (int k = 0; k <= j; k++) {
            const T *vk = S.V.p + (long long)k * ld;
            launch_multidot<T, false>(dim3(kRedCtas, 1), s, vk, ld, 1, w, ld, S.red.part.p,
                                                                         S.red.ticket.p, S.coef.p, hcol + k, gate);
            if (k == j)
                launch_update<T, kEpiGmres>(kRedCtas, s, vk, ld, 1, S.coef.p, w, ld, S.red.part.p,
                                                                     S.red.ticket.p, nullptr, S.st.p, g, gate);
            else
                launch_update<T, kEpiNone>(kRedCtas, s, vk, ld, 1, S.coef.p, w, ld, S.red.part.p,
                                                                    S.red.ticket.p, nullptr, S.st.p, none, gate);
        }
        return;
    }
    launch_multidot<T, false>(gdot, s, S.V.p, ld, nv, w, ld, S.red.part.p, S.red.ticket.p, S.coef.p,
                                                   hcol, gate);
    if (orth == SENK_ORTH_CGS) {
        launch_update<T, kEpiGmres>(kRedCtas, s, S.V.p, ld, nv, S.coef.p, w, ld, S.red.part.p,
                                                             S.red.ticket.p, nullptr, S.st.p, g, gate);
        return;
    }
    // CGS2: second pass corrects the coefficients (H += correction).
    launch_update<T, kEpiNone>(kRedCtas, s, S.V.p, ld, nv, S.coef.p, w, ld, S.red.part.p,
                                                        S.red.ticket.p, nullptr, S.st.p, none, gate);
    launch_multidot<T, true>(gdot, s, S.V.p, ld, nv, w, ld, S.red.part.p, S.red.ticket.p, S.coef.p,
                                                  hcol, gate);
    launch_update<T, kEpiGmres>(kRedCtas, s, S.V.p, ld, nv, S.coef.p, w, ld, S.red.part.p,
                                                         S.red.ticket.p, nullptr, S.st.p, g, gate);
}

// One restart cycle (include/senk_gmres.hpp:214-257, and :47-84 without a
// preconditioner), every kernel on S.stream.
template <typename T>
void System<T>::enqueue_gmres_cycle(int m)
{
    const int *gate = &st.p->done;
    const long long ld = n;
    // r0 = b - A x, e0 = ||r0||, V0 = r0 / e0
    A.residual(x.p, b.p, V.p, red, e.p, &st.p->scale, stream);
    ew<T, 3>(nullptr, V.p, nullptr, n, T(0), T(0), &st.p->scale, 1.0, stream, nullptr);
    for (int j = 0; j < m; j++) {
        T *vj = V.p + (long long)j * ld;
        T *w = V.p + (long long)(j + 1) * ld;
        if (has_pc()) {
            precondition(vj, t.p, gate);
            A.apply(t.p, w, stream, gate);
        } else {
            A.apply(vj, w, stream, gate);
        }
        enqueue_orth(*this, j, m, opt.orth, gate);
        ew<T, 3>(nullptr, w, nullptr, n, T(0), T(0), &st.p->scale, 1.0, stream, gate);
    }
    k_gmres_trsv<<<1, 32, 0, stream>>>(st.p, H.p, e.p, y.p, m);
    const int grid = stream_grid(n, kThreads, 8);
    if (has_pc()) {
        k_gmres_combine<T, true><<<grid, kThreads, 0, stream>>>(V.p, ld, y.p, st.p, x.p, n, m);
        precondition(V.p, t.p, nullptr);
        ew<T, 0>(t.p, x.p, nullptr, n, T(1), T(0), nullptr, 1.0, stream, nullptr);
    } else {
        k_gmres_combine<T, false><<<grid, kThreads, 0, stream>>>(V.p, ld, y.p, st.p, x.p, n, m);
    }
    SENK_LAUNCH_CHECK();
}

template <typename T>
int System<T>::gmres(double nrm_b, int outer, int m, double eps, senk_result *res)
{
    SENK_REQUIRE(!ir_only, "this system was created for GMRES-IR only (mixed = 2)");
    SENK_REQUIRE(outer >= 0, "outer must be non-negative");
    ensure_gmres(m);
    const int orth = opt.orth;
    SENK_REQUIRE(orth == SENK_ORTH_CGS2 || orth == SENK_ORTH_CGS || orth == SENK_ORTH_MGS, "unknown orthogonalisation");
    if (!cycle || cycle_m != m || cycle_orth != orth) {
        PhaseClock clk{opt.verbose >= 2, sizeof(T) == 8 ? "fp64" : "fp32"};
        if (cycle) cudaGraphExecDestroy(cycle);
        cycle = nullptr;
        cudaGraph_t g;
        SENK_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_gmres_cycle(m);
        } catch (...) {
            cudaStreamEndCapture(stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        SENK_CUDA(cudaStreamEndCapture(stream, &g));
        clk.lap("GMRES cycle capture");
        size_t nodes = 0;
        SENK_CUDA(cudaGraphGetNodes(g, nullptr, &nodes));
        cycle_nodes = (long long)nodes;
        cudaError_t ie = cudaGraphInstantiate(&cycle, g, 0);
        cudaGraphDestroy(g);
        SENK_CUDA(ie);
        clk.lap("GMRES cycle instantiate");
        cycle_m = m;
        cycle_orth = orth;
    }
    KrylovState init{};
    init.nrm_b = nrm_b;
    init.eps = eps;
    *st_host = init;
    SENK_CUDA(cudaMemcpyAsync(st.p, st_host, sizeof(KrylovState), cudaMemcpyHostToDevice, stream));
    SENK_CUDA(cudaEventRecord(ev0, stream));
    int cycles = 0, iters = outer * m, conv = 0;
    double resid = -1;
    for (int i = 0; i < outer; i++) {
        SENK_CUDA(cudaGraphLaunch(cycle, stream));
        SENK_CUDA(cudaMemcpyAsync(st_host, st.p, sizeof(KrylovState), cudaMemcpyDeviceToHost, stream));
        SENK_CUDA(cudaStreamSynchronize(stream));
        cycles++;
        if (st_host->done) {
            conv = 1;
            iters = i * m + st_host->jconv;
            resid = st_host->res;
            break;
        }
    }
    SENK_CUDA(cudaEventRecord(ev1, stream));
    SENK_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    SENK_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    check_pc();
    if (opt.verbose) {
        if (conv) {
            printf("I iter %d\n", iters);
            printf("# res %e\n", resid);
        } else {
            printf("# iter %d\n", outer * m);
            printf("# res : Check by using senk::test\n");
        }
        fflush(stdout);
    }
    if (res) {
        res->iters = iters;
        res->converged = conv;
        res->res = resid;
        res->solve_ms = ms;
        res->breakdown = st_host->breakdown;
        res->cycles = cycles;
        res->launches = cycle_nodes * cycles;
    }
    return kOk;
}

template <typename T>
void System<T>::time_op(int op, int reps, double *ms_out, long long *bytes_out)
{
    SENK_REQUIRE(op == SENK_OP_SPMV || op == SENK_OP_DOT || op == SENK_OP_MULTIDOT || op == SENK_OP_UPDATE ||
                     has_pc(),
                 "system has no preconditioner");
    constexpr int kBasis = 16;  // columns of the Arnoldi-step ops (the middle of a GMRES(30) cycle)
    ensure_gmres(std::max(m_alloc, (op == SENK_OP_MULTIDOT || op == SENK_OP_UPDATE) ? kBasis : 1));
    T *v0 = V.p, *v1 = V.p + n;
    const long long vb = sizeof(T);
    long long bytes = 0;
    auto run = [&]() {
        switch (op) {
        case SENK_OP_SPMV: A.apply(v0, v1, stream, nullptr); break;
        case SENK_OP_PRECOND: SENK_REQUIRE(has_pc(), "system has no preconditioner"); precondition(v0, t.p, nullptr); break;
        case SENK_OP_SWEEP_L:
            if (pcb) pcb->sweep(false, v0, t.p, stream, nullptr);
            else pc->sweep(pc->L, v0, t.p, stream, nullptr);
            break;
        case SENK_OP_SWEEP_U:
            if (pcb) pcb->sweep(true, (const T *)t.p, t.p, stream, nullptr);
            else pc->sweep(pc->U, (const T *)t.p, t.p, stream, nullptr);
            break;
        case SENK_OP_DOT:
            launch_multidot<T, false>(dim3(red.ctas, 1), stream, v0, n, 1, v1, n, red.part.p, red.ticket.p, coef.p, nullptr, nullptr);
            break;
        case SENK_OP_MULTIDOT:
            launch_multidot<T, false>(dim3(red.ctas, (kBasis + 7) / 8), stream, V.p, n, kBasis, V.p + (long long)kBasis * n,
                                      n, red.part.p, red.ticket.p, coef.p, nullptr, nullptr);
            break;
        case SENK_OP_UPDATE:
            launch_update<T, kEpiNone>(red.ctas, stream, V.p, n, kBasis, coef.p, V.p + (long long)kBasis * n, n,
                                       red.part.p, red.ticket.p, nullptr, st.p, GmresEpi{}, nullptr);
            break;
        default: throw ArgError("unknown op");
        }
    };
    switch (op) {
    case SENK_OP_SPMV: bytes = (long long)A.nnz * (vb + 4) + 4LL * (n + 1) + 2LL * n * vb; break;
    case SENK_OP_PRECOND: bytes = pcb ? pcb->apply_bytes() : pc->apply_bytes(); break;
    case SENK_OP_SWEEP_L:
        bytes = pcb ? pcb->lblocks * (pcb->bnl * pcb->bnw * vb + 4) + 4LL * (pcb->nbr + 1) + 2LL * n * vb
                    : pc->L.nnz * (vb + 4) + 2LL * n * vb;
        break;
    case SENK_OP_SWEEP_U:
        bytes = pcb ? pcb->ublocks * (pcb->bnl * pcb->bnw * vb + 4) + 4LL * (pcb->nbr + 1) + 2LL * n * vb
                    : (pc->U.nnz - n) * (vb + 4) + 3LL * n * vb;
        break;
    case SENK_OP_DOT: bytes = 2LL * n * vb; break;
    case SENK_OP_MULTIDOT: bytes = (kBasis + 1LL) * n * vb; break;
    case SENK_OP_UPDATE: bytes = (kBasis + 2LL) * n * vb; break;
    }
    // deterministic finite inputs
    if (op == SENK_OP_MULTIDOT || op == SENK_OP_UPDATE) {
        SENK_CUDA(cudaMemsetAsync(V.p, 0, vb * n * (kBasis + 1), stream));
        SENK_CUDA(cudaMemsetAsync(coef.p, 0, sizeof(double) * kBasis, stream));
        for (int k = 0; k <= kBasis; k++)
            ew<T, 4>(x.p, V.p + (long long)k * n, nullptr, n, T(0), T(0), nullptr, 1.0, stream, nullptr);
    } else {
        ew<T, 4>(x.p, v0, nullptr, n, T(0), T(0), nullptr, 1.0, stream, nullptr);
        SENK_CUDA(cudaMemsetAsync(v1, 0, vb * n, stream));
    }
    run();
    SENK_CUDA(cudaEventRecord(ev0, stream));
    for (int i = 0; i < reps; i++) run();
    SENK_CUDA(cudaEventRecord(ev1, stream));
    SENK_CUDA(cudaEventSynchronize(ev1));
    SENK_LAUNCH_CHECK();
    float ms = 0;
    SENK_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    *ms_out = ms / reps;
    *bytes_out = bytes;
}

template <typename T>
int System<T>::gmres_ir(double nrm_b, int max_outer, int m, double eps, double inner_tol, int inner_cycles,
                        senk_result *res)
{
    SENK_REQUIRE(inner, "GMRES-IR needs a system created with mixed = 1");
    SENK_REQUIRE(max_outer >= 0 && inner_cycles >= 1 && inner_tol > 0, "bad GMRES-IR parameters");
    inner->ensure_gmres(m);
    return refine(nrm_b, max_outer, eps, res, [&](senk_result *ri) {
        inner->gmres(1.0, inner_cycles, m, inner_tol, ri);
    });
}

template <typename T>
int System<T>::gcr_ir(double nrm_b, int max_outer, int m, double eps, double inner_tol, int inner_cycles,
                      senk_result *res)
{
    SENK_REQUIRE(inner && !ir_only, "GCR-IR needs a system created with mixed = 1");
    SENK_REQUIRE(max_outer >= 0 && inner_cycles >= 1 && inner_tol > 0, "bad GCR-IR parameters");
    return refine(nrm_b, max_outer, eps, res, [&](senk_result *ri) {
        inner->gcr(1.0, inner_cycles, m, inner_tol, ri);
    });
}

template <typename T>
int System<T>::refine(double nrm_b, int max_outer, double eps, senk_result *res,
                      const std::function<void(senk_result *)> &inner_solve)
{
    const int grid = stream_grid(n, kThreads, 8);
    SENK_CUDA(cudaEventRecord(ev0, stream));
    long long iters = 0, launches = 0;
    int outer = 0, conv = 0, brk = 0;
    double rel = -1;
    for (int k = 0;; k++) {
        // FP64 true residual r = b - A x (into t), its norm and inverse
        A.residual(x.p, b.p, t.p, red, irs.p, irs.p + 1, stream);
        SENK_CUDA(cudaMemcpyAsync(ir_host, irs.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SENK_CUDA(cudaStreamSynchronize(stream));
        launches++;
        rel = ir_host[0] / nrm_b;
        if (ir_host[0] <= eps * nrm_b) {
            conv = 1;
            break;
        }
        if (k == max_outer || !(ir_host[0] == ir_host[0])) break;
        // inner FP32 solve of A d = r/||r|| from d = 0
        k_ir_demote<<<grid, kThreads, 0, stream>>>(t.p, irs.p + 1, inner->b.p, n);
        SENK_CUDA(cudaMemsetAsync(inner->x.p, 0, inner->x.bytes(), stream));
        senk_result ri{};
        inner_solve(&ri);
        iters += ri.iters;
        launches += ri.launches + 2;
        brk |= ri.breakdown;
        // x += ||r|| d in FP64
        k_ir_correct<<<grid, kThreads, 0, stream>>>((double *)x.p, irs.p, inner->x.p, n);
        SENK_LAUNCH_CHECK();
        outer++;
    }
    SENK_CUDA(cudaEventRecord(ev1, stream));
    SENK_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    SENK_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    if (opt.verbose) {
        printf(conv ? "I iter %lld\n" : "# iter %lld\n", iters);
        printf("# res %e\n", rel);
        fflush(stdout);
    }
    if (res) {
        res->iters = (int)iters;
        res->converged = conv;
        res->res = rel;
        res->solve_ms = ms;
        res->breakdown = brk;
        res->cycles = outer;
        res->launches = launches;
    }
    return kOk;
}

template <>
int System<float>::refine(double, int, double, senk_result *, const std::function<void(senk_result *)> &)
{
    throw ArgError("iterative refinement runs on an FP64 system");
}

template struct System<double>;
template struct System<float>;

namespace {

template <typename T>
int dropin_gmres(const char *fn, const T *val, const int *cind, const int *rptr, const T *lval, const int *lcind,
                 const int *lrptr, const T *uval, const int *ucind, const int *urptr, int precond, const int *cptr,
                 int cnum, int bsize, const T *b, T *x, double nrm_b, int outer, int m, int N, double eps,
                 const senk_options *opt, senk_result *res)
{
    return guarded(fn, [&] {
        SENK_REQUIRE(val && cind && rptr && b && x, "null argument");
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
        d.m_max = m;
        senk_options o{};
        if (opt) o = *opt;
        std::lock_guard<std::mutex> lk(dropin_mutex());
        bool built = false;
        auto sp = dropin_system<T>(fn, d, o, &built);
        System<T> &S = *sp;
        S.b.upload(b, N, S.stream);
        S.x.upload(x, N, S.stream);
        senk_result r{};
        S.gmres(nrm_b, outer, m, eps, &r);
        SENK_CUDA(cudaMemcpyAsync(x, S.x.p, sizeof(T) * N, cudaMemcpyDeviceToHost, S.stream));
        SENK_CUDA(cudaStreamSynchronize(S.stream));
        r.h2d_bytes = (built ? S.h2d_bytes : 0) + 2LL * sizeof(T) * N;
        r.d2h_bytes = (long long)sizeof(T) * N;
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

}  // namespace

}  // namespace senkgpu

using namespace senkgpu;

extern "C" {

int senk_system_create(senk_system **out, const senk_system_desc *desc, const senk_options *opt)
{
    return guarded("senk_system_create", [&] {
        SENK_REQUIRE(out && desc, "null argument");
        auto h = std::make_unique<senk_system>();
        h->dtype = desc->dtype;
        if (desc->dtype == SENK_F64) {
            h->d = std::make_unique<System<double>>();
            h->d->create(*desc, opt);
        } else if (desc->dtype == SENK_F32) {
            h->f = std::make_unique<System<float>>();
            h->f->create(*desc, opt);
        } else {
            throw ArgError("dtype must be SENK_F64 or SENK_F32");
        }
        *out = h.release();
        return (int)kOk;
    });
}

int senk_system_destroy(senk_system *sys)
{
    return guarded("senk_system_destroy", [&] {
        delete sys;
        return (int)kOk;
    });
}

void *senk_system_stream(senk_system *sys)
{
    if (!sys) return nullptr;
    return sys->d ? (void *)sys->d->stream : (void *)sys->f->stream;
}

void *senk_system_b(senk_system *sys)
{
    if (!sys) return nullptr;
    return sys->d ? (void *)sys->d->b.p : (void *)sys->f->b.p;
}

void *senk_system_x(senk_system *sys)
{
    if (!sys) return nullptr;
    return sys->d ? (void *)sys->d->x.p : (void *)sys->f->x.p;
}

int senk_system_set_rhs(senk_system *sys, const void *b, const void *x0)
{
    return guarded("senk_system_set_rhs", [&] {
        SENK_REQUIRE(sys && b, "null argument");
        if (sys->d) {
            auto &S = *sys->d;
            S.b.upload((const double *)b, S.n, S.stream);
            if (x0) S.x.upload((const double *)x0, S.n, S.stream);
            else SENK_CUDA(cudaMemsetAsync(S.x.p, 0, S.x.bytes(), S.stream));
            SENK_CUDA(cudaStreamSynchronize(S.stream));
        } else {
            auto &S = *sys->f;
            S.b.upload((const float *)b, S.n, S.stream);
            if (x0) S.x.upload((const float *)x0, S.n, S.stream);
            else SENK_CUDA(cudaMemsetAsync(S.x.p, 0, S.x.bytes(), S.stream));
            SENK_CUDA(cudaStreamSynchronize(S.stream));
        }
        return (int)kOk;
    });
}

int senk_system_zero_x(senk_system *sys)
{
    return guarded("senk_system_zero_x", [&] {
        SENK_REQUIRE(sys, "null system");
        if (sys->d) SENK_CUDA(cudaMemsetAsync(sys->d->x.p, 0, sys->d->x.bytes(), sys->d->stream));
        else SENK_CUDA(cudaMemsetAsync(sys->f->x.p, 0, sys->f->x.bytes(), sys->f->stream));
        return (int)kOk;
    });
}

int senk_system_get_x(senk_system *sys, void *x)
{
    return guarded("senk_system_get_x", [&] {
        SENK_REQUIRE(sys && x, "null argument");
        if (sys->d) {
            SENK_CUDA(cudaMemcpyAsync(x, sys->d->x.p, sys->d->x.bytes(), cudaMemcpyDeviceToHost, sys->d->stream));
            SENK_CUDA(cudaStreamSynchronize(sys->d->stream));
        } else {
            SENK_CUDA(cudaMemcpyAsync(x, sys->f->x.p, sys->f->x.bytes(), cudaMemcpyDeviceToHost, sys->f->stream));
            SENK_CUDA(cudaStreamSynchronize(sys->f->stream));
        }
        return (int)kOk;
    });
}

int senk_system_time_op(senk_system *sys, int op, int reps, double *ms_per_rep, long long *bytes_per_rep)
{
    return guarded("senk_system_time_op", [&] {
        SENK_REQUIRE(sys && reps > 0, "bad argument");
        double ms = 0;
        long long bytes = 0;
        if (op >= SENK_OP_INNER) {
            SENK_REQUIRE(sys->d && sys->d->inner, "system has no FP32 copy (mixed = 0)");
            sys->d->inner->time_op(op - SENK_OP_INNER, reps, &ms, &bytes);
        } else if (sys->d) {
            sys->d->time_op(op, reps, &ms, &bytes);
        } else {
            sys->f->time_op(op, reps, &ms, &bytes);
        }
        if (ms_per_rep) *ms_per_rep = ms;
        if (bytes_per_rep) *bytes_per_rep = bytes;
        return (int)kOk;
    });
}

int senk_system_gmres_ir(senk_system *sys, double nrm_b, int max_outer, int m, double epsilon, double inner_tol,
                         int inner_cycles, senk_result *res)
{
    return guarded("senk_system_gmres_ir", [&] {
        SENK_REQUIRE(sys && sys->d, "GMRES-IR needs an FP64 system");
        senk_result r{};
        sys->d->gmres_ir(nrm_b, max_outer, m, epsilon, inner_tol, inner_cycles, &r);
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

int senk_dropin_cache(int mode)
{
    std::lock_guard<std::mutex> lk(dropin_mutex());
    const int prev = dropin_cache_mode();
    dropin_cache_mode() = mode ? 1 : 0;
    if (!mode) dropin_cache_clear();
    return prev;
}

int senk_system_apply_pc(senk_system *sys, const void *x, void *y)
{
    return guarded("senk_system_apply_pc", [&] {
        SENK_REQUIRE(sys && x && y, "null argument");
        if (sys->d) {
            SENK_REQUIRE(sys->d->has_pc(), "the system has no preconditioner");
            sys->d->precondition_base((const double *)x, (double *)y, nullptr);
            SENK_CUDA(cudaStreamSynchronize(sys->d->stream));
            sys->d->check_pc();
        } else {
            SENK_REQUIRE(sys->f->has_pc(), "the system has no preconditioner");
            sys->f->precondition_base((const float *)x, (float *)y, nullptr);
            SENK_CUDA(cudaStreamSynchronize(sys->f->stream));
            sys->f->check_pc();
        }
        return (int)kOk;
    });
}

int senk_system_apply_a(senk_system *sys, const void *x, void *y)
{
    return guarded("senk_system_apply_a", [&] {
        SENK_REQUIRE(sys && x && y, "null argument");
        if (sys->d) {
            sys->d->A.apply((const double *)x, (double *)y, sys->d->stream, nullptr);
            SENK_CUDA(cudaStreamSynchronize(sys->d->stream));
        } else {
            sys->f->A.apply((const float *)x, (float *)y, sys->f->stream, nullptr);
            SENK_CUDA(cudaStreamSynchronize(sys->f->stream));
        }
        return (int)kOk;
    });
}

int senk_system_gcr_ir(senk_system *sys, double nrm_b, int max_outer, int m, double epsilon, double inner_tol,
                       int inner_cycles, senk_result *res)
{
    return guarded("senk_system_gcr_ir", [&] {
        SENK_REQUIRE(sys && sys->d, "GCR-IR needs an FP64 system");
        senk_result r{};
        sys->d->gcr_ir(nrm_b, max_outer, m, epsilon, inner_tol, inner_cycles, &r);
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

int senk_abmc_ilu_gmres_ir_d(const double *val, const int *cind, const int *rptr, const double *lval,
                             const int *lcind, const int *lrptr, const double *uval, const int *ucind,
                             const int *urptr, const int *cptr, int cnum, int bsize, const double *b, double *x,
                             double nrm_b, int max_outer, int m, int N, double epsilon, double inner_tol,
                             int inner_cycles, const senk_options *opt, senk_result *res)
{
    return guarded("senk_abmc_ilu_gmres_ir_d", [&] {
        SENK_REQUIRE(val && cind && rptr && b && x, "null argument");
        senk_system_desc d{};
        d.N = N;
        d.dtype = SENK_F64;
        d.val = val; d.cind = cind; d.rptr = rptr;
        d.precond = SENK_PC_ILU_ABMC;
        d.lval = lval; d.lcind = lcind; d.lrptr = lrptr;
        d.uval = uval; d.ucind = ucind; d.urptr = urptr;
        d.cptr = cptr; d.cnum = cnum; d.bsize = bsize;
        d.mixed = 2;  // the FP64 part only computes residuals and updates
        senk_options o{};
        if (opt) o = *opt;
        std::lock_guard<std::mutex> lk(dropin_mutex());
        bool built = false;
        auto sp = dropin_system<double>("senk_abmc_ilu_gmres_ir_d", d, o, &built);
        System<double> &S = *sp;
        S.b.upload(b, N, S.stream);
        S.x.upload(x, N, S.stream);
        senk_result r{};
        S.gmres_ir(nrm_b, max_outer, m, epsilon, inner_tol, inner_cycles, &r);
        SENK_CUDA(cudaMemcpyAsync(x, S.x.p, sizeof(double) * N, cudaMemcpyDeviceToHost, S.stream));
        SENK_CUDA(cudaStreamSynchronize(S.stream));
        r.h2d_bytes = (built ? S.h2d_bytes : 0) + 2LL * sizeof(double) * N;
        r.d2h_bytes = (long long)sizeof(double) * N;
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

int senk_system_gmres(senk_system *sys, double nrm_b, int outer, int m, double epsilon, senk_result *res)
{
    return guarded("senk_system_gmres", [&] {
        SENK_REQUIRE(sys, "null system");
        senk_result r{};
        if (sys->d) sys->d->gmres(nrm_b, outer, m, epsilon, &r);
        else sys->f->gmres(nrm_b, outer, m, epsilon, &r);
        if (res) *res = r;
        return r.breakdown ? (int)kErrBreakdown : (int)kOk;
    });
}

int senk_gmres_d(const double *val, const int *cind, const int *rptr, const double *b, double *x, double nrm_b,
                 int outer, int m, int N, double epsilon, const senk_options *opt, senk_result *res)
{
    return dropin_gmres<double>("senk_gmres_d", val, cind, rptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                nullptr, SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_gmres_s(const float *val, const int *cind, const int *rptr, const float *b, float *x, float nrm_b, int outer,
                 int m, int N, float epsilon, const senk_options *opt, senk_result *res)
{
    return dropin_gmres<float>("senk_gmres_s", val, cind, rptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                               SENK_PC_NONE, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_amc_ilu_gmres_s(const float *val, const int *cind, const int *rptr, const float *lval, const int *lcind,
                         const int *lrptr, const float *uval, const int *ucind, const int *urptr, const int *cptr,
                         int cnum, const float *b, float *x, float nrm_b, int outer, int m, int N, float epsilon,
                         const senk_options *opt, senk_result *res)
{
    return dropin_gmres<float>("senk_amc_ilu_gmres_s", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                               SENK_PC_ILU_AMC, cptr, cnum, 1, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_ilu_gmres_d(const double *val, const int *cind, const int *rptr, const double *lval, const int *lcind,
                     const int *lrptr, const double *uval, const int *ucind, const int *urptr, const double *b,
                     double *x, double nrm_b, int outer, int m, int N, double epsilon, const senk_options *opt,
                     senk_result *res)
{
    return dropin_gmres<double>("senk_ilu_gmres_d", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                SENK_PC_ILU, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_ilu_gmres_s(const float *val, const int *cind, const int *rptr, const float *lval, const int *lcind,
                     const int *lrptr, const float *uval, const int *ucind, const int *urptr, const float *b,
                     float *x, float nrm_b, int outer, int m, int N, float epsilon, const senk_options *opt,
                     senk_result *res)
{
    return dropin_gmres<float>("senk_ilu_gmres_s", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                               SENK_PC_ILU, nullptr, 0, 0, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_amc_ilu_gmres_d(const double *val, const int *cind, const int *rptr, const double *lval, const int *lcind,
                         const int *lrptr, const double *uval, const int *ucind, const int *urptr, const int *cptr,
                         int cnum, const double *b, double *x, double nrm_b, int outer, int m, int N,
                         double epsilon, const senk_options *opt, senk_result *res)
{
    return dropin_gmres<double>("senk_amc_ilu_gmres_d", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                SENK_PC_ILU_AMC, cptr, cnum, 1, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_abmc_ilu_gmres_d(const double *val, const int *cind, const int *rptr, const double *lval,
                          const int *lcind, const int *lrptr, const double *uval, const int *ucind,
                          const int *urptr, const int *cptr, int cnum, int bsize, const double *b, double *x,
                          double nrm_b, int outer, int m, int N, double epsilon, const senk_options *opt,
                          senk_result *res)
{
    return dropin_gmres<double>("senk_abmc_ilu_gmres_d", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                                SENK_PC_ILU_ABMC, cptr, cnum, bsize, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

int senk_abmc_ilu_gmres_s(const float *val, const int *cind, const int *rptr, const float *lval, const int *lcind,
                          const int *lrptr, const float *uval, const int *ucind, const int *urptr, const int *cptr,
                          int cnum, int bsize, const float *b, float *x, float nrm_b, int outer, int m, int N,
                          float epsilon, const senk_options *opt, senk_result *res)
{
    return dropin_gmres<float>("senk_abmc_ilu_gmres_s", val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr,
                               SENK_PC_ILU_ABMC, cptr, cnum, bsize, b, x, nrm_b, outer, m, N, epsilon, opt, res);
}

}  // extern "C"
