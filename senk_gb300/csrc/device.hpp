// Host-side device objects of libsenk_gpu: buffers, the ILU sweep plan, the SpMV
// operator and the resident system used by the Krylov engines.
#pragma once

#include <cstring>
#include <functional>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/senk_gpu.h"
#include "kernels.cuh"

namespace senkgpu {

struct ArgError : std::runtime_error {
    explicit ArgError(const std::string &m) : std::runtime_error(m) {}
};

#define SENK_REQUIRE(cond, msg) \
    do { if (!(cond)) throw ::senkgpu::ArgError(msg); } while (0)

// Runs an entry point body, mapping exceptions to status codes + last error.
template <typename F>
int guarded(const char *fn, F &&body)
{
    try {
        return body();
    } catch (const CudaError &e) {
        set_last_error(std::string(fn) + ": " + e.what + " failed: " + cudaGetErrorString(e.code) +
                       " (" + e.file + ":" + std::to_string(e.line) + ")");
        cudaGetLastError();  // clear a sticky-free error so the next call starts clean
        return e.code == cudaErrorMemoryAllocation ? kErrAlloc : kErrCuda;
    } catch (const ArgError &e) {
        set_last_error(std::string(fn) + ": " + e.what());
        return kErrArg;
    } catch (const std::bad_alloc &) {
        set_last_error(std::string(fn) + ": host allocation failed");
        return kErrAlloc;
    } catch (const std::exception &e) {
        set_last_error(std::string(fn) + ": " + e.what());
        return kErrArg;
    }
}

// Owning device allocation.
template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count)
    {
        release();
        if (count) SENK_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
        n = count;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void upload(const T *h, size_t count, cudaStream_t s)
    {
        if (count) SENK_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T> &h, cudaStream_t s)
    {
        if (h.size() > n) alloc(h.size());
        upload(h.data(), h.size(), s);
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Partials + ticket for the last-CTA-finishes reductions. One per stream: the
// reduction kernels of a stream run one after another and share it. `ctas`
// (4 per SM of the device) is the grid of the multi-dot and update kernels;
// the partials hold kMaxCols columns of that many CTAs.
struct ReduceScratch {
    static constexpr int kMaxCols = 64;
    int ctas = 0;
    DevBuf<double> part;
    DevBuf<unsigned> ticket;
    void ensure(cudaStream_t s)
    {
        if (!part.p) {
            ctas = 4 * sm_count();
            part.alloc((size_t)kMaxCols * ctas);
            ticket.alloc(1);
            SENK_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s));
        }
    }
};

// ----------------------------------------------------------------- SpMV op

// A on the device. CSR always (for the residual); optionally a SELL-32 copy.
// Sorting window of the solver's SELL-32-sigma copy of A (SENK_SPMV_AUTO and
// SENK_SPMV_SELL_SIGMA): rows taken longest first within each 256 rows.
constexpr int kSellSigma = 256;

template <typename T>
struct SpmvOp {
    int n = 0, nnz = 0;
    int lanes = 8;              // lanes per row of the CSR kernel
    DevBuf<T> val;
    DevBuf<int> cind, rptr;
    bool use_sell = false;
    DevBuf<T> sval;
    DevBuf<int> scol, soff;
    DevBuf<int> sperm;           // SELL-32-sigma: slice position -> row

    // keep_csr = false (with a SELL format): only the SELL copy stays on the device
    void upload(const T *v, const int *c, const int *r, int N, int format, cudaStream_t s, bool keep_csr = true);
    template <typename S>
    void convert_from(const SpmvOp<S> &src, int format, cudaStream_t s, bool keep_csr);
    template <typename S>
    void sell_from_device(const S *dv, const int *dc, const int *dr, const std::vector<int> &off,
                          const std::vector<int> &perm, cudaStream_t s);
    void drop_csr(cudaStream_t s);
    bool has_csr = false;
    std::vector<int> sell_off;  // host copy of the SELL slice offsets
    std::vector<int> sell_perm; // host copy of the sigma permutation (empty: rows in order)
    long long h2d = 0;          // bytes copied from the host
    // y = A x (MODE 0) or y = b - A x (MODE 1)
    void apply(const T *x, T *y, cudaStream_t s, const int *gate) const;
    // y = b - A x, ||y|| -> *norm_out, 1/||y|| -> *inv_out
    void residual(const T *x, const T *b, T *y, ReduceScratch &red, double *norm_out, double *inv_out,
                  cudaStream_t s) const;
};

// Lanes per row of the CSR kernel: the smallest power of two covering the mean
// row length, between 2 and 32.
int csr_lanes(long long nnz, int n);

void launch_spmv_csr_d(const double *v, const int *c, const int *r, const double *x, const double *b,
                       double *y, int n, int lanes, int mode, cudaStream_t s, const int *gate);
void launch_spmv_csr_s(const float *v, const int *c, const int *r, const float *x, const float *b,
                       float *y, int n, int lanes, int mode, cudaStream_t s, const int *gate);

// ----------------------------------------------------------- ILU sweeps

// One triangular factor in the chain-sliced layout.
template <typename VT>
struct SweepFactor {
    bool upper = false;
    bool mapped = false;           // schedule positions map to rows through rowmap
    int bs = 1;                    // rows per chain
    DevBuf<VT> val;
    DevBuf<int> col;
    DevBuf<VT> dinv;               // U: inverted diagonal per schedule position
    DevBuf<int> rowmap;
    DevBuf<GroupDesc> groups;
    DevBuf<unsigned char> widths;  // per group: we[bs], wi[bs]
    std::vector<int> colour_groups; // group range of each colour, in processing order
    std::vector<size_t> colour_smem; // bytes to stage the largest group of each colour
    long long elems = 0;           // padded slots
    long long nnz = 0;             // stored off-diagonal entries (+N for U's diagonal)
    // compact chain layout (one warp per group): groups, chain descriptors and,
    // for the dataflow launch, the groups each group reads from, per-group flags
    // and the launch's control words
    bool compact = false;          // compact chain layout (else row slots)
    bool dataflow = false;         // compact: one launch per sweep (else one per colour)
    std::vector<int> colour_slots; // compact: widest block of each colour
    DevBuf<unsigned char> wcounts; // compact: per chain, external and in-chain counts of each row
    DevBuf<int> dcolour_groups;    // compact: colour_groups on the device
    DevBuf<int4> levels;           // compact, per colour: {first group, groups, first slot, slots}
    DevBuf<VT> cdinv;              // compact U: inverted diagonal per chain (small systems)
    size_t level_bytes = 0;        // compact, chains of one row: most bytes one colour stages
    // compact, per colour: the launches of a sweep in order
    struct Launch {
        int g0, g1;        // groups of the colour
        int early_x;       // 1: x is read before the wait on the previous kernel
        size_t smem;       // dynamic shared memory
        // a cooperative launch (k_sweep_cp) of colours [cbeg, cend) on `grid` CTAs
        // instead of one colour (k_sweep_cc)
        int coop = 0, cbeg = 0, cend = 0, grid = 0;
        // 1: k_sweep_cc2 (two rows per thread) instead of k_sweep_cc
        int wide = 0;
    };
    std::vector<Launch> launches;
    DevBuf<WfGroup> wgroups;
    DevBuf<int2> wchains;
    DevBuf<int> dep_ptr, dep_idx, flags, ctrl;
    int ngroups = 0;
    int slots_max = 0;             // widest group block (slots of 32 entries)
    int wf_warps = 0, wf_grid = 0; // warps per CTA, CTAs
    size_t wf_smem = 0;            // dynamic shared memory per CTA
    // compact: runs of colours that fit one wave of co-resident CTAs sweep in
    // one cooperative launch each (k_sweep_cp; bytes of each of its two staging
    // buffers; ctrl holds its barrier words)
    bool persistent = false;
    size_t cp_buf = 0;
    // compact, per colour: every colour takes k_sweep_cc2 (SENK_SWEEP_WIDE), or
    // with rowlane every colour k_sweep_rl with two chains per lane
    bool force_wide = false;
    // compact, per colour, external entries chain-major: k_sweep_rl (lanes =
    // rows of a chain) instead of k_sweep_cc
    bool rowlane = false;
};

// A split ILU factorisation with its sweep schedule.
template <typename VT>
struct IluPlan {
    int n = 0;
    int precond = SENK_PC_NONE;
    SweepFactor<VT> L, U;
    DevBuf<int> status;  // non-zero after a sweep whose bounded wait ran out (1: flag, 2: TMA)
    // small systems (the vector fits in shared memory): both sweeps in one CTA
    bool small = false;
    int small_threads = 0;
    size_t small_buf = 0;          // bytes of each staging buffer
    int small_nbuf = 2;            // staging buffers (levels staged ahead + 1)
    void sweep_small(int which, const VT *x, VT *y, cudaStream_t s, const int *gate) const;
    void build_small(int N, const VT *lval, const int *lcind, const int *lrptr, const VT *uval, const int *ucind,
                     const int *urptr, int precond, const int *cptr, int cnum, int bsize, cudaStream_t s);

    // sweep_mode: SENK_SWEEP_AUTO / SENK_SWEEP_DATAFLOW (one dataflow launch per
    // sweep where the schedule is colours of chains) or SENK_SWEEP_COLOURS (one
    // launch per colour)
    void build(int N, const VT *lval, const int *lcind, const int *lrptr, const VT *uval, const int *ucind,
               const int *urptr, int precond, const int *cptr, int cnum, int bsize, cudaStream_t s,
               int sweep_mode = 0);
    template <typename XT>
    void sweep(const SweepFactor<VT> &F, const XT *x, XT *y, cudaStream_t s, const int *gate) const;
    template <typename XT>
    void apply(const XT *x, XT *y, cudaStream_t s, const int *gate) const
    {
        if (small) {
            sweep_small(3, (const VT *)x, (VT *)y, s, gate);
            return;
        }
        sweep(L, x, y, s, gate);
        sweep(U, (const XT *)y, y, s, gate);
    }
    // Algorithmic bytes of one application (values + indices once, x read once,
    // y written once per sweep and re-read by the U sweep), for roofline figures.
    long long apply_bytes() const;
    // Throws if a sweep reported a failed wait, and clears the report
    // (synchronises the stream).
    void check_status(cudaStream_t s) const;
};

// ILUB: split factors kept in BCSR (bnl x bnw blocks, block-column-major
// values), swept block row by block row. A chain is a run of consecutive block
// rows swept in order by one group of lanes (ascending for L, descending for
// U); chains of one phase run concurrently, phases one after another (L in
// order, U in reverse). Natural order: one phase holding one chain of every
// block row. ABMC: one phase per colour, one chain per ABMC block.
template <typename T>
struct IlubPlan {
    int n = 0, bnl = 1, bnw = 1, nbr = 0;
    DevBuf<T> lval, uval;
    DevBuf<int> lcind, lrptr, ucind, urptr;
    DevBuf<int2> chains;               // (first block row, block rows)
    std::vector<int> phase_chains;     // chain range of each phase
    long long lblocks = 0, ublocks = 0;

    void build(int N, int bnl, int bnw, const T *blval, const int *blcind, const int *blrptr, const T *buval,
               const int *bucind, const int *burptr, const int *cptr, int cnum, int bsize, cudaStream_t s);
    void sweep(bool upper, const T *x, T *y, cudaStream_t s, const int *gate) const;
    void apply(const T *x, T *y, cudaStream_t s, const int *gate) const
    {
        sweep(false, x, y, s, gate);
        sweep(true, (const T *)y, y, s, gate);
    }
    long long apply_bytes() const;
    long long h2d_bytes() const
    {
        return (long long)(lval.bytes() + uval.bytes() + lcind.bytes() + lrptr.bytes() + ucind.bytes() +
                           urptr.bytes() + chains.bytes());
    }
};

// --------------------------------------------------------- Krylov system

template <typename T>
struct System {
    int n = 0;
    cudaStream_t stream = nullptr;
    senk_options opt{};
    SpmvOp<T> A;
    std::unique_ptr<IluPlan<T>> pc;
    std::unique_ptr<IlubPlan<T>> pcb;  // ILUB (BCSR factors) instead of pc
    bool has_pc() const { return pc || pcb; }
    // out = K v: the ILU/ILUB application (the identity copy when the system
    // has no preconditioner), plus the learned correction when one is attached
    void precondition(const T *v, T *out, const int *gate);
    void precondition_base(const T *v, T *out, const int *gate);
    // learned correction (FP64 systems): a bound senk_mpnn, used by GCR; the
    // GCR falls back to the plain preconditioner when a restart cycle reduces
    // the residual by less than the factor learned_stall
    void *learned = nullptr;
    double learned_stall = 0.9;
    int learned_fallback = -1;        // restart cycle of the last solve's fall-back (-1: none)
    bool gcr_learned_in_graph = false;
    void check_pc() const;
    DevBuf<T> b, x, t;
    // GMRES workspace
    int m_alloc = 0;
    DevBuf<T> V;
    DevBuf<double> H, cs, sn, e, y, coef;
    DevBuf<KrylovState> st;
    ReduceScratch red;
    KrylovState *st_host = nullptr;  // pinned mirror
    // captured restart cycle
    cudaGraphExec_t cycle = nullptr;
    int cycle_m = -1, cycle_orth = -1;
    long long cycle_nodes = 0;       // kernel nodes of the captured cycle
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // Mixed precision (FP64 systems created with desc.mixed): the FP32 copy
    // that runs the inner solves of GMRES-IR on the same stream.
    std::unique_ptr<System<float>> inner;
    DevBuf<double> irs;               // ||r||, 1/||r|| of the outer residual
    double *ir_host = nullptr;        // pinned mirror of irs
    bool own_stream = true;

    System() = default;
    System(const System &) = delete;
    ~System();
    // `shared` (optional): run on this stream instead of creating one.
    // sell_only: keep A on the device as SELL only (no CSR copy).
    // csr_src: an FP64 operator holding the same matrix (CSR on the device) to
    // convert A from, instead of desc.val.
    void create(const senk_system_desc &d, const senk_options *o, cudaStream_t shared = nullptr,
                bool sell_only = false, const SpmvOp<double> *csr_src = nullptr);
    bool ir_only = false;  // desc.mixed == 2: the FP64 part serves GMRES-IR's outer loop only
    int gmres_ir(double nrm_b, int max_outer, int m, double eps, double inner_tol, int inner_cycles,
                 senk_result *res);
    // FP64 outer refinement around FP32 inner GCR(m) (mixed = 1 systems)
    int gcr_ir(double nrm_b, int max_outer, int m, double eps, double inner_tol, int inner_cycles,
               senk_result *res);
    // The refinement loop: r = b - A x in FP64 until ||r|| <= eps nrm_b; each
    // step solves the FP32 system for r / ||r|| with inner_solve and adds
    // ||r|| d to x.
    int refine(double nrm_b, int max_outer, double eps, senk_result *res,
               const std::function<void(senk_result *)> &inner_solve);
    void ensure_gmres(int m);
    void enqueue_gmres_cycle(int m);
    int gmres(double nrm_b, int outer, int m, double eps, senk_result *res);
    void time_op(int op, int reps, double *ms, long long *bytes);
    long long h2d_bytes = 0;         // bytes uploaded by create()
    // GCR(m): directions p_0..p_m and Kr in P; A p_0..A p_m, r and A K r in AP
    int gcr_m = -1;
    DevBuf<T> P, AP;
    DevBuf<double> dAp;
    cudaGraphExec_t gcr_cycle = nullptr;
    long long gcr_nodes = 0;
    int gcr(double nrm_b, int outer, int m, double eps, senk_result *res);
    // BiCGStab: r, r*, p, Kp, AKp, s, AKs, Ks (s and AKs adjacent)
    DevBuf<T> BW;
    DevBuf<double> hist;             // ||r||/||b|| after each iteration
    cudaGraphExec_t bicg_step = nullptr;
    long long bicg_nodes = 0;
    int bicgstab(double nrm_b, int max_iter, double eps, senk_result *res);
};

}  // namespace senkgpu

// The opaque handles of the C ABI.
struct senk_system {
    int dtype = SENK_F64;
    std::unique_ptr<senkgpu::System<double>> d;
    std::unique_ptr<senkgpu::System<float>> f;
};

struct senk_ilu_plan {
    int dtype = SENK_F64;
    std::unique_ptr<senkgpu::IluPlan<double>> d;
    std::unique_ptr<senkgpu::IluPlan<float>> f;
    std::unique_ptr<senkgpu::IlubPlan<double>> b;  // senk_ilub_plan_create
};
