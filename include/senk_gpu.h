/*
 * senk_gpu.h — C ABI of libsenk_gpu.so, the GB300 (sm_103a) implementation of
 * SenK's preconditioned Krylov path.
 *
 * Plain C types only: host or device pointers, sizes, and opaque handles. Every
 * function returns a status code (SENK_OK == 0); senk_last_error() gives a
 * message for the last failure on the calling thread. Each declaration names the
 * reference interface it replaces (sapporosaburo/SenK, include/*.hpp file:line).
 *
 * Layout conventions are the reference's: CSR with int32 indices, sorted columns
 * (val[nnz], cind[nnz], rptr[N+1]); split ILU factors as made by
 * senk::matrix::Split(..., "L-DU", invDiag=true) (L strictly lower; each U row
 * starts with the inverted diagonal); BCSR blocks column-major.
 */
#ifndef SENK_GPU_H
#define SENK_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------- status codes */
#define SENK_OK 0
#define SENK_ERR_ARG 1
#define SENK_ERR_CUDA 2
#define SENK_ERR_ALLOC 3
#define SENK_ERR_BREAKDOWN 4
#define SENK_ERR_ZERO_PIVOT 5

/* Message of the last failure on this thread ("" if none). */
const char *senk_last_error(void);
/* Library version (major*10000 + minor*100 + patch). */
int senk_version(void);
/* Number of visible CUDA devices (0 on a host without a GPU; never fails). */
int senk_device_count(void);
/* Make `device` current for the calling thread's later calls. */
int senk_set_device(int device);

/* ------------------------------------------------------- solver reporting */
/* The reference reports only on stdout (include/senk_gmres.hpp:72-73,86-87;
 * senk_bicgstab.hpp:63-66,77-78; senk_gcr.hpp:48,115). The same numbers are
 * returned here; with opt->verbose the same lines are also printed. */
typedef struct {
    int iters;        /* iteration count exactly as the reference prints it */
    int converged;    /* 1 when the stopping test was met */
    double res;       /* relative residual as the reference prints it */
    double solve_ms;  /* device time of the iteration, uploads excluded */
    int breakdown;    /* 1 if a Krylov scalar was zero or not finite */
    int cycles;       /* restart cycles (GMRES/GCR) or iterations (BiCGStab) run */
    long long h2d_bytes; /* host -> device bytes this call copied */
    long long d2h_bytes; /* device -> host bytes this call copied */
    long long launches;  /* kernels launched by the solve (graph nodes x cycles) */
} senk_result;

/* Orthogonalisation of the Arnoldi step (new: the reference always uses MGS,
 * include/senk_gmres.hpp:224-227). */
#define SENK_ORTH_CGS 0  /* one classical pass: one fused multi-dot + one update (default) */
#define SENK_ORTH_CGS2 1 /* classical Gram-Schmidt + one re-orthogonalisation */
#define SENK_ORTH_MGS 2  /* modified Gram-Schmidt, the reference's order */

#define SENK_SPMV_AUTO 0  /* SELL-32-sigma(256) for the solver's SpMV */
#define SENK_SPMV_CSR 1   /* CSR, lanes per row from the mean row length */
#define SENK_SPMV_SELL 2  /* SELL-32 built on upload, rows in order */
#define SENK_SPMV_SELL_SIGMA 3 /* SELL-32-sigma: within each window of 256 rows
                                  the rows are taken longest first (stable) before
                                  they are cut into slices of 32; y is written
                                  through the position -> row map */

typedef struct {
    int orth;         /* SENK_ORTH_* */
    int spmv;         /* SENK_SPMV_* */
    int verbose;      /* print the reference's stdout lines (2: also setup timings) */
    int sweep;        /* SENK_SWEEP_* */
} senk_options;

/* How the ILU sweeps are scheduled. Chains (ABMC blocks; single rows for AMC
 * and the natural order's level sets) are taken 32 to a group from one colour
 * (level set). */
#define SENK_SWEEP_AUTO 0     /* the fastest as measured: natural-order or AMC
                                 systems whose vector fits in shared memory (up to
                                 192 KB) sweep both factors in one CTA; otherwise
                                 FP32 factors take SENK_SWEEP_ROWS and FP64
                                 factors SENK_SWEEP_COLOURS */
#define SENK_SWEEP_COLOURS 1  /* row-slot layout, one launch per colour (level set),
                                 one CTA per group */
#define SENK_SWEEP_DATAFLOW 2 /* compact chain layout, one launch per sweep: each
                                 warp takes a group, waits on the flags of the
                                 groups it reads, solves it and publishes its own */
#define SENK_SWEEP_COMPACT 3  /* compact chain layout (chains packed per lane,
                                 padding only to the widest chain of a group), one
                                 launch per colour, one CTA per group */
#define SENK_SWEEP_PERSISTENT 4 /* compact chain layout; every run of consecutive
                                 colours whose groups fit one wave of co-resident
                                 CTAs sweeps in one cooperative launch (the CTAs
                                 take the groups of a colour in turn, a grid
                                 barrier separates the colours, each group's block
                                 is staged while the group before it is solved);
                                 wider colours keep one launch each */
#define SENK_SWEEP_WIDE 5     /* as SENK_SWEEP_COMPACT, every colour with two rows
                                 per thread (CTAs of bsize/2 warps) where the ABMC
                                 block size is at least 4 (smaller blocks: one row
                                 per thread). COMPACT and AUTO take that kernel
                                 only for colours with more groups than one wave
                                 of one-row-per-thread CTAs holds */
#define SENK_SWEEP_ROWS 6     /* compact chain layout with each group's external
                                 entries chain after chain; one launch per colour,
                                 the lanes of a chain holding its rows in every
                                 phase (coalesced x and y, neighbouring gathers,
                                 no CTA barrier after staging); colours with more
                                 groups than one wave holds take two chains per
                                 lane */
#define SENK_SWEEP_ROWS_WIDE 7 /* as SENK_SWEEP_ROWS, two chains per lane in
                                 every colour (ABMC block size >= 2) */

/* Preconditioners and the schedules of their triangular sweeps. */
#define SENK_PC_NONE 0
#define SENK_PC_ILU 1       /* natural order: sweeps run level set by level set */
#define SENK_PC_ILU_AMC 2   /* AMC order: cptr counts rows, cnum colours */
#define SENK_PC_ILU_ABMC 3  /* ABMC order: cptr counts blocks of bsize rows */
#define SENK_PC_ILUB 4      /* BCSR factors (bnl x bnw blocks), natural order */
#define SENK_PC_ILUB_ABMC 5 /* BCSR factors of an ABMC-ordered system */

/* ======================================================= drop-in solvers ==
 * Host arrays in, x updated in place; one call uploads, solves on the GPU and
 * copies x back, like one call of the reference template. opt may be NULL.
 * The device copies of A and the factors (with their sweep layout and the
 * captured solver graphs) are kept for the next call: a call whose entry,
 * sizes, build options (spmv, sweep), host array addresses and array contents
 * (a 64-bit hash of every input array, computed on each call) match a kept
 * system uploads only b and x. The two most recent systems of each precision
 * are kept; drop-in calls are serialised by the library. */
/* Turns that cache on (mode 1, the default) or off (0: every call builds its
 * system, and the kept ones are freed now). Returns the previous mode. */
int senk_dropin_cache(int mode);

/* senk::solver::Gmresm<double> (include/senk_gmres.hpp:33-37) */
int senk_gmres_d(const double *val, const int *cind, const int *rptr,
                 const double *b, double *x, double nrm_b,
                 int outer, int m, int N, double epsilon,
                 const senk_options *opt, senk_result *res);

/* senk::solver::Gmresm<float> (include/senk_gmres.hpp:33-37) */
int senk_gmres_s(const float *val, const int *cind, const int *rptr,
                 const float *b, float *x, float nrm_b,
                 int outer, int m, int N, float epsilon,
                 const senk_options *opt, senk_result *res);

/* senk::solver::IluGmresm<T> (include/senk_gmres.hpp:197-203) */
int senk_ilu_gmres_d(const double *val, const int *cind, const int *rptr,
                     const double *lval, const int *lcind, const int *lrptr,
                     const double *uval, const int *ucind, const int *urptr,
                     const double *b, double *x, double nrm_b,
                     int outer, int m, int N, double epsilon,
                     const senk_options *opt, senk_result *res);
int senk_ilu_gmres_s(const float *val, const int *cind, const int *rptr,
                     const float *lval, const int *lcind, const int *lrptr,
                     const float *uval, const int *ucind, const int *urptr,
                     const float *b, float *x, float nrm_b,
                     int outer, int m, int N, float epsilon,
                     const senk_options *opt, senk_result *res);

/* senk::solver::AmcIluGmresm<double> (include/senk_gmres.hpp:293-300) */
int senk_amc_ilu_gmres_d(const double *val, const int *cind, const int *rptr,
                         const double *lval, const int *lcind, const int *lrptr,
                         const double *uval, const int *ucind, const int *urptr,
                         const int *cptr, int cnum,
                         const double *b, double *x, double nrm_b,
                         int outer, int m, int N, double epsilon,
                         const senk_options *opt, senk_result *res);

/* senk::solver::AmcIluGmresm<float> (include/senk_gmres.hpp:293-300) */
int senk_amc_ilu_gmres_s(const float *val, const int *cind, const int *rptr,
                         const float *lval, const int *lcind, const int *lrptr,
                         const float *uval, const int *ucind, const int *urptr,
                         const int *cptr, int cnum,
                         const float *b, float *x, float nrm_b,
                         int outer, int m, int N, float epsilon,
                         const senk_options *opt, senk_result *res);

/* senk::solver::AbmcIluGmresm<T> (include/senk_gmres.hpp:391-398) */
int senk_abmc_ilu_gmres_d(const double *val, const int *cind, const int *rptr,
                          const double *lval, const int *lcind, const int *lrptr,
                          const double *uval, const int *ucind, const int *urptr,
                          const int *cptr, int cnum, int bsize,
                          const double *b, double *x, double nrm_b,
                          int outer, int m, int N, double epsilon,
                          const senk_options *opt, senk_result *res);
int senk_abmc_ilu_gmres_s(const float *val, const int *cind, const int *rptr,
                          const float *lval, const int *lcind, const int *lrptr,
                          const float *uval, const int *ucind, const int *urptr,
                          const int *cptr, int cnum, int bsize,
                          const float *b, float *x, float nrm_b,
                          int outer, int m, int N, float epsilon,
                          const senk_options *opt, senk_result *res);

/* AbmcIluGmresm arguments, solved by mixed-precision GMRES-IR (see
 * senk_system_gmres_ir): FP32 ILU factors, SpTRSV sweeps, inner SpMV and Krylov
 * basis inside an FP64 refinement loop that stops on the FP64 true residual.
 * No direct counterpart in the reference (its FP32/FP64 refinement prototypes
 * are commented out, include/senk_bicgstab.hpp:269-296). */
int senk_abmc_ilu_gmres_ir_d(const double *val, const int *cind, const int *rptr,
                             const double *lval, const int *lcind, const int *lrptr,
                             const double *uval, const int *ucind, const int *urptr,
                             const int *cptr, int cnum, int bsize,
                             const double *b, double *x, double nrm_b,
                             int max_outer, int m, int N, double epsilon, double inner_tol,
                             int inner_cycles, const senk_options *opt, senk_result *res);

/* senk::solver::Gmresm<T,bnl,bnw> on a BCSR matrix (include/senk_gmres.hpp:113-117).
 * Every block entry, zeros included, enters the products as in SpmvBcsr. */
int senk_bcsr_gmres_d(const double *bval, const int *bcind, const int *brptr,
                      const double *b, double *x, double nrm_b,
                      int outer, int m, int N, double epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res);

/* senk::solver::BjIluGmresm<double> (include/senk_gmres.hpp:487-494): factors of
 * the block-Jacobi matrix (RemoveOffDiagonal with bnum blocks); a factor entry
 * that couples two blocks is rejected (SENK_ERR_ARG). */
int senk_bj_ilu_gmres_d(const double *val, const int *cind, const int *rptr,
                        const double *lval, const int *lcind, const int *lrptr,
                        const double *uval, const int *ucind, const int *urptr, int bnum,
                        const double *b, double *x, double nrm_b,
                        int outer, int m, int N, double epsilon,
                        const senk_options *opt, senk_result *res);

/* ILUB preconditioning: the split factors in BCSR form (Csr2Bcsr of the split
 * L/U of the AllocBlockZero pattern), bnl x bnw blocks; the template arguments
 * bnl/bnw of the reference are run-time arguments here.
 * senk::solver::IlubGmresm<T,bnl,bnw> (include/senk_gmres.hpp:582-588) */
int senk_ilub_gmres_d(const double *val, const int *cind, const int *rptr,
                      const double *blval, const int *blcind, const int *blrptr,
                      const double *buval, const int *bucind, const int *burptr,
                      const double *b, double *x, double nrm_b,
                      int outer, int m, int N, double epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res);
/* senk::solver::AbmcIlubGmresm<T,bnl,bnw> (include/senk_gmres.hpp:679-686) */
int senk_abmc_ilub_gmres_d(const double *val, const int *cind, const int *rptr,
                           const double *blval, const int *blcind, const int *blrptr,
                           const double *buval, const int *bucind, const int *burptr,
                           const int *cptr, int cnum, int bsize,
                           const double *b, double *x, double nrm_b,
                           int outer, int m, int N, double epsilon, int bnl, int bnw,
                           const senk_options *opt, senk_result *res);

/* senk::solver::Gcrm<double> (include/senk_gcr.hpp:30-34). The residual is
 * tested at restarts only; res->iters = the i*m of the restart that met it. */
int senk_gcr_d(const double *val, const int *cind, const int *rptr,
               const double *b, double *x, double nrm_b,
               int outer, int m, int N, double epsilon,
               const senk_options *opt, senk_result *res);
/* senk::solver::IluGcrm<double> (include/senk_gcr.hpp:93-99) */
int senk_ilu_gcr_d(const double *val, const int *cind, const int *rptr,
                   const double *lval, const int *lcind, const int *lrptr,
                   const double *uval, const int *ucind, const int *urptr,
                   const double *b, double *x, double nrm_b,
                   int outer, int m, int N, double epsilon,
                   const senk_options *opt, senk_result *res);
/* senk::solver::Gcrm<float>, IluGcrm<float> (include/senk_gcr.hpp:30-34, 93-99) */
int senk_gcr_s(const float *val, const int *cind, const int *rptr,
               const float *b, float *x, float nrm_b,
               int outer, int m, int N, float epsilon,
               const senk_options *opt, senk_result *res);
int senk_ilu_gcr_s(const float *val, const int *cind, const int *rptr,
                   const float *lval, const int *lcind, const int *lrptr,
                   const float *uval, const int *ucind, const int *urptr,
                   const float *b, float *x, float nrm_b,
                   int outer, int m, int N, float epsilon,
                   const senk_options *opt, senk_result *res);
/* senk::solver::IlubGcrm<double,bnl,bnw> (include/senk_gcr.hpp:163-169) */
int senk_ilub_gcr_d(const double *val, const int *cind, const int *rptr,
                    const double *blval, const int *blcind, const int *blrptr,
                    const double *buval, const int *bucind, const int *burptr,
                    const double *b, double *x, double nrm_b,
                    int outer, int m, int N, double epsilon, int bnl, int bnw,
                    const senk_options *opt, senk_result *res);

/* senk::solver::Bicgstab<double> (include/senk_bicgstab.hpp:29-33) */
int senk_bicgstab_d(const double *val, const int *cind, const int *rptr,
                    const double *b, double *x, double nrm_b,
                    int max_iter, int N, double epsilon,
                    const senk_options *opt, senk_result *res);
/* senk::solver::Bicgstab<float>, IluBicgstab<float> (include/senk_bicgstab.hpp:29-33, 107-113) */
int senk_bicgstab_s(const float *val, const int *cind, const int *rptr,
                    const float *b, float *x, float nrm_b,
                    int max_iter, int N, float epsilon,
                    const senk_options *opt, senk_result *res);
int senk_ilu_bicgstab_s(const float *val, const int *cind, const int *rptr,
                        const float *lval, const int *lcind, const int *lrptr,
                        const float *uval, const int *ucind, const int *urptr,
                        const float *b, float *x, float nrm_b,
                        int max_iter, int N, float epsilon,
                        const senk_options *opt, senk_result *res);
/* senk::solver::IluBicgstab<double> (include/senk_bicgstab.hpp:107-113) */
int senk_ilu_bicgstab_d(const double *val, const int *cind, const int *rptr,
                        const double *lval, const int *lcind, const int *lrptr,
                        const double *uval, const int *ucind, const int *urptr,
                        const double *b, double *x, double nrm_b,
                        int max_iter, int N, double epsilon,
                        const senk_options *opt, senk_result *res);
/* IluBicgstab's arguments plus an ABMC colour schedule for the sweeps (new: the
 * reference pairs ABMC only with GMRES). */
int senk_abmc_ilu_bicgstab_d(const double *val, const int *cind, const int *rptr,
                             const double *lval, const int *lcind, const int *lrptr,
                             const double *uval, const int *ucind, const int *urptr,
                             const int *cptr, int cnum, int bsize,
                             const double *b, double *x, double nrm_b,
                             int max_iter, int N, double epsilon,
                             const senk_options *opt, senk_result *res);
/* senk::solver::IlubBicgstab<double,bnl,bnw> (include/senk_bicgstab.hpp:198-204) */
int senk_ilub_bicgstab_d(const double *val, const int *cind, const int *rptr,
                         const double *blval, const int *blcind, const int *blrptr,
                         const double *buval, const int *bucind, const int *burptr,
                         const double *b, double *x, double nrm_b,
                         int max_iter, int N, double epsilon, int bnl, int bnw,
                         const senk_options *opt, senk_result *res);

/* The FP32 forms (T = float) of the block, block-Jacobi and ILUB solvers:
 * senk::solver::Gmresm<float,bnl,bnw> (include/senk_gmres.hpp:113-117),
 * BjIluGmresm<float> (:487-494), IlubGmresm<float,bnl,bnw> (:582-588),
 * AbmcIlubGmresm<float,bnl,bnw> (:679-686), IlubGcrm<float,bnl,bnw>
 * (include/senk_gcr.hpp:163-169), IlubBicgstab<float,bnl,bnw>
 * (include/senk_bicgstab.hpp:198-204); arguments as in the _d forms. */
int senk_bcsr_gmres_s(const float *bval, const int *bcind, const int *brptr,
                      const float *b, float *x, float nrm_b,
                      int outer, int m, int N, float epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res);
int senk_bj_ilu_gmres_s(const float *val, const int *cind, const int *rptr,
                        const float *lval, const int *lcind, const int *lrptr,
                        const float *uval, const int *ucind, const int *urptr, int bnum,
                        const float *b, float *x, float nrm_b,
                        int outer, int m, int N, float epsilon,
                        const senk_options *opt, senk_result *res);
int senk_ilub_gmres_s(const float *val, const int *cind, const int *rptr,
                      const float *blval, const int *blcind, const int *blrptr,
                      const float *buval, const int *bucind, const int *burptr,
                      const float *b, float *x, float nrm_b,
                      int outer, int m, int N, float epsilon, int bnl, int bnw,
                      const senk_options *opt, senk_result *res);
int senk_abmc_ilub_gmres_s(const float *val, const int *cind, const int *rptr,
                           const float *blval, const int *blcind, const int *blrptr,
                           const float *buval, const int *bucind, const int *burptr,
                           const int *cptr, int cnum, int bsize,
                           const float *b, float *x, float nrm_b,
                           int outer, int m, int N, float epsilon, int bnl, int bnw,
                           const senk_options *opt, senk_result *res);
int senk_ilub_gcr_s(const float *val, const int *cind, const int *rptr,
                    const float *blval, const int *blcind, const int *blrptr,
                    const float *buval, const int *bucind, const int *burptr,
                    const float *b, float *x, float nrm_b,
                    int outer, int m, int N, float epsilon, int bnl, int bnw,
                    const senk_options *opt, senk_result *res);
int senk_ilub_bicgstab_s(const float *val, const int *cind, const int *rptr,
                         const float *blval, const int *blcind, const int *blrptr,
                         const float *buval, const int *bucind, const int *burptr,
                         const float *b, float *x, float nrm_b,
                         int max_iter, int N, float epsilon, int bnl, int bnw,
                         const senk_options *opt, senk_result *res);

/* ================================================ device-resident systems ==
 * Upload once, solve many times (the timed path of the benchmark). */
typedef struct senk_system senk_system;

#define SENK_F64 0
#define SENK_F32 1

typedef struct {
    int N;
    int dtype;                 /* SENK_F64 or SENK_F32: type of every value array */
    const void *val; const int *cind; const int *rptr;   /* A (CSR, host) */
    int precond;               /* SENK_PC_* */
    const void *lval; const int *lcind; const int *lrptr; /* split L (host) */
    const void *uval; const int *ucind; const int *urptr; /* split U (host) */
    const int *cptr; int cnum; int bsize;                 /* colour schedule */
    int m_max;                 /* largest restart length to be used (<= 63) */
    int mixed;                 /* 1 (SENK_F64 systems): also build the FP32 copies
                                  (A, factors, Krylov basis) used by GMRES-IR;
                                  2: GMRES-IR only: the FP64 part keeps A (SELL)
                                  for residuals and no preconditioner or basis */
    int bnl, bnw;              /* SENK_PC_ILUB*: block shape; l* and u* then hold
                                  the BCSR factors (bval, bcind, brptr) */
} senk_system_desc;

int senk_system_create(senk_system **out, const senk_system_desc *desc, const senk_options *opt);
int senk_system_destroy(senk_system *sys);
/* The CUDA stream (cudaStream_t) every operation of this system runs on. */
void *senk_system_stream(senk_system *sys);
/* Copy b and the initial x from host memory (x may be NULL for x0 = 0). */
int senk_system_set_rhs(senk_system *sys, const void *b, const void *x0);
/* Read the current x back to host memory. */
int senk_system_get_x(senk_system *sys, void *x);
/* x = 0 on the device (enqueued on the system's stream). */
int senk_system_zero_x(senk_system *sys);
/* Device pointers of b and x (type of desc->dtype), for callers that fill them. */
void *senk_system_b(senk_system *sys);
void *senk_system_x(senk_system *sys);
/* Restarted GMRES(m) on the resident system (right-preconditioned when the system
 * has a preconditioner): include/senk_gmres.hpp:33-95 / 197-270 / 293-367 /
 * 391-465. */
int senk_system_gmres(senk_system *sys, double nrm_b, int outer, int m, double epsilon,
                      senk_result *res);

/* Mixed-precision GMRES iterative refinement on a system created with
 * desc->mixed = 1 (new: the reference has only commented-out FP32/FP64 refinement
 * prototypes, include/senk_bicgstab.hpp:269-296). Outer loop in FP64: r = b - A x,
 * stop when ||r|| <= epsilon * nrm_b (the FP64 true residual), else solve
 * A d = r / ||r|| with FP32 right-preconditioned GMRES(m) (FP32 A, ILU factors,
 * sweeps and Krylov basis; FP64 Hessenberg/Givens) to inner_tol or
 * inner_cycles restart cycles, and x += ||r|| d in FP64. res->iters counts inner
 * iterations, res->cycles outer steps, res->res is the final FP64 true residual. */
int senk_system_gmres_ir(senk_system *sys, double nrm_b, int max_outer, int m, double epsilon,
                         double inner_tol, int inner_cycles, senk_result *res);

/* Restarted GCR(m) on the resident system (include/senk_gcr.hpp:30-91 /
 * 93-161, and IlubGcrm :163-231 for ILUB systems): one CUDA graph per restart
 * cycle. */
int senk_system_gcr(senk_system *sys, double nrm_b, int outer, int m, double epsilon,
                    senk_result *res);
/* y = K x with the system's preconditioner (ILU or ILUB application, the
 * reference's SptrsvCsr_l/_u or SptrsvBcsr_l/_u pair as its solvers apply it,
 * e.g. include/senk_gcr.hpp:119-120); x and y are device vectors of the
 * system's dtype. Synchronous; reports a sweep whose bounded wait ran out. */
int senk_system_apply_pc(senk_system *sys, const void *x, void *y);
/* y = A x with the system's own SpMV (the format opt.spmv chose: SELL-32-sigma,
 * SELL-32 or CSR; senk::sparse::SpmvCsr, include/senk_sparse.hpp:25-35, and
 * SpmvSell, :103-121, as its solvers apply it); x and y are device vectors of
 * the system's dtype. Synchronous. */
int senk_system_apply_a(senk_system *sys, const void *x, void *y);
/* Mixed-precision GCR iterative refinement on a system created with
 * desc->mixed = 1 (new, like senk_system_gmres_ir): FP64 outer residual
 * r = b - A x and update x += ||r|| d, stopping on the FP64 true residual
 * (||r|| <= epsilon * nrm_b); d from FP32 GCR(m) (the reference's IluGcrm /
 * IlubGcrm recurrence, include/senk_gcr.hpp:93-231, on FP32 A, factors and
 * vectors) to inner_tol or inner_cycles restart cycles. res as for GMRES-IR. */
int senk_system_gcr_ir(senk_system *sys, double nrm_b, int max_outer, int m, double epsilon,
                       double inner_tol, int inner_cycles, senk_result *res);
/* BiCGStab on the resident system (include/senk_bicgstab.hpp:29-105 / 107-196):
 * one CUDA graph per iteration, launched a few at a time; res->iters is exact. */
int senk_system_bicgstab(senk_system *sys, double nrm_b, int max_iter, double epsilon,
                         senk_result *res);

/* Times `reps` back-to-back runs of one operation of the system's solve path on
 * its stream with CUDA events (after one untimed run). Reports the mean time of
 * one run and its algorithmic bytes (matrix values and indices once, each vector
 * read or written once). */
#define SENK_OP_SPMV 0      /* y = A x with the solve's SpMV format */
#define SENK_OP_PRECOND 1   /* t = U^-1 L^-1 v, all colours of both sweeps */
#define SENK_OP_SWEEP_L 2   /* the L sweep alone */
#define SENK_OP_SWEEP_U 3   /* the U sweep alone (in place) */
#define SENK_OP_DOT 4       /* one dot product of two vectors */
#define SENK_OP_MULTIDOT 5  /* the Arnoldi step's dot products: 16 basis vectors with w */
#define SENK_OP_UPDATE 6    /* the Arnoldi step's update w -= V c over 16 basis vectors, with ||w|| */
#define SENK_OP_INNER 16    /* added to an op: the FP32 copy of a mixed system */
int senk_system_time_op(senk_system *sys, int op, int reps, double *ms_per_rep, long long *bytes_per_rep);

/* ==================================================== device memory ======
 * For host code that stages arrays without CUDA headers (the drop-in headers). */
int senk_mem_alloc(void **p, size_t bytes);
int senk_mem_free(void *p);
int senk_mem_h2d(void *dst, const void *src, size_t bytes);  /* synchronous */
int senk_mem_d2h(void *dst, const void *src, size_t bytes);  /* synchronous */
int senk_mem_sync(void);
/* 1: device or managed memory; 0: host memory; < 0: error */
int senk_mem_is_device(const void *p);

/* ================================================ device kernels (one op) ==
 * Device pointers; stream is a cudaStream_t (NULL = legacy default stream). */

/* senk::sparse::SpmvCsr<T> (include/senk_sparse.hpp:25-35): y = A x */
int senk_dev_spmv_csr_d(const double *val, const int *cind, const int *rptr,
                        const double *x, double *y, int N, int nnz, void *stream);
int senk_dev_spmv_csr_s(const float *val, const int *cind, const int *rptr,
                        const float *x, float *y, int N, int nnz, void *stream);
/* senk::sparse::SpmvCsr<T> with diag (include/senk_sparse.hpp:47-57) */
int senk_dev_spmv_csr_diag_d(const double *val, const int *cind, const int *rptr,
                             const double *diag, const double *x, double *y, int N, void *stream);
/* senk::sparse::SpmvBcsr<T,bnl,bnw> (include/senk_sparse.hpp:70-91); supported
 * block shapes: 1x1, 2x2, 3x3, 4x4, 8x1, 4x1, 2x1 */
int senk_dev_spmv_bcsr_d(const double *bval, const int *bcind, const int *brptr,
                         const double *x, double *y, int N, int bnl, int bnw, void *stream);
/* senk::sparse::SpmvSell<T> (include/senk_sparse.hpp:103-121) on the layout of
 * senk::matrix::Csr2Sell (include/senk_matrix.hpp:90-142) */
int senk_dev_spmv_sell_d(const double *val, const int *cind, const int *wid, int len,
                         const double *x, double *y, int N, void *stream);

/* senk::blas1::Dot / Nrm2 (include/senk_blas1.hpp:92-112); result to host */
int senk_dev_dot_d(const double *x, const double *y, int N, double *result, void *stream);
int senk_dev_nrm2_d(const double *x, int N, double *result, void *stream);
/* Column dot products out[k] = V_k . w for k < nv (V_k = V + k*ldv; all device
 * pointers, out holds nv doubles), computed without allocating device memory.
 * No counterpart in the reference. It is for callers that cannot allocate at the
 * point of the call: applications that hand all GPU memory to their own pool at
 * start-up and forbid later cudaMalloc, and latency-critical loops where
 * cudaMalloc/cudaFree could synchronise the device. Same kernel as
 * senk_dev_dot_d per column; the CTA partition can differ, so results agree to
 * rounding, not bit for bit. Its reduction scratch is a fixed 39,168-byte
 * array inside the library's device image, held by every GPU that loads the
 * library until the process exits. Limits: 1 <= nv <= 16 (other values return
 * SENK_ERR_ARG); at most 304 CTAs per column block. The first call on each
 * device looks up that array's device address and keeps it for the life of the
 * process; make it before any stream capture, and do not call cudaDeviceReset
 * between calls. All calls share the one array (each call clears what must
 * start at zero), so calls that overlap on the GPU, e.g. on two streams at
 * once, race and give wrong results. */
int senk_dev_multidot_d_noalloc(const double *V, long long ldv, int nv, const double *w, int N,
                                double *out, void *stream);
/* senk::blas1::HadProd / HadDiv (include/senk_blas1.hpp:120-136): y *= x, y /= x */
int senk_dev_hadprod_d(const double *x, double *y, int N, void *stream);
int senk_dev_haddiv_d(const double *x, double *y, int N, void *stream);
/* senk::blas1::Axpy / Axpby / Axpyz / Scal / Copy (include/senk_blas1.hpp:26-83) */
int senk_dev_axpy_d(double a, const double *x, double *y, int N, void *stream);
int senk_dev_axpby_d(double a, const double *x, double b, double *y, int N, void *stream);
int senk_dev_axpyz_d(double a, const double *x, const double *y, double *z, int N, void *stream);
int senk_dev_scal_d(double a, double *x, int N, void *stream);
int senk_dev_copy_d(const double *x, double *y, int N, void *stream);

/* ILU sweep plan: the split factors re-laid out for colour-by-colour sweeps.
 * Replaces the reference's sweeps SptrsvCsr_l/_u: sequential
 * (include/senk_sparse.hpp:132-167, run by level sets), AMC (:180-236) and
 * ABMC (:250-315). Factor arrays are host memory, dtype SENK_F64/SENK_F32. */
typedef struct senk_ilu_plan senk_ilu_plan;
int senk_ilu_plan_create(senk_ilu_plan **out, int dtype, int N,
                         const void *lval, const int *lcind, const int *lrptr,
                         const void *uval, const int *ucind, const int *urptr,
                         int precond, const int *cptr, int cnum, int bsize);
/* The same plan for BCSR (ILUB) factors, FP64: SptrsvBcsr_l/_u
 * (include/senk_sparse.hpp:392-465; with cptr, the ABMC forms 481-581, cptr
 * counting blocks of bsize rows). The factors are checked against the schedule:
 * a block row that would read a row the schedule has not finished is rejected. */
int senk_ilub_plan_create(senk_ilu_plan **out, int N, int bnl, int bnw,
                          const double *blval, const int *blcind, const int *blrptr,
                          const double *buval, const int *bucind, const int *burptr,
                          const int *cptr, int cnum, int bsize);
/* senk_ilu_plan_create with the sweep schedule of AMC/ABMC factors chosen
 * (SENK_SWEEP_*). The natural order always runs level set by level set. */
int senk_ilu_plan_create_sched(senk_ilu_plan **out, int dtype, int N,
                               const void *lval, const int *lcind, const int *lrptr,
                               const void *uval, const int *ucind, const int *urptr,
                               int precond, const int *cptr, int cnum, int bsize, int sweep);
/* y = U^-1 L^-1 x (device vectors of the plan's dtype); x == y allowed.
 * Enqueued on `stream` without waiting: a sweep whose bounded wait ran out
 * (it then leaves y incomplete) is reported by senk_ilu_plan_status. */
int senk_ilu_plan_apply(senk_ilu_plan *plan, const void *x, void *y, void *stream);
/* One triangular sweep: y = L^-1 x (upper=0) or y = U^-1 x (upper=1). */
int senk_ilu_plan_sweep(senk_ilu_plan *plan, int upper, const void *x, void *y, void *stream);
/* Waits for the device, then returns SENK_ERR_CUDA (with a message naming the
 * wait) if a sweep of this plan gave up on a bounded wait since the last call,
 * else SENK_OK; the report is cleared. */
int senk_ilu_plan_status(senk_ilu_plan *plan, void *stream);
/* For tests of the error path: makes `group` of the dataflow sweep (upper = 0:
 * L, 1: U) wait on its own flag, which is never set before the group runs, so
 * its bounded wait runs out (about a second) on the next sweep. For the
 * cooperative sweep (SENK_SWEEP_PERSISTENT; `group` ignored) the first grid
 * barrier of the sweep's first cooperative launch waits for more arrivals than
 * there are CTAs. The
 * plan keeps this defect; destroy it afterwards. */
int senk_ilu_plan_test_stall(senk_ilu_plan *plan, int upper, int group);
int senk_ilu_plan_destroy(senk_ilu_plan *plan);

/* ============================================= learned preconditioner ==
 * New (no counterpart in the reference): a message-passing network over the
 * matrix graph (4 layers, hidden 64; node features a_ii, sum_j |a_ij| and the
 * residual) whose output corrects the ILU application inside flexible GCR(m):
 *     K(r) = ILU(r) + (||r||_rms / mean a_ii) * net(r).
 * Node MLPs run as BF16 tcgen05 GEMMs with FP32 accumulation; aggregation is a
 * CSR SpMM. Parameters are senk_mpnn_num_params() FP32 values:
 * W_in[3][64], b_in[64], then per layer Theta[128][64], beta[64], then w_out[64],
 * b_out. Vectors passed to the functions below are device vectors of the bound
 * (FP64, ILU-preconditioned) system. */
typedef struct senk_mpnn senk_mpnn;
int senk_mpnn_num_params(void);
int senk_mpnn_create(senk_mpnn **out, const float *params, int nparams);
int senk_mpnn_destroy(senk_mpnn *net);
int senk_mpnn_get_params(senk_mpnn *net, float *params, int nparams);
int senk_mpnn_set_params(senk_mpnn *net, const float *params, int nparams);
/* Graph data (row-normalised |A| off-diagonal, its transpose, diagonal and row
 * sums) and activations for the system's matrix. */
int senk_mpnn_bind(senk_mpnn *net, senk_system *sys);
/* Training objective: 1 (default) residual space, q = (r - A ILU(r)) / ||r||_rms,
 * loss = |A c / mean(a_ii) - q|^2 / |q|^2 with c = net(r); 0 error space,
 * t = (e - ILU(r)) mean(a_ii) / ||r||_rms, loss = |c - t|^2 / |t|^2. */
int senk_mpnn_set_loss(senk_mpnn *net, int mode);
/* Global gradient-norm clip of the Adam steps (default 1; <= 0: off). */
int senk_mpnn_set_clip(senk_mpnn *net, float clip);
/* Step of the correction (the GCR hook and senk_mpnn_apply): 1 (default)
 * K(r) = ILU(r) + alpha c, alpha = argmin |r - A(ILU(r) + alpha c)|, computed on
 * the device (one extra SpMV pair and a reduction per application), so that one
 * application never leaves a larger residual than ILU(r) alone; 0 K(r) = ILU(r)
 * + c. */
int senk_mpnn_set_step(senk_mpnn *net, int mode);
/* Loss of one residual/error pair; gradient to grad (host, may be NULL). */
int senk_mpnn_loss_grad(senk_mpnn *net, senk_system *sys, const double *r, const double *e, double *loss,
                        float *grad);
/* loss_grad, then one Adam step (beta 0.9 / 0.999, eps 1e-8) with rate lr. */
int senk_mpnn_train_step(senk_mpnn *net, senk_system *sys, const double *r, const double *e, float lr,
                         double *loss);
/* out = K(r) (device vectors), with the step mode set by senk_mpnn_set_step. */
int senk_mpnn_apply(senk_mpnn *net, senk_system *sys, const double *r, double *out);
/* Use K in the system's GCR (net NULL: plain ILU again). When a restart cycle
 * reduces the residual by less than `stall`, the solve falls back to plain ILU
 * for its remaining cycles; senk_system_learned_fallback gives that cycle. */
int senk_system_set_learned(senk_system *sys, senk_mpnn *net, double stall);
int senk_system_learned_fallback(senk_system *sys);
/* The tensor-core products alone, for tests: C = A Bt^T (A n x K, Bt NO x K,
 * BF16; C FP32; K = 128 with NO = 64, or K = 64 with NO = 128; A, Bt and C
 * 16-byte aligned, else SENK_ERR_ARG) and
 * out[128][64] = X^T dZ (X n x 128, dZ n x 64, BF16). */
int senk_dev_gemm_bf16(const void *A, const void *Bt, float *C, int n, int K, int NO, void *stream);
int senk_dev_gemm_tn_bf16(const void *X, const void *dZ, float *out, int n, void *stream);

/* senk::matrix::Ilu0<T> (include/senk_matrix.hpp:418-448) on the device, in
 * place: val, cind, rptr are device arrays of a CSR matrix with sorted columns.
 * With cptr (host, cnum colours; AMC: bsize 1, ABMC: blocks of bsize rows) the
 * chains of each colour are factorised concurrently, one thread per chain; the
 * matrix must be in that colour order (a row reading a row of its own colour
 * outside its chain is rejected with SENK_ERR_ARG). cptr NULL: the natural
 * order, level set by level set (the pattern is read back to form them). Each
 * row performs the reference's operations in its order without FMA
 * contraction, so the factors equal Ilu0's bit for bit. A zero pivot returns
 * SENK_ERR_ZERO_PIVOT (the reference prints and exits). Synchronous. */
int senk_dev_ilu0_d(double *val, const int *cind, const int *rptr, int N,
                    const int *cptr, int cnum, int bsize, void *stream);
int senk_dev_ilu0_s(float *val, const int *cind, const int *rptr, int N,
                    const int *cptr, int cnum, int bsize, void *stream);

/* ================================================ device ABMC ordering ==
 * senk::graph::GetABMCPermutation(cind, rptr, ..., N, bsize, isSym = false,
 * "simple") (include/senk_graph.hpp:291-334) on a CSR pattern in device
 * memory; with bsize = 1 it is GetAMCPermutation(..., isSym = false)
 * (:250-277). The outputs are the reference's, identical: *num_color,
 * *size_color (host, malloc'd, num_color + 1 entries, in blocks; release with
 * senk_free), LP (new -> old) and RP (old -> new) in caller-provided device
 * arrays of N. Each colour is found by parallel rounds that give the same set
 * as the reference's index-order greedy sweep. Fails (SENK_ERR_ARG) when N is
 * not a multiple of bsize or a block has more than 128 neighbour blocks.
 * Synchronous. (The reference's "connect" blocking is a sequential
 * breadth-first search and stays on the host.) */
int senk_dev_abmc_ordering(const int *cind, const int *rptr, int N, int bsize, int *num_color, int **size_color,
                           int *LP, int *RP, void *stream);
/* senk::matrix::Reordering (include/senk_matrix.hpp:703-730) on the device:
 * out row i = row LP[i] with columns RP[c], sorted by column; oval/ocind hold
 * nnz entries, orptr N + 1 (all device). Bit-identical to the host function.
 * Synchronous. */
int senk_dev_reordering_d(const double *val, const int *cind, const int *rptr, const int *LP, const int *RP, int N,
                          double *oval, int *ocind, int *orptr, void *stream);
int senk_dev_reordering_s(const float *val, const int *cind, const int *rptr, const int *LP, const int *RP, int N,
                          float *oval, int *ocind, int *orptr, void *stream);

/* ===================================================== host setup (CPU) ==
 * The reference's setup functions, bit-exact, for callers without C++ headers.
 * Outputs are malloc'd; release them with senk_free. */
void senk_free(void *p);
/* senk::matrix::Ilu0<double> (include/senk_matrix.hpp:418-448), in place */
int senk_setup_ilu0(double *val, const int *cind, const int *rptr, int N);
/* senk::matrix::Split<double> (include/senk_matrix.hpp:257-333) */
int senk_setup_split(const double *val, const int *cind, const int *rptr,
                     double **lval, int **lcind, int **lrptr,
                     double **uval, int **ucind, int **urptr,
                     double **diag, int N, const char *key, int invDiag);
/* senk::graph::GetABMCPermutation (include/senk_graph.hpp:291-334) */
int senk_setup_abmc_permutation(const int *cind, const int *rptr, int *num_color,
                                int **size_color, int **LP, int **RP,
                                int N, int bsize, int isSym, const char *bmethod);
/* senk::graph::GetAMCPermutation (include/senk_graph.hpp:250-277) */
int senk_setup_amc_permutation(const int *cind, const int *rptr, int *num_color,
                               int **size_color, int **LP, int **RP, int N, int isSym);
/* senk::matrix::Reordering<double>(val, cind, rptr, LP, RP, N)
 * (include/senk_matrix.hpp:703-730), in place */
int senk_setup_reordering(double *val, int *cind, int *rptr, const int *LP, const int *RP, int N);
/* senk::matrix::Csr2Bcsr<double> (include/senk_matrix.hpp:144-211) */
int senk_setup_csr2bcsr(const double *val, const int *cind, const int *rptr,
                        double **bval, int **bcind, int **brptr, int N, int bnl, int bnw);
/* senk::matrix::AllocBlockZero<double> (include/senk_matrix.hpp:652-666) */
int senk_setup_alloc_block_zero(double **val, int **cind, int **rptr, int N, int bnl, int bnw);
/* senk::matrix::Ilup<double> / AllocLevelZero<double>
 * (include/senk_matrix.hpp:450-549 / 551-650) */
int senk_setup_ilup(double **val, int **cind, int **rptr, int N, int p);
int senk_setup_alloc_level_zero(double **val, int **cind, int **rptr, int N, int p);
/* senk::matrix::RemoveOffDiagonal<double> (include/senk_matrix.hpp:668-689) */
int senk_setup_remove_off_diagonal(double **val, int **cind, int **rptr, int N, int bnum);
/* senk::io::ReadMatrixMarket (include/senk_io.hpp:41-103): CSR of the file's
 * entries (a symmetric file's stored triangle; *symmetric = 1), rows sorted by
 * column; SENK_ERR_ARG (with the reason) for a file the reader rejects. */
int senk_io_read_matrix_market(const char *filename, double **val, int **cind, int **rptr, int *N, int *M,
                               int *symmetric, int remove_zeros);
/* senk::matrix::Expand<double> (include/senk_matrix.hpp:336-370): the full
 * matrix from its stored triangle, key "L" or "U" */
int senk_setup_expand(const double *tval, const int *tcind, const int *trptr, double **val, int **cind,
                      int **rptr, int N, const char *key);

/* ============================================= device diagonal scaling ==
 * The reference's GetDiag / Scaling (include/senk_matrix.hpp:391-416) on a CSR
 * matrix in device memory, and the symmetric scaling its driver applies
 * (main.cpp:65-73: d_i = 1 / sqrt|a_ii|, a_ij <- d_i a_ij d_j). Each value is
 * (ld[i] * a_ij) * rd[j], two roundings in the reference's order, so results
 * equal the host functions' bit for bit. A row without a diagonal entry gets
 * diag 0 (the reference leaves it unset). Asynchronous on `stream`. */
int senk_dev_get_diag_d(const double *val, const int *cind, const int *rptr, double *diag, int N, void *stream);
int senk_dev_get_diag_s(const float *val, const int *cind, const int *rptr, float *diag, int N, void *stream);
int senk_dev_scaling_d(double *val, const int *cind, const int *rptr, const double *ld, const double *rd, int N,
                       void *stream);
int senk_dev_scaling_s(float *val, const int *cind, const int *rptr, const float *ld, const float *rd, int N,
                       void *stream);
/* GetDiag, d = 1 / sqrt|d|, Scaling(d, d); `d` (N entries, device) receives the
 * scaling factors. */
int senk_dev_diag_scaling_d(double *val, const int *cind, const int *rptr, double *d, int N, void *stream);
int senk_dev_diag_scaling_s(float *val, const int *cind, const int *rptr, float *d, int N, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SENK_GPU_H */
