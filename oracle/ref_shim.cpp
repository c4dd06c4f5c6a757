// ORACLE — test infrastructure, not product code.
//
// extern "C" wrappers that instantiate the UNMODIFIED reference headers
// (sapporosaburo/SenK include/*.hpp, compiled where they lie by oracle/Makefile)
// so that tests can call the reference itself through ctypes.  The reference
// prints its convergence lines to stdout; the solver wrappers capture that text
// into a caller buffer so tests can parse "I iter N" / "# res r" exactly as the
// reference prints them.  Built into oracle/_ref/ only in a container that has the
// reference sources; nothing on the GPU path loads it.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <omp.h>
#include <unistd.h>

#include "senk.hpp"
#include "senk_test.hpp"

namespace {

// Run fn with stdout redirected into buf (NUL-terminated, truncated to cap).
template <typename F>
int capture_stdout(char *buf, int cap, F fn)
{
    fflush(stdout);
    FILE *tmp = tmpfile();
    if (!tmp) { fn(); return -1; }
    int saved = dup(1);
    dup2(fileno(tmp), 1);
    fn();
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
    long n = ftell(tmp);
    rewind(tmp);
    if (buf && cap > 0) {
        long k = n < cap - 1 ? n : cap - 1;
        size_t got = fread(buf, 1, (size_t)k, tmp);
        buf[got] = 0;
    }
    fclose(tmp);
    return 0;
}

// BCSR templates need compile-time block shapes; dispatch the shapes the tests use.
#define SENK_REF_BLOCK_SHAPES(X) X(1, 1) X(2, 1) X(2, 2) X(3, 3) X(4, 1) X(4, 2) X(8, 1) X(8, 2)

}  // namespace

extern "C" {

void ref_free(void *p) { free(p); }
void ref_set_threads(int n) { omp_set_num_threads(n); }

// ------------------------------------------------------------------- sparse
void ref_spmv_csr_d(double *v, int *c, int *r, double *x, double *y, int N) { senk::sparse::SpmvCsr<double>(v, c, r, x, y, N); }
void ref_spmv_csr_s(float *v, int *c, int *r, float *x, float *y, int N) { senk::sparse::SpmvCsr<float>(v, c, r, x, y, N); }
void ref_spmv_csr_diag_d(double *v, int *c, int *r, double *d, double *x, double *y, int N) { senk::sparse::SpmvCsr<double>(v, c, r, d, x, y, N); }
void ref_spmv_sell_d(double *v, int *c, int *w, int len, double *x, double *y, int N) { senk::sparse::SpmvSell<double>(v, c, w, len, x, y, N); }

int ref_spmv_bcsr_d(double *v, int *c, int *r, double *x, double *y, int N, int bnl, int bnw)
{
#define X(A, B) if (bnl == A && bnw == B) { senk::sparse::SpmvBcsr<double, A, B>(v, c, r, x, y, N); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

void ref_sptrsv_l_d(double *v, int *c, int *r, double *x, double *y, int N) { senk::sparse::SptrsvCsr_l<double>(v, c, r, x, y, N); }
void ref_sptrsv_u_d(double *v, int *c, int *r, double *x, double *y, int N) { senk::sparse::SptrsvCsr_u<double>(v, c, r, x, y, N); }
void ref_sptrsv_l_s(float *v, int *c, int *r, float *x, float *y, int N) { senk::sparse::SptrsvCsr_l<float>(v, c, r, x, y, N); }
void ref_sptrsv_u_s(float *v, int *c, int *r, float *x, float *y, int N) { senk::sparse::SptrsvCsr_u<float>(v, c, r, x, y, N); }
void ref_sptrsv_l_amc_d(double *v, int *c, int *r, double *x, double *y, int N, int *cp, int cn) { senk::sparse::SptrsvCsr_l<double>(v, c, r, x, y, N, cp, cn); }
void ref_sptrsv_u_amc_d(double *v, int *c, int *r, double *x, double *y, int N, int *cp, int cn) { senk::sparse::SptrsvCsr_u<double>(v, c, r, x, y, N, cp, cn); }
void ref_sptrsv_l_abmc_d(double *v, int *c, int *r, double *x, double *y, int N, int *cp, int cn, int bs) { senk::sparse::SptrsvCsr_l<double>(v, c, r, x, y, N, cp, cn, bs); }
void ref_sptrsv_u_abmc_d(double *v, int *c, int *r, double *x, double *y, int N, int *cp, int cn, int bs) { senk::sparse::SptrsvCsr_u<double>(v, c, r, x, y, N, cp, cn, bs); }
void ref_sptrsv_l_abmc_s(float *v, int *c, int *r, float *x, float *y, int N, int *cp, int cn, int bs) { senk::sparse::SptrsvCsr_l<float>(v, c, r, x, y, N, cp, cn, bs); }
void ref_sptrsv_u_abmc_s(float *v, int *c, int *r, float *x, float *y, int N, int *cp, int cn, int bs) { senk::sparse::SptrsvCsr_u<float>(v, c, r, x, y, N, cp, cn, bs); }
void ref_sptrsv_l_bj_d(double *v, int *c, int *r, double *x, double *y, int N, int bn) { senk::sparse::SptrsvCsr_l<double>(v, c, r, x, y, N, bn); }
void ref_sptrsv_u_bj_d(double *v, int *c, int *r, double *x, double *y, int N, int bn) { senk::sparse::SptrsvCsr_u<double>(v, c, r, x, y, N, bn); }

int ref_sptrsv_bcsr_d(int upper, double *v, int *c, int *r, double *x, double *y, int N, int bnl, int bnw)
{
#define X(A, B) if (bnl == A && bnw == B) { \
        if (upper) senk::sparse::SptrsvBcsr_u<double, A, B>(v, c, r, x, y, N); \
        else senk::sparse::SptrsvBcsr_l<double, A, B>(v, c, r, x, y, N); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

int ref_sptrsv_bcsr_abmc_d(int upper, double *v, int *c, int *r, double *x, double *y, int N,
                           int *cp, int cn, int bs, int bnl, int bnw)
{
#define X(A, B) if (bnl == A && bnw == B) { \
        if (upper) senk::sparse::SptrsvBcsr_u<double, A, B>(v, c, r, x, y, N, cp, cn, bs); \
        else senk::sparse::SptrsvBcsr_l<double, A, B>(v, c, r, x, y, N, cp, cn, bs); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

// -------------------------------------------------------------------- blas1
double ref_dot_d(double *x, double *y, int N) { return senk::blas1::Dot<double>(x, y, N); }
double ref_nrm2_d(double *x, int N) { return senk::blas1::Nrm2<double>(x, N); }

// ------------------------------------------------------------------ solvers
void ref_gmres_d(double *v, int *c, int *r, double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::Gmresm<double>(v, c, r, b, x, nb, outer, m, N, eps); }); }

void ref_ilu_gmres_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                     double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::IluGmresm<double>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, outer, m, N, eps); }); }

void ref_ilu_gmres_s(float *v, int *c, int *r, float *lv, int *lc, int *lr, float *uv, int *uc, int *ur,
                     float *b, float *x, float nb, int outer, int m, int N, float eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::IluGmresm<float>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, outer, m, N, eps); }); }

void ref_amc_ilu_gmres_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                         int *cp, int cn, double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::AmcIluGmresm<double>(v, c, r, lv, lc, lr, uv, uc, ur, cp, cn, b, x, nb, outer, m, N, eps); }); }

void ref_abmc_ilu_gmres_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                          int *cp, int cn, int bs, double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::AbmcIluGmresm<double>(v, c, r, lv, lc, lr, uv, uc, ur, cp, cn, bs, b, x, nb, outer, m, N, eps); }); }

void ref_bj_ilu_gmres_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                        int bn, double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::BjIluGmresm<double>(v, c, r, lv, lc, lr, uv, uc, ur, bn, b, x, nb, outer, m, N, eps); }); }

int ref_ilub_gmres_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                     double *b, double *x, double nb, int outer, int m, int N, double eps, int bnl, int bnw, char *out, int cap)
{
#define X(A, B) if (bnl == A && bnw == B) { capture_stdout(out, cap, [&] { \
        senk::solver::IlubGmresm<double, A, B>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, outer, m, N, eps); }); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

int ref_abmc_ilub_gmres_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                          int *cp, int cn, int bs, double *b, double *x, double nb, int outer, int m, int N, double eps,
                          int bnl, int bnw, char *out, int cap)
{
#define X(A, B) if (bnl == A && bnw == B) { capture_stdout(out, cap, [&] { \
        senk::solver::AbmcIlubGmresm<double, A, B>(v, c, r, lv, lc, lr, uv, uc, ur, cp, cn, bs, b, x, nb, outer, m, N, eps); }); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

int ref_bcsr_gmres_d(double *bv, int *bc, int *br, double *b, double *x, double nb, int outer, int m, int N, double eps,
                     int bnl, int bnw, char *out, int cap)
{
#define X(A, B) if (bnl == A && bnw == B) { capture_stdout(out, cap, [&] { \
        senk::solver::Gmresm<double, A, B>(bv, bc, br, b, x, nb, outer, m, N, eps); }); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

void ref_gcr_d(double *v, int *c, int *r, double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::Gcrm<double>(v, c, r, b, x, nb, outer, m, N, eps); }); }

void ref_ilu_gcr_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                   double *b, double *x, double nb, int outer, int m, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::IluGcrm<double>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, outer, m, N, eps); }); }

int ref_ilub_gcr_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                   double *b, double *x, double nb, int outer, int m, int N, double eps, int bnl, int bnw, char *out, int cap)
{
#define X(A, B) if (bnl == A && bnw == B) { capture_stdout(out, cap, [&] { \
        senk::solver::IlubGcrm<double, A, B>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, outer, m, N, eps); }); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

void ref_bicgstab_d(double *v, int *c, int *r, double *b, double *x, double nb, int it, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::Bicgstab<double>(v, c, r, b, x, nb, it, N, eps); }); }

void ref_ilu_bicgstab_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                        double *b, double *x, double nb, int it, int N, double eps, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::solver::IluBicgstab<double>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, it, N, eps); }); }

int ref_ilub_bicgstab_d(double *v, int *c, int *r, double *lv, int *lc, int *lr, double *uv, int *uc, int *ur,
                        double *b, double *x, double nb, int it, int N, double eps, int bnl, int bnw, char *out, int cap)
{
#define X(A, B) if (bnl == A && bnw == B) { capture_stdout(out, cap, [&] { \
        senk::solver::IlubBicgstab<double, A, B>(v, c, r, lv, lc, lr, uv, uc, ur, b, x, nb, it, N, eps); }); return 0; }
    SENK_REF_BLOCK_SHAPES(X)
#undef X
    return -1;
}

// -------------------------------------------------------------------- setup
int ref_check_structure(double *v, int *c, int *r, int N) { return senk::matrix::CheckStructure<double>(v, c, r, N) ? 1 : 0; }
void ref_csr2csc(double *v, int *c, int *r, double **cv, int **cr, int **cc, int N, int M) { senk::matrix::Csr2Csc<double>(v, c, r, cv, cr, cc, N, M); }
int ref_csr2sell(double *v, int *c, int *r, double **sv, int **sc, int **sl, int size, int N) { return senk::matrix::Csr2Sell<double>(v, c, r, sv, sc, sl, size, N); }
void ref_csr2bcsr(double *v, int *c, int *r, double **bv, int **bc, int **br, int N, int bnl, int bnw) { senk::matrix::Csr2Bcsr<double>(v, c, r, bv, bc, br, N, bnl, bnw); }
int ref_bcsr2csr(double *bv, int *bc, int *br, double **v, int **c, int **r, int N, int bnl, int bnw) { return senk::matrix::Bcsr2Csr<double>(bv, bc, br, v, c, r, N, bnl, bnw); }
void ref_split(double *v, int *c, int *r, double **lv, int **lc, int **lr, double **uv, int **uc, int **ur,
               double **d, int N, const char *key, int inv)
{ senk::matrix::Split<double>(v, c, r, lv, lc, lr, uv, uc, ur, d, N, key, inv != 0); }
void ref_get_diag(double *v, int *c, int *r, double **d, int N) { senk::matrix::GetDiag<double>(v, c, r, d, N); }
void ref_scaling(double *v, int *c, int *r, double *ld, double *rd, int N) { senk::matrix::Scaling<double>(v, c, r, ld, rd, N); }
void ref_ilu0(double *v, int *c, int *r, int N) { senk::matrix::Ilu0<double>(v, c, r, N); }
void ref_ilup(double **v, int **c, int **r, int N, int p) { senk::matrix::Ilup<double>(v, c, r, N, p); }
void ref_alloc_level_zero(double **v, int **c, int **r, int N, int p) { senk::matrix::AllocLevelZero<double>(v, c, r, N, p); }
void ref_alloc_block_zero(double **v, int **c, int **r, int N, int bnl, int bnw) { senk::matrix::AllocBlockZero<double>(v, c, r, N, bnl, bnw); }
void ref_remove_off_diagonal(double **v, int **c, int **r, int N, int bnum) { senk::matrix::RemoveOffDiagonal<double>(v, c, r, N, bnum); }
void ref_reordering(double *v, int *c, int *r, int *LP, int *RP, int N) { senk::matrix::Reordering<double>(v, c, r, LP, RP, N); }
void ref_reordering_cols(double *v, int *c, int *r, int *RP, int N) { senk::matrix::Reordering<double>(v, c, r, RP, N); }
void ref_amc_permutation(int *c, int *r, int *nc, int **sc, int **LP, int **RP, int N, int sym)
{ senk::graph::GetAMCPermutation(c, r, nc, sc, LP, RP, N, sym != 0); }
void ref_abmc_permutation(int *c, int *r, int *nc, int **sc, int **LP, int **RP, int N, int bs, int sym, const char *method)
{ senk::graph::GetABMCPermutation(c, r, nc, sc, LP, RP, N, bs, sym != 0, method); }
void ref_expand(double *tv, int *tc, int *tr, double **v, int **c, int **r, int N, const char *key)
{ senk::matrix::Expand<double>(tv, tc, tr, v, c, r, N, key); }
// senk::io::ReadMatrixMarket; its stdout lines go to `out`; returns its result
int ref_read_matrix_market(const char *path, double **v, int **c, int **r, int *N, int *M, int *sym, int rz,
                           char *out, int cap)
{
    bool ok = false;
    senk::io::Shape shape = senk::io::Unsym;
    capture_stdout(out, cap, [&] { ok = senk::io::ReadMatrixMarket(path, v, c, r, N, M, &shape, rz != 0); });
    *sym = shape == senk::io::Sym ? 1 : 0;
    return ok ? 0 : -1;
}
void ref_relative_residual(double *v, int *c, int *r, double *b, double *x, int N, char *out, int cap)
{ capture_stdout(out, cap, [&] { senk::test::RelativeResidualError(v, c, r, b, x, N); }); }

}  // extern "C"
