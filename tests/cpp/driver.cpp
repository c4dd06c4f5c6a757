// A SenK program written against the reference's header API, built with this
// repository's include/ and linked with libsenk_gpu.so. It solves the 2D Poisson
// problem on a 128 x 128 grid (b = A * 1, x0 = 0, 1e-8) with several solver
// families, and exercises senk::sparse / senk::blas1 on host arrays. The
// solvers print the reference's stdout lines; the checks print "# check ...".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "senk.hpp"
#include "senk_blas1.hpp"
#include "senk_sparse.hpp"
#include "senk_test.hpp"

namespace {

// 5-point Laplacian, lexicographic order, Dirichlet boundary; malloc'd like the
// reference's readers so that the realloc-based setup functions can take it.
void Poisson(int n, double **val, int **cind, int **rptr)
{
    const int N = n * n;
    *rptr = (int *)std::malloc(sizeof(int) * (N + 1));
    *val = (double *)std::malloc(sizeof(double) * 5 * N);
    *cind = (int *)std::malloc(sizeof(int) * 5 * N);
    int k = 0;
    (*rptr)[0] = 0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const int r = j * n + i;
            auto put = [&](int c, double v) { (*cind)[k] = c; (*val)[k++] = v; };
            if (j > 0) put(r - n, -1);
            if (i > 0) put(r - 1, -1);
            put(r, 4);
            if (i < n - 1) put(r + 1, -1);
            if (j < n - 1) put(r + n, -1);
            (*rptr)[r + 1] = k;
        }
}

double MaxRelDiff(const std::vector<double> &a, const std::vector<double> &b)
{
    double d = 0, s = 0;
    for (size_t i = 0; i < a.size(); i++) {
        d = std::fmax(d, std::fabs(a[i] - b[i]));
        s = std::fmax(s, std::fabs(b[i]));
    }
    return d / s;
}

}  // namespace

int main()
{
    const int n = 128, N = n * n;
    double *val;
    int *cind, *rptr;
    Poisson(n, &val, &cind, &rptr);
    std::vector<double> b(N), x(N), ones(N, 1.0);
    senk::sparse::SpmvCsr<double>(val, cind, rptr, ones.data(), b.data(), N);
    const double nrm_b = senk::blas1::Nrm2<double>(b.data(), N);
    // host check of the GPU SpMV and Nrm2
    {
        double s = 0, e = 0;
        for (int i = 0; i < N; i++) {
            double t = 0;
            for (int j = rptr[i]; j < rptr[i + 1]; j++) t += val[j];
            e = std::fmax(e, std::fabs(t - b[i]));
            s += t * t;
        }
        std::printf("# check spmv %e nrm2 %e\n", e, std::fabs(std::sqrt(s) - nrm_b) / nrm_b);
    }

    // ILU(0), natural order
    double *fval = (double *)std::malloc(sizeof(double) * rptr[N]);
    for (int i = 0; i < rptr[N]; i++) fval[i] = val[i];
    senk::matrix::Ilu0<double>(fval, cind, rptr, N);
    double *lval, *uval;
    int *lcind, *lrptr, *ucind, *urptr;
    senk::matrix::Split<double>(fval, cind, rptr, &lval, &lcind, &lrptr, &uval, &ucind, &urptr, nullptr, N, "L-DU",
                                true);

    std::printf("## IluGmresm\n");
    std::fill(x.begin(), x.end(), 0.0);
    senk::solver::IluGmresm<double>(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b.data(), x.data(), nrm_b,
                                    10000 / 30, 30, N, 1e-8);
    senk::test::RelativeResidualError(val, cind, rptr, b.data(), x.data(), N);

    std::printf("## IluBicgstab\n");
    std::fill(x.begin(), x.end(), 0.0);
    senk::solver::IluBicgstab<double>(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b.data(), x.data(),
                                      nrm_b, 10000, N, 1e-8);
    senk::test::RelativeResidualError(val, cind, rptr, b.data(), x.data(), N);

    std::printf("## IluGcrm\n");
    std::fill(x.begin(), x.end(), 0.0);
    senk::solver::IluGcrm<double>(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b.data(), x.data(), nrm_b,
                                  10000 / 20, 20, N, 1e-8);
    senk::test::RelativeResidualError(val, cind, rptr, b.data(), x.data(), N);

    // the sweeps of senk::sparse against a host loop in the reference's order
    {
        std::vector<double> v(N), t(N), y(N), want_t(N), want_y(N);
        for (int i = 0; i < N; i++) v[i] = std::sin(0.37 * i);
        senk::sparse::SptrsvCsr_l<double>(lval, lcind, lrptr, v.data(), t.data(), N);
        senk::sparse::SptrsvCsr_u<double>(uval, ucind, urptr, t.data(), y.data(), N);
        for (int i = 0; i < N; i++) {
            double s = v[i];
            for (int j = lrptr[i]; j < lrptr[i + 1]; j++) s -= lval[j] * want_t[lcind[j]];
            want_t[i] = s;
        }
        for (int i = N - 1; i >= 0; i--) {
            double s = want_t[i];
            for (int j = urptr[i + 1] - 1; j > urptr[i]; j--) s -= uval[j] * want_y[ucind[j]];
            want_y[i] = s * uval[urptr[i]];
        }
        std::printf("# check sptrsv_l %e sptrsv_u %e\n", MaxRelDiff(t, want_t), MaxRelDiff(y, want_y));
        const double d = senk::blas1::Dot<double>(v.data(), y.data(), N);
        double dh = 0;
        for (int i = 0; i < N; i++) dh += v[i] * y[i];
        std::printf("# check dot %e\n", std::fabs(d - dh) / std::fabs(dh));
    }

    // ABMC (bsize 16) ILU(0)
    int num_color, *size_color, *LP, *RP;
    senk::graph::GetABMCPermutation(cind, rptr, &num_color, &size_color, &LP, &RP, N, 16, false, "connect");
    double *aval = (double *)std::malloc(sizeof(double) * rptr[N]);
    int *acind = (int *)std::malloc(sizeof(int) * rptr[N]);
    int *arptr = (int *)std::malloc(sizeof(int) * (N + 1));
    for (int i = 0; i < rptr[N]; i++) { aval[i] = val[i]; acind[i] = cind[i]; }
    for (int i = 0; i <= N; i++) arptr[i] = rptr[i];
    senk::matrix::Reordering<double>(aval, acind, arptr, LP, RP, N);
    std::vector<double> br(N);
    for (int i = 0; i < N; i++) br[i] = b[LP[i]];
    double *rval = (double *)std::malloc(sizeof(double) * arptr[N]);
    for (int i = 0; i < arptr[N]; i++) rval[i] = aval[i];
    senk::matrix::Ilu0<double>(rval, acind, arptr, N);
    double *rl, *ru;
    int *rlc, *rlr, *ruc, *rur;
    senk::matrix::Split<double>(rval, acind, arptr, &rl, &rlc, &rlr, &ru, &ruc, &rur, nullptr, N, "L-DU", true);
    std::printf("## AbmcIluGmresm %d\n", num_color);
    std::fill(x.begin(), x.end(), 0.0);
    senk::solver::AbmcIluGmresm<double>(aval, acind, arptr, rl, rlc, rlr, ru, ruc, rur, size_color, num_color, 16,
                                        br.data(), x.data(), nrm_b, 10000 / 30, 30, N, 1e-8);
    senk::test::RelativeResidualError(aval, acind, arptr, br.data(), x.data(), N);

    // ILUB 8x1, natural order (AllocBlockZero + Ilu0 + Split + Csr2Bcsr)
    double *tval = (double *)std::malloc(sizeof(double) * rptr[N]);
    int *tcind = (int *)std::malloc(sizeof(int) * rptr[N]);
    int *trptr = (int *)std::malloc(sizeof(int) * (N + 1));
    for (int i = 0; i < rptr[N]; i++) { tval[i] = val[i]; tcind[i] = cind[i]; }
    for (int i = 0; i <= N; i++) trptr[i] = rptr[i];
    senk::matrix::AllocBlockZero<double>(&tval, &tcind, &trptr, N, 8, 1);
    senk::matrix::Ilu0<double>(tval, tcind, trptr, N);
    double *bl, *bu;
    int *blc, *blr, *buc, *bur;
    senk::matrix::Split<double>(tval, tcind, trptr, &bl, &blc, &blr, &bu, &buc, &bur, nullptr, N, "L-DU", true);
    double *blv, *buv;
    int *blcb, *blrb, *bucb, *burb;
    senk::matrix::Csr2Bcsr<double>(bl, blc, blr, &blv, &blcb, &blrb, N, 8, 1);
    senk::matrix::Csr2Bcsr<double>(bu, buc, bur, &buv, &bucb, &burb, N, 8, 1);
    std::printf("## IlubGmresm\n");
    std::fill(x.begin(), x.end(), 0.0);
    senk::solver::IlubGmresm<double, 8, 1>(val, cind, rptr, blv, blcb, blrb, buv, bucb, burb, b.data(), x.data(),
                                           nrm_b, 10000 / 30, 30, N, 1e-8);
    senk::test::RelativeResidualError(val, cind, rptr, b.data(), x.data(), N);
    std::printf("## done\n");
    return 0;
}
