/**
 * @file senk_sparse.hpp
 * @brief senk::sparse SpMV and triangular sweeps, computed on the GPU.
 *
 * Same templates and arguments as the reference's include/senk_sparse.hpp.
 * Arrays may be in host or device memory: host arrays are staged through
 * device buffers for the call, device arrays are used in place. Each call is
 * synchronous, like the reference's. The triangular sweeps build a sweep plan
 * for the factor on every call; a caller that sweeps the same factor many times
 * keeps a plan (senk_ilu_plan_create / senk_ilub_plan_create) instead.
 */
#ifndef SENK_SPARSE_HPP
#define SENK_SPARSE_HPP

#include <vector>

#include "senk_device.hpp"

namespace senk {

namespace sparse {

/** SpmvCsr<T> (reference include/senk_sparse.hpp:25-35): y = A x. */
template <typename T>
void SpmvCsr(T *val, int *cind, int *rptr, T *x, T *y, int N)
{
    const int nnz = device::LastPointer(rptr, N);
    device::Staged<T> v(val, nnz, true, false), xx(x, N, true, false), yy(y, N, false, true);
    device::Staged<int> c(cind, nnz, true, false), r(rptr, N + 1, true, false);
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_dev_spmv_csr_s(v.get(), c.get(), r.get(), xx.get(), yy.get(), N, nnz, nullptr),
                      "senk_dev_spmv_csr_s");
    } else {
        static_assert(device::IsDouble<T>::value, "SpmvCsr: T must be double or float");
        device::Check(senk_dev_spmv_csr_d(v.get(), c.get(), r.get(), xx.get(), yy.get(), N, nnz, nullptr),
                      "senk_dev_spmv_csr_d");
    }
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** SpmvCsr<T> with diag (:47-57): y = (A + diag) x, diag kept apart. */
template <typename T>
void SpmvCsr(T *val, int *cind, int *rptr, T *diag, T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "SpmvCsr(diag): the GPU library implements T = double");
    const int nnz = device::LastPointer(rptr, N);
    device::Staged<T> v(val, nnz, true, false), d(diag, N, true, false), xx(x, N, true, false),
        yy(y, N, false, true);
    device::Staged<int> c(cind, nnz, true, false), r(rptr, N + 1, true, false);
    device::Check(senk_dev_spmv_csr_diag_d(v.get(), c.get(), r.get(), d.get(), xx.get(), yy.get(), N, nullptr),
                  "senk_dev_spmv_csr_diag_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** SpmvBcsr<T,bnl,bnw> (:70-91): y = A x, A in BCSR. */
template <typename T, int bnl, int bnw>
void SpmvBcsr(T *bval, int *bcind, int *brptr, T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "SpmvBcsr: the GPU library implements T = double");
    const int nb = device::LastPointer(brptr, N / bnl);
    device::Staged<T> v(bval, (long long)nb * bnl * bnw, true, false), xx(x, N, true, false), yy(y, N, false, true);
    device::Staged<int> c(bcind, nb, true, false), r(brptr, N / bnl + 1, true, false);
    device::Check(senk_dev_spmv_bcsr_d(v.get(), c.get(), r.get(), xx.get(), yy.get(), N, bnl, bnw, nullptr),
                  "senk_dev_spmv_bcsr_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** SpmvSell<T> (:103-121): y = A x, A in the reference's SELL layout (Csr2Sell). */
template <typename T>
void SpmvSell(T *val, int *cind, int *wid, int len, T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "SpmvSell: the GPU library implements T = double");
    const int slices = (N + len - 1) / len;
    const long long ne = (long long)device::LastPointer(wid, slices) * len;
    device::Staged<T> v(val, ne, true, false), xx(x, N, true, false), yy(y, N, false, true);
    device::Staged<int> c(cind, ne, true, false), w(wid, slices + 1, true, false);
    device::Check(senk_dev_spmv_sell_d(v.get(), c.get(), w.get(), len, xx.get(), yy.get(), N, nullptr),
                  "senk_dev_spmv_sell_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

namespace detail {

// One CSR sweep through an ILU plan whose other factor is the identity.
template <typename T>
void Sweep(bool upper, T *val, int *cind, int *rptr, T *x, T *y, int N, int precond, int *cptr, int cnum,
           int bsize)
{
    const int nnz = device::LastPointer(rptr, N);
    device::HostView<T> hv(val, nnz);
    device::HostView<int> hc(cind, nnz), hr(rptr, N + 1);
    device::HostView<int> hp(cptr, cptr ? cnum + 1 : 0);
    // the identity partner: U = I (inverted diagonal 1) or L = 0 (no entries;
    // its value and column arrays are only placeholders)
    std::vector<T> one(N, T(1));
    std::vector<int> diag(N), ptr(N + 1), zero(N + 1, 0);
    for (int i = 0; i < N; i++) diag[i] = ptr[i] = i;
    ptr[N] = N;
    senk_ilu_plan *plan = nullptr;
    const int dtype = std::is_same<T, float>::value ? SENK_F32 : SENK_F64;
    if (upper)
        device::Check(senk_ilu_plan_create(&plan, dtype, N, one.data(), diag.data(), zero.data(), hv.get(), hc.get(),
                                           hr.get(), precond, hp.get(), cnum, bsize),
                      "senk_ilu_plan_create");
    else
        device::Check(senk_ilu_plan_create(&plan, dtype, N, hv.get(), hc.get(), hr.get(), one.data(), diag.data(),
                                           ptr.data(), precond, hp.get(), cnum, bsize),
                      "senk_ilu_plan_create");
    {
        device::Staged<T> xx(x, N, true, false), yy(y, N, x == y, true);
        device::Check(senk_ilu_plan_sweep(plan, upper ? 1 : 0, xx.get(), yy.get(), nullptr), "senk_ilu_plan_sweep");
        device::Check(senk_mem_sync(), "senk_mem_sync");
    }
    senk_ilu_plan_destroy(plan);
}

// One BCSR sweep through an ILUB plan whose other factor is the identity.
template <typename T, int bnl, int bnw>
void SweepB(bool upper, T *bval, int *bcind, int *brptr, T *x, T *y, int N, int *cptr, int cnum, int bsize)
{
    static_assert(device::IsDouble<T>::value, "SptrsvBcsr: the GPU library implements T = double");
    constexpr int rem = bnl / bnw, bs = bnl * bnw;
    const int nbr = N / bnl;
    const int nb = device::LastPointer(brptr, nbr);
    device::HostView<T> hv(bval, (long long)nb * bs);
    device::HostView<int> hc(bcind, nb), hr(brptr, nbr + 1), hp(cptr, cptr ? cnum + 1 : 0);
    // identity U: the diagonal square with 1 (inverted diagonal) on its diagonal
    std::vector<T> iv((size_t)nbr * rem * bs, T(0));
    std::vector<int> ic((size_t)nbr * rem), ir(nbr + 1), zero(nbr + 1, 0);
    for (int br = 0; br < nbr; br++) {
        ir[br] = br * rem;
        for (int q = 0; q < rem; q++) {
            ic[(size_t)br * rem + q] = br * rem + q;
            for (int j = 0; j < bnw; j++) iv[((size_t)br * rem + q) * bs + j * bnl + q * bnw + j] = T(1);
        }
    }
    ir[nbr] = nbr * rem;
    senk_ilu_plan *plan = nullptr;
    if (upper)
        device::Check(senk_ilub_plan_create(&plan, N, bnl, bnw, iv.data(), ic.data(), zero.data(), hv.get(),
                                            hc.get(), hr.get(), hp.get(), cnum, bsize),
                      "senk_ilub_plan_create");
    else
        device::Check(senk_ilub_plan_create(&plan, N, bnl, bnw, hv.get(), hc.get(), hr.get(), iv.data(), ic.data(),
                                            ir.data(), hp.get(), cnum, bsize),
                      "senk_ilub_plan_create");
    {
        device::Staged<T> xx(x, N, true, false), yy(y, N, x == y, true);
        device::Check(senk_ilu_plan_sweep(plan, upper ? 1 : 0, xx.get(), yy.get(), nullptr), "senk_ilu_plan_sweep");
        device::Check(senk_mem_sync(), "senk_mem_sync");
    }
    senk_ilu_plan_destroy(plan);
}

}  // namespace detail

/** SptrsvCsr_l<T> (:132-152): L y = x, L unit lower (diagonal not stored). */
template <typename T>
void SptrsvCsr_l(T *val, int *cind, int *rptr, T *x, T *y, int N)
{
    detail::Sweep<T>(false, val, cind, rptr, x, y, N, SENK_PC_ILU, nullptr, 0, 1);
}

/** SptrsvCsr_u<T> (:154-167): U y = x, inverted diagonal first in each row. */
template <typename T>
void SptrsvCsr_u(T *val, int *cind, int *rptr, T *x, T *y, int N)
{
    detail::Sweep<T>(true, val, cind, rptr, x, y, N, SENK_PC_ILU, nullptr, 0, 1);
}

/** SptrsvCsr_l<T> for an AMC-ordered factor (:180-212). */
template <typename T>
void SptrsvCsr_l(T *val, int *cind, int *rptr, T *x, T *y, int N, int *cptr, int cnum)
{
    detail::Sweep<T>(false, val, cind, rptr, x, y, N, SENK_PC_ILU_AMC, cptr, cnum, 1);
}

/** SptrsvCsr_u<T> for an AMC-ordered factor (:214-236). */
template <typename T>
void SptrsvCsr_u(T *val, int *cind, int *rptr, T *x, T *y, int N, int *cptr, int cnum)
{
    detail::Sweep<T>(true, val, cind, rptr, x, y, N, SENK_PC_ILU_AMC, cptr, cnum, 1);
}

/** SptrsvCsr_l<T> for an ABMC-ordered factor (:250-287). */
template <typename T>
void SptrsvCsr_l(T *val, int *cind, int *rptr, T *x, T *y, int N, int *cptr, int cnum, int bsize)
{
    detail::Sweep<T>(false, val, cind, rptr, x, y, N, SENK_PC_ILU_ABMC, cptr, cnum, bsize);
}

/** SptrsvCsr_u<T> for an ABMC-ordered factor (:289-315). */
template <typename T>
void SptrsvCsr_u(T *val, int *cind, int *rptr, T *x, T *y, int N, int *cptr, int cnum, int bsize)
{
    detail::Sweep<T>(true, val, cind, rptr, x, y, N, SENK_PC_ILU_ABMC, cptr, cnum, bsize);
}

/** SptrsvCsr_l<T> block Jacobi (:328-346): the level sets of the factor give the
 * same rows in the same order as the reference's per-block sweeps. */
template <typename T>
void SptrsvCsr_l(T *val, int *cind, int *rptr, T *x, T *y, int N, int bnum)
{
    (void)bnum;
    detail::Sweep<T>(false, val, cind, rptr, x, y, N, SENK_PC_ILU, nullptr, 0, 1);
}

/** SptrsvCsr_u<T> block Jacobi (:359-379). */
template <typename T>
void SptrsvCsr_u(T *val, int *cind, int *rptr, T *x, T *y, int N, int bnum)
{
    (void)bnum;
    detail::Sweep<T>(true, val, cind, rptr, x, y, N, SENK_PC_ILU, nullptr, 0, 1);
}

/** SptrsvBcsr_l<T,bnl,bnw> (:392-416). */
template <typename T, int bnl, int bnw>
void SptrsvBcsr_l(T *bval, int *bcind, int *brptr, T *x, T *y, int N)
{
    detail::SweepB<T, bnl, bnw>(false, bval, bcind, brptr, x, y, N, nullptr, 0, 0);
}

/** SptrsvBcsr_u<T,bnl,bnw> (:429-465). */
template <typename T, int bnl, int bnw>
void SptrsvBcsr_u(T *bval, int *bcind, int *brptr, T *x, T *y, int N)
{
    detail::SweepB<T, bnl, bnw>(true, bval, bcind, brptr, x, y, N, nullptr, 0, 0);
}

/** SptrsvBcsr_l<T,bnl,bnw> for an ABMC-ordered factor (:481-517). */
template <typename T, int bnl, int bnw>
void SptrsvBcsr_l(T *bval, int *bcind, int *brptr, T *x, T *y, int N, int *cptr, int cnum, int bsize)
{
    detail::SweepB<T, bnl, bnw>(false, bval, bcind, brptr, x, y, N, cptr, cnum, bsize);
}

/** SptrsvBcsr_u<T,bnl,bnw> for an ABMC-ordered factor (:533-581). */
template <typename T, int bnl, int bnw>
void SptrsvBcsr_u(T *bval, int *bcind, int *brptr, T *x, T *y, int N, int *cptr, int cnum, int bsize)
{
    detail::SweepB<T, bnl, bnw>(true, bval, bcind, brptr, x, y, N, cptr, cnum, bsize);
}

}  // namespace sparse

}  // namespace senk

#endif
