/**
 * @file senk_gmres.hpp
 * @brief senk::solver GMRES(m) family, solved on the GPU.
 *
 * Same templates, arguments and stdout lines as the reference's
 * include/senk_gmres.hpp. Each call uploads the host arrays, runs the restarted
 * GMRES on the GPU (libsenk_gpu.so) and writes x back. Instantiations the GPU
 * library does not provide fail at compile time.
 */
#ifndef SENK_GMRES_HPP
#define SENK_GMRES_HPP

#include "senk_device.hpp"

namespace senk {

namespace solver {

/** Gmresm<T> (reference include/senk_gmres.hpp:33-95): GMRES(m), no preconditioner. */
template <typename T>
void Gmresm(T *val, int *cind, int *rptr, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    senk_options o = device::Printing();
    o.orth = SENK_ORTH_MGS;  // the reference's Gram-Schmidt
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_gmres_s(val, cind, rptr, b, x, nrm_b, outer, m, N, epsilon, &o, nullptr), "senk_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "Gmresm: T must be double or float");
        device::Check(senk_gmres_d(val, cind, rptr, b, x, nrm_b, outer, m, N, epsilon, &o, nullptr), "senk_gmres_d");
    }
}

/** Gmresm<T,bnl,bnw> (:113-195): GMRES(m) on a BCSR matrix. */
template <typename T, int bnl, int bnw>
void Gmresm(T *bval, int *bcind, int *brptr, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    senk_options o = device::Printing();
    o.orth = SENK_ORTH_MGS;
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_bcsr_gmres_s(bval, bcind, brptr, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_bcsr_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "Gmresm<T,bnl,bnw>: T must be double or float");
        device::Check(senk_bcsr_gmres_d(bval, bcind, brptr, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_bcsr_gmres_d");
    }
}

/** IluGmresm<T> (:197-270): right ILU-preconditioned GMRES(m). */
template <typename T>
void IluGmresm(T *val, int *cind, int *rptr, T *lval, int *lcind, int *lrptr, T *uval, int *ucind, int *urptr, T *b,
               T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_ilu_gmres_s(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, outer,
                                       m, N, epsilon, &o, nullptr),
                      "senk_ilu_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "IluGmresm: T must be double or float");
        device::Check(senk_ilu_gmres_d(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, outer,
                                       m, N, epsilon, &o, nullptr),
                      "senk_ilu_gmres_d");
    }
}

/** AmcIluGmresm<T> (:293-367): sweeps colour by colour over AMC colours. */
template <typename T>
void AmcIluGmresm(T *val, int *cind, int *rptr, T *lval, int *lcind, int *lrptr, T *uval, int *ucind, int *urptr,
                  int *cptr, int cnum, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_amc_ilu_gmres_s(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum, b, x,
                                           nrm_b, outer, m, N, epsilon, &o, nullptr),
                      "senk_amc_ilu_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "AmcIluGmresm: T must be double or float");
        device::Check(senk_amc_ilu_gmres_d(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum, b, x,
                                           nrm_b, outer, m, N, epsilon, &o, nullptr),
                      "senk_amc_ilu_gmres_d");
    }
}

/** AbmcIluGmresm<T> (:391-465): sweeps colour by colour over ABMC blocks. */
template <typename T>
void AbmcIluGmresm(T *val, int *cind, int *rptr, T *lval, int *lcind, int *lrptr, T *uval, int *ucind, int *urptr,
                   int *cptr, int cnum, int bsize, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_abmc_ilu_gmres_s(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum,
                                            bsize, b, x, nrm_b, outer, m, N, epsilon, &o, nullptr),
                      "senk_abmc_ilu_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "AbmcIluGmresm: T must be double or float");
        device::Check(senk_abmc_ilu_gmres_d(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, cptr, cnum,
                                            bsize, b, x, nrm_b, outer, m, N, epsilon, &o, nullptr),
                      "senk_abmc_ilu_gmres_d");
    }
}

/** BjIluGmresm<T> (:487-580): block-Jacobi ILU with bnum diagonal blocks. */
template <typename T>
void BjIluGmresm(T *val, int *cind, int *rptr, T *lval, int *lcind, int *lrptr, T *uval, int *ucind, int *urptr,
                 int bnum, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_bj_ilu_gmres_s(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, bnum, b, x, nrm_b,
                                          outer, m, N, epsilon, &o, nullptr),
                      "senk_bj_ilu_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "BjIluGmresm: T must be double or float");
        device::Check(senk_bj_ilu_gmres_d(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, bnum, b, x, nrm_b,
                                          outer, m, N, epsilon, &o, nullptr),
                      "senk_bj_ilu_gmres_d");
    }
}

/** IlubGmresm<T,bnl,bnw> (:582-677): ILUB (BCSR factors). */
template <typename T, int bnl, int bnw>
void IlubGmresm(T *val, int *cind, int *rptr, T *blval, int *blcind, int *blrptr, T *buval, int *bucind,
                int *burptr, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_ilub_gmres_s(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b,
                                        outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_ilub_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "IlubGmresm: T must be double or float");
        device::Check(senk_ilub_gmres_d(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b,
                                        outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_ilub_gmres_d");
    }
}

/** AbmcIlubGmresm<T,bnl,bnw> (:679-776): ILUB on an ABMC-ordered system. */
template <typename T, int bnl, int bnw>
void AbmcIlubGmresm(T *val, int *cind, int *rptr, T *blval, int *blcind, int *blrptr, T *buval, int *bucind,
                    int *burptr, int *cptr, int cnum, int bsize, T *b, T *x, T nrm_b, int outer, int m, int N,
                    T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_abmc_ilub_gmres_s(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, cptr,
                                             cnum, bsize, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_abmc_ilub_gmres_s");
    } else {
        static_assert(device::IsDouble<T>::value, "AbmcIlubGmresm: T must be double or float");
        device::Check(senk_abmc_ilub_gmres_d(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, cptr,
                                             cnum, bsize, b, x, nrm_b, outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_abmc_ilub_gmres_d");
    }
}

}  // namespace solver

}  // namespace senk

#endif
