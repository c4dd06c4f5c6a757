/**
 * @file senk_gcr.hpp
 * @brief senk::solver GCR(m) family, solved on the GPU (reference
 * include/senk_gcr.hpp: same templates, arguments and stdout lines).
 */
#ifndef SENK_GCR_HPP
#define SENK_GCR_HPP

#include "senk_device.hpp"

namespace senk {

namespace solver {

/** Gcrm<T> (reference include/senk_gcr.hpp:30-91). */
template <typename T>
void Gcrm(T *val, int *cind, int *rptr, T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_gcr_s(val, cind, rptr, b, x, nrm_b, outer, m, N, epsilon, &o, nullptr), "senk_gcr_s");
    } else {
        static_assert(device::IsDouble<T>::value, "Gcrm: T must be double or float");
        device::Check(senk_gcr_d(val, cind, rptr, b, x, nrm_b, outer, m, N, epsilon, &o, nullptr), "senk_gcr_d");
    }
}

/** IluGcrm<T> (:93-161). */
template <typename T>
void IluGcrm(T *val, int *cind, int *rptr, T *lval, int *lcind, int *lrptr, T *uval, int *ucind, int *urptr, T *b,
             T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_ilu_gcr_s(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, outer, m,
                                     N, epsilon, &o, nullptr),
                      "senk_ilu_gcr_s");
    } else {
        static_assert(device::IsDouble<T>::value, "IluGcrm: T must be double or float");
        device::Check(senk_ilu_gcr_d(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b, outer, m,
                                     N, epsilon, &o, nullptr),
                      "senk_ilu_gcr_d");
    }
}

/** IlubGcrm<T,bnl,bnw> (:163-231). */
template <typename T, int bnl, int bnw>
void IlubGcrm(T *val, int *cind, int *rptr, T *blval, int *blcind, int *blrptr, T *buval, int *bucind, int *burptr,
              T *b, T *x, T nrm_b, int outer, int m, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_ilub_gcr_s(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b,
                                      outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_ilub_gcr_s");
    } else {
        static_assert(device::IsDouble<T>::value, "IlubGcrm: T must be double or float");
        device::Check(senk_ilub_gcr_d(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x, nrm_b,
                                      outer, m, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_ilub_gcr_d");
    }
}

}  // namespace solver

}  // namespace senk

#endif
