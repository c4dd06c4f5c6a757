/**
 * @file senk_bicgstab.hpp
 * @brief senk::solver BiCGStab family, solved on the GPU (reference
 * include/senk_bicgstab.hpp: same templates, arguments and stdout lines).
 */
#ifndef SENK_BICGSTAB_HPP
#define SENK_BICGSTAB_HPP

#include "senk_device.hpp"

namespace senk {

namespace solver {

/** Bicgstab<T> (reference include/senk_bicgstab.hpp:29-105). */
template <typename T>
void Bicgstab(T *val, int *cind, int *rptr, T *b, T *x, T nrm_b, int max_iter, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_bicgstab_s(val, cind, rptr, b, x, nrm_b, max_iter, N, epsilon, &o, nullptr),
                      "senk_bicgstab_s");
    } else {
        static_assert(device::IsDouble<T>::value, "Bicgstab: T must be double or float");
        device::Check(senk_bicgstab_d(val, cind, rptr, b, x, nrm_b, max_iter, N, epsilon, &o, nullptr),
                      "senk_bicgstab_d");
    }
}

/** IluBicgstab<T> (:107-196). */
template <typename T>
void IluBicgstab(T *val, int *cind, int *rptr, T *lval, int *lcind, int *lrptr, T *uval, int *ucind, int *urptr,
                 T *b, T *x, T nrm_b, int max_iter, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_ilu_bicgstab_s(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b,
                                          max_iter, N, epsilon, &o, nullptr),
                      "senk_ilu_bicgstab_s");
    } else {
        static_assert(device::IsDouble<T>::value, "IluBicgstab: T must be double or float");
        device::Check(senk_ilu_bicgstab_d(val, cind, rptr, lval, lcind, lrptr, uval, ucind, urptr, b, x, nrm_b,
                                          max_iter, N, epsilon, &o, nullptr),
                      "senk_ilu_bicgstab_d");
    }
}

/** IlubBicgstab<T,bnl,bnw> (:198-267). */
template <typename T, int bnl, int bnw>
void IlubBicgstab(T *val, int *cind, int *rptr, T *blval, int *blcind, int *blrptr, T *buval, int *bucind,
                  int *burptr, T *b, T *x, T nrm_b, int max_iter, int N, T epsilon)
{
    const senk_options o = device::Printing();
    if constexpr (std::is_same<T, float>::value) {
        device::Check(senk_ilub_bicgstab_s(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x,
                                           nrm_b, max_iter, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_ilub_bicgstab_s");
    } else {
        static_assert(device::IsDouble<T>::value, "IlubBicgstab: T must be double or float");
        device::Check(senk_ilub_bicgstab_d(val, cind, rptr, blval, blcind, blrptr, buval, bucind, burptr, b, x,
                                           nrm_b, max_iter, N, epsilon, bnl, bnw, &o, nullptr),
                      "senk_ilub_bicgstab_d");
    }
}

}  // namespace solver

}  // namespace senk

#endif
