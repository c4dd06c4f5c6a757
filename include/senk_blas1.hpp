/**
 * @file senk_blas1.hpp
 * @brief senk::blas1 vector operations, computed on the GPU (reference
 * include/senk_blas1.hpp). Arrays may be in host or device memory (host arrays
 * are staged for the call); each call is synchronous. Ggen and Grot act on two
 * scalars and stay on the host.
 */
#ifndef SENK_BLAS1_HPP
#define SENK_BLAS1_HPP

#include <cmath>

#include "senk_device.hpp"

namespace senk {

namespace blas1 {

/** Copy (:26-30): y = x. */
template <typename T>
void Copy(T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "Copy: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, false, true);
    device::Check(senk_dev_copy_d(xx.get(), yy.get(), N, nullptr), "senk_dev_copy_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** Scal (:38-42): x = a x. */
template <typename T>
void Scal(T a, T *x, int N)
{
    static_assert(device::IsDouble<T>::value, "Scal: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, true);
    device::Check(senk_dev_scal_d(a, xx.get(), N, nullptr), "senk_dev_scal_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** Axpy (:51-55): y = a x + y. */
template <typename T>
void Axpy(T a, T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "Axpy: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, true, true);
    device::Check(senk_dev_axpy_d(a, xx.get(), yy.get(), N, nullptr), "senk_dev_axpy_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** Axpby (:65-69): y = a x + b y. */
template <typename T>
void Axpby(T a, T *x, T b, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "Axpby: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, true, true);
    device::Check(senk_dev_axpby_d(a, xx.get(), b, yy.get(), N, nullptr), "senk_dev_axpby_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** Axpyz (:79-83): z = a x + y. */
template <typename T>
void Axpyz(T a, T *x, T *y, T *z, int N)
{
    static_assert(device::IsDouble<T>::value, "Axpyz: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, true, false), zz(z, N, z == x || z == y, true);
    device::Check(senk_dev_axpyz_d(a, xx.get(), yy.get(), zz.get(), N, nullptr), "senk_dev_axpyz_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** Dot (:92-98). */
template <typename T>
T Dot(T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "Dot: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, true, false);
    double r = 0;
    device::Check(senk_dev_dot_d(xx.get(), yy.get(), N, &r, nullptr), "senk_dev_dot_d");
    return r;
}

/** Nrm2 (:106-112). */
template <typename T>
T Nrm2(T *x, int N)
{
    static_assert(device::IsDouble<T>::value, "Nrm2: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false);
    double r = 0;
    device::Check(senk_dev_nrm2_d(xx.get(), N, &r, nullptr), "senk_dev_nrm2_d");
    return r;
}

/** HadProd (:120-124): y = y .* x. */
template <typename T>
void HadProd(T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "HadProd: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, true, true);
    device::Check(senk_dev_hadprod_d(xx.get(), yy.get(), N, nullptr), "senk_dev_hadprod_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** HadDiv (:132-136): y = y ./ x. */
template <typename T>
void HadDiv(T *x, T *y, int N)
{
    static_assert(device::IsDouble<T>::value, "HadDiv: the GPU library implements T = double");
    device::Staged<T> xx(x, N, true, false), yy(y, N, true, true);
    device::Check(senk_dev_haddiv_d(xx.get(), yy.get(), N, nullptr), "senk_dev_haddiv_d");
    device::Check(senk_mem_sync(), "senk_mem_sync");
}

/** Ggen (:145-153): the Givens rotation (c, s) that zeroes b under a; returns
 * the new a. */
template <typename T>
T Ggen(T a, T b, T *c, T *s)
{
    const T r = std::sqrt(a * a + b * b);
    *c = a / r;
    *s = -b / r;
    return r;
}

/** Grot (:162-168): applies the rotation (c, s) to the pair (a, b). */
template <typename T>
void Grot(T c, T s, T *a, T *b)
{
    const T a0 = *a, b0 = *b;
    *a = c * a0 - s * b0;
    *b = s * a0 + c * b0;
}

}  // namespace blas1

}  // namespace senk

#endif
