/**
 * @file senk_utils.hpp
 * @brief Allocation and fill helpers of the SenK API (drop-in for
 *        include/senk_utils.hpp of sapporosaburo/SenK).
 *
 * Allocation failures print a message and exit(1), as the reference's Safe*
 * helpers do (senk_utils.hpp:22-64); outputs of setup functions are malloc'd so
 * callers release them with free().
 */
#ifndef SENK_UTILS_HPP
#define SENK_UTILS_HPP

#include <cstdio>
#include <cstdlib>

namespace senk {
namespace utils {

/** malloc of `size` elements; exits on failure (reference senk_utils.hpp:22-28). */
template <typename T>
T *SafeMalloc(int size)
{
    T *p = static_cast<T *>(std::malloc(sizeof(T) * (size_t)(size > 0 ? size : 1)));
    if (!p) { std::printf("Error: SafeMalloc\n"); std::exit(1); }
    return p;
}

/** calloc of `size` zeroed elements (senk_utils.hpp:34-40). */
template <typename T>
T *SafeCalloc(int size)
{
    T *p = static_cast<T *>(std::calloc((size_t)(size > 0 ? size : 1), sizeof(T)));
    if (!p) { std::printf("Error: SafeCalloc\n"); std::exit(1); }
    return p;
}

/** realloc to `size` elements (senk_utils.hpp:47-53). */
template <typename T>
T *SafeRealloc(T *old, int size)
{
    T *p = static_cast<T *>(std::realloc(old, sizeof(T) * (size_t)(size > 0 ? size : 1)));
    if (!p) { std::printf("Error: SafeRealloc\n"); std::exit(1); }
    return p;
}

/** free and null the pointer (senk_utils.hpp:59-64). */
template <typename T>
void SafeFree(T **ptr)
{
    if (*ptr) std::free(*ptr);
    *ptr = nullptr;
}

/** out[i] = in[i] (senk_utils.hpp:72-79). */
template <typename T>
void Copy(T *in, T *out, int size)
{
    for (int i = 0; i < size; i++) out[i] = in[i];
}

/** out[i] = val (senk_utils.hpp:87-94). */
template <typename T>
void Set(T val, T *out, int size)
{
    for (int i = 0; i < size; i++) out[i] = val;
}

/** out[i] = (T2)in[i], e.g. FP64 -> FP32 factors (senk_utils.hpp:103-110). */
template <typename T1, typename T2>
void Convert(T1 *in, T2 *out, int size)
{
    for (int i = 0; i < size; i++) out[i] = static_cast<T2>(in[i]);
}

}  // namespace utils
}  // namespace senk

#endif
