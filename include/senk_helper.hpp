/**
 * @file senk_helper.hpp
 * @brief Co-sorting helpers of the SenK API (drop-in for include/senk_helper.hpp).
 *
 * QuickSort / QuickSortDesc sort the inclusive range [left, right] of `key` and
 * apply the same permutation to the companion arrays. The API callers (row
 * sorts in Reordering and the blocking step of the ABMC ordering) sort distinct
 * keys or plain integers, where every correct sort yields the same arrays, so the
 * implementation here is a plain index sort rather than the reference's
 * recursive quicksort.
 */
#ifndef SENK_HELPER_HPP
#define SENK_HELPER_HPP

#include <algorithm>
#include <numeric>
#include <vector>

namespace senk {
namespace helper {

/** Exchange two values. */
template <typename T>
void Swap(T *a, T *b)
{
    T t = *a;
    *a = *b;
    *b = t;
}

namespace detail {
template <typename T, typename Cmp, typename... Subs>
void co_sort(T *key, int left, int right, Cmp cmp, Subs *...subs)
{
    if (right <= left) return;
    const int n = right - left + 1;
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return cmp(key[left + a], key[left + b]); });
    auto apply = [&](auto *arr) {
        using V = std::remove_pointer_t<decltype(arr)>;
        std::vector<V> tmp(n);
        for (int i = 0; i < n; i++) tmp[i] = arr[left + ord[i]];
        std::copy(tmp.begin(), tmp.end(), arr + left);
    };
    (apply(subs), ...);
    apply(key);
}
}  // namespace detail

/** Ascending sort of key[left..right]. */
template <typename T>
void QuickSort(T *key, int left, int right)
{
    if (right > left) std::sort(key + left, key + right + 1);
}
/** Ascending sort of key[left..right], permuting sub alike. */
template <typename T, typename T2>
void QuickSort(T *key, T2 *sub, int left, int right)
{
    detail::co_sort(key, left, right, [](const T &a, const T &b) { return a < b; }, sub);
}
/** Ascending sort of key[left..right], permuting sub and sub2 alike. */
template <typename T, typename T2, typename T3>
void QuickSort(T *key, T2 *sub, T3 *sub2, int left, int right)
{
    detail::co_sort(key, left, right, [](const T &a, const T &b) { return a < b; }, sub, sub2);
}
/** Descending sort of key[left..right]. */
template <typename T>
void QuickSortDesc(T *key, int left, int right)
{
    if (right > left) std::sort(key + left, key + right + 1, [](const T &a, const T &b) { return a > b; });
}
/** Descending sort of key[left..right], permuting sub alike. */
template <typename T, typename T2>
void QuickSortDesc(T *key, T2 *sub, int left, int right)
{
    detail::co_sort(key, left, right, [](const T &a, const T &b) { return a > b; }, sub);
}
/** Descending sort of key[left..right], permuting sub and sub2 alike. */
template <typename T, typename T2, typename T3>
void QuickSortDesc(T *key, T2 *sub, T3 *sub2, int left, int right)
{
    detail::co_sort(key, left, right, [](const T &a, const T &b) { return a > b; }, sub, sub2);
}

}  // namespace helper
}  // namespace senk

#endif
