/**
 * @file senk_device.hpp
 * @brief Host-side glue between SenK's header API and libsenk_gpu.so.
 *
 * The reference's headers compute on host arrays. Their drop-in counterparts
 * here compute on the GPU through the C ABI (senk_gpu.h); this file holds what
 * they share: status checks with the reference's failure behaviour (print and
 * exit), and staging of arrays that may live in host or device memory.
 */
#ifndef SENK_DEVICE_HPP
#define SENK_DEVICE_HPP

#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "senk_gpu.h"

namespace senk {

namespace device {

/** Prints the library's message and exits, as the reference does on errors. */
inline void Check(int rc, const char *fn)
{
    if (rc != SENK_OK && rc != SENK_ERR_BREAKDOWN) {
        std::fprintf(stderr, "Error: %s: %s\n", fn, senk_last_error());
        std::exit(EXIT_FAILURE);
    }
}

/** True when the GPU can dereference p directly. */
inline bool OnDevice(const void *p)
{
    const int r = senk_mem_is_device(p);
    if (r < 0) Check(-r, "senk_mem_is_device");
    return r == 1;
}

/**
 * A device view of an array that may be in host or device memory. Host arrays
 * are copied in (when `in`) and back out on destruction (when `out`).
 */
template <typename T>
class Staged {
public:
    Staged(const T *p, long long n, bool in, bool out) : host_(const_cast<T *>(p)), n_(n), out_(out)
    {
        if (p == nullptr || n <= 0 || OnDevice(p)) {
            dev_ = const_cast<T *>(p);
            return;
        }
        Check(senk_mem_alloc(reinterpret_cast<void **>(&dev_), sizeof(T) * (size_t)n), "senk_mem_alloc");
        own_ = true;
        if (in) Check(senk_mem_h2d(dev_, host_, sizeof(T) * (size_t)n), "senk_mem_h2d");
    }
    Staged(const Staged &) = delete;
    Staged &operator=(const Staged &) = delete;
    ~Staged()
    {
        if (!own_) return;
        if (out_) Check(senk_mem_d2h(host_, dev_, sizeof(T) * (size_t)n_), "senk_mem_d2h");
        senk_mem_free(dev_);
    }
    T *get() const { return dev_; }

private:
    T *host_ = nullptr;
    T *dev_ = nullptr;
    long long n_ = 0;
    bool out_ = false;
    bool own_ = false;
};

/** A host copy of an array that may be in device memory (read only). */
template <typename T>
class HostView {
public:
    HostView(const T *p, long long n)
    {
        if (p == nullptr || n <= 0 || !OnDevice(p)) {
            ptr_ = p;
            return;
        }
        copy_.resize((size_t)n);
        Check(senk_mem_d2h(copy_.data(), p, sizeof(T) * (size_t)n), "senk_mem_d2h");
        ptr_ = copy_.data();
    }
    const T *get() const { return ptr_; }
    T operator[](long long i) const { return ptr_[i]; }

private:
    const T *ptr_ = nullptr;
    std::vector<T> copy_;
};

/** rptr[N] of a CSR (or block-CSR) row pointer in host or device memory. */
inline int LastPointer(const int *rptr, int rows)
{
    HostView<int> h(rptr + rows, 1);
    return h[0];
}

/** The options under which the solver templates run: the reference's stdout. */
inline senk_options Printing()
{
    senk_options o{};
    o.orth = SENK_ORTH_CGS;
    o.spmv = SENK_SPMV_AUTO;
    o.verbose = 1;
    return o;
}

template <typename T>
struct IsDouble : std::is_same<T, double> {};

}  // namespace device

}  // namespace senk

#endif
