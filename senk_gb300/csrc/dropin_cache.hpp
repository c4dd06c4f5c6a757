// Device-resident systems kept between drop-in solver calls.
//
// A drop-in call (senk_*_gmres_d, senk_*_gcr_d, ...) takes host arrays, as the
// reference's templates do. Uploading A and the factors and laying the factors
// out for the sweeps costs about as much as a solve on the benchmark's system,
// and applications call the solver many times with the same matrix. The cache
// keeps the last systems built, keyed by the entry, sizes, build options and
// host addresses of every input array plus a hash of their contents, so a
// matrix changed in place (same addresses, new values) is rebuilt. Only b and
// the initial x travel on a hit.
#pragma once

#include <cstdint>
#include <cstring>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "device.hpp"

namespace senkgpu {

// 64-bit hash of a list of byte ranges: each 1 MiB chunk is hashed on its own
// (multiply-xorshift over 8-byte words in four independent lanes, so a core
// keeps four multiplies in flight; chunks in parallel), then the lanes and the
// chunk hashes are combined in order, so the result does not depend on the
// number of threads.
inline uint64_t content_hash(const std::vector<std::pair<const void *, size_t>> &ranges)
{
    constexpr size_t kChunk = 1 << 20;
    struct Piece {
        const unsigned char *p;
        size_t n;
    };
    std::vector<Piece> pieces;
    for (const auto &r : ranges) {
        const unsigned char *p = static_cast<const unsigned char *>(r.first);
        for (size_t o = 0; o < r.second; o += kChunk) pieces.push_back({p + o, std::min(kChunk, r.second - o)});
        pieces.push_back({nullptr, r.second});  // separates the ranges and mixes in their sizes
    }
    std::vector<uint64_t> h(pieces.size());
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)pieces.size(); i++) {
        const Piece pc = pieces[i];
        uint64_t x = 0x243F6A8885A308D3ull ^ pc.n;
        if (pc.p) {
            uint64_t l[4] = {x, x ^ 0xA4093822299F31D0ull, x ^ 0x082EFA98EC4E6C89ull, x ^ 0x452821E638D01377ull};
            size_t k = 0;
            for (; k + 32 <= pc.n; k += 32) {
                uint64_t w[4];
                std::memcpy(w, pc.p + k, 32);
                for (int q = 0; q < 4; q++) {
                    l[q] = (l[q] ^ w[q]) * 0x9E3779B97F4A7C15ull;
                    l[q] ^= l[q] >> 29;
                }
            }
            for (; k + 8 <= pc.n; k += 8) {
                uint64_t w;
                std::memcpy(&w, pc.p + k, 8);
                l[0] = (l[0] ^ w) * 0x9E3779B97F4A7C15ull;
                l[0] ^= l[0] >> 29;
            }
            uint64_t w = 0;
            std::memcpy(&w, pc.p + k, pc.n - k);
            x = l[0] ^ w;
            for (int q = 1; q < 4; q++) {
                x = (x ^ l[q]) * 0x9E3779B97F4A7C15ull;
                x ^= x >> 32;
            }
            x = x * 0x9E3779B97F4A7C15ull;
            x ^= x >> 32;
        }
        h[i] = x;
    }
    uint64_t acc = 0x13198A2E03707344ull;
    for (uint64_t v : h) {
        acc = (acc ^ v) * 0xBF58476D1CE4E5B9ull;
        acc ^= acc >> 31;
    }
    return acc;
}

struct DropinKey {
    std::string entry;
    std::vector<long long> ints;       // sizes, kinds and build options
    std::vector<const void *> ptrs;    // host addresses of the inputs
    uint64_t hash = 0;
    bool operator==(const DropinKey &o) const
    {
        return entry == o.entry && ints == o.ints && ptrs == o.ptrs && hash == o.hash;
    }
};

// Whether drop-in calls keep their systems (senk_dropin_cache).
inline int &dropin_cache_mode()
{
    static int mode = 1;
    return mode;
}

inline std::mutex &dropin_mutex()
{
    static std::mutex mu;
    return mu;
}

template <typename T>
struct DropinCache {
    static constexpr size_t kKeep = 2;  // systems kept per value type
    std::list<std::pair<DropinKey, std::shared_ptr<System<T>>>> items;  // most recent first
    static DropinCache &get()
    {
        static DropinCache c;
        return c;
    }
};

inline void dropin_cache_clear()
{
    DropinCache<double>::get().items.clear();
    DropinCache<float>::get().items.clear();
}

// The system of a drop-in call: a cached one if every key field matches, else
// a new one (cached unless the cache is off). *built tells which. The caller
// holds dropin_mutex() for the whole call.
template <typename T>
std::shared_ptr<System<T>> dropin_system(const char *entry, const senk_system_desc &d, const senk_options &o,
                                         bool *built)
{
    const int N = d.N;
    const bool block = d.precond == SENK_PC_ILUB || d.precond == SENK_PC_ILUB_ABMC;
    const size_t vb = d.dtype == SENK_F64 ? 8 : 4;
    DropinKey k;
    k.entry = entry;
    k.ints = {N, d.dtype, d.precond, d.cnum, d.bsize, d.bnl, d.bnw, d.mixed, o.spmv, o.sweep};
    k.ptrs = {d.val, d.cind, d.rptr, d.lval, d.lcind, d.lrptr, d.uval, d.ucind, d.urptr, d.cptr};
    std::vector<std::pair<const void *, size_t>> ranges;
    const long long nnz = d.rptr[N];
    ranges.push_back({d.val, (size_t)nnz * vb});
    ranges.push_back({d.cind, (size_t)nnz * 4});
    ranges.push_back({d.rptr, (size_t)(N + 1) * 4});
    if (d.precond != SENK_PC_NONE && d.lrptr && d.urptr) {
        const int rows = block ? N / std::max(d.bnl, 1) : N;
        const size_t per = block ? (size_t)d.bnl * d.bnw : 1;
        for (const auto &f : {std::make_tuple(d.lval, d.lcind, d.lrptr), std::make_tuple(d.uval, d.ucind, d.urptr)}) {
            const int *rp = std::get<2>(f);
            const long long cnt = rp[rows];
            ranges.push_back({std::get<0>(f), (size_t)cnt * per * vb});
            ranges.push_back({std::get<1>(f), (size_t)cnt * 4});
            ranges.push_back({rp, (size_t)(rows + 1) * 4});
        }
    }
    if (d.cptr) ranges.push_back({d.cptr, (size_t)(d.cnum + 1) * 4});
    auto &items = DropinCache<T>::get().items;
    if (dropin_cache_mode()) {
        k.hash = content_hash(ranges);
        for (auto it = items.begin(); it != items.end(); ++it) {
            if (it->first == k) {
                items.splice(items.begin(), items, it);
                *built = false;
                auto S = items.front().second;
                S->opt.orth = o.orth;
                S->opt.verbose = o.verbose;
                return S;
            }
        }
    } else {
        items.clear();
    }
    auto S = std::make_shared<System<T>>();
    S->create(d, &o);
    *built = true;
    if (dropin_cache_mode()) {
        items.emplace_front(std::move(k), S);
        while (items.size() > DropinCache<T>::kKeep) items.pop_back();
    }
    return S;
}

}  // namespace senkgpu
