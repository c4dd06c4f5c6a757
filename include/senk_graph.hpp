/**
 * @file senk_graph.hpp
 * @brief Multicolour orderings of the SenK API (drop-in for
 *        include/senk_graph.hpp): AMC (point colouring) and ABMC (colouring of
 *        row blocks), returned as LP (new -> old), RP (old -> new) and colour
 *        pointers.
 *
 * The colour sweep, the BFS that forms "connect" blocks and the order in which
 * blocks are listed are the reference's (senk_graph.hpp:77-139, 218-238,
 * 291-334): the GPU sweeps consume these arrays, and the iteration counts of the
 * preconditioned solvers depend on them, so they must come out identical.
 */
#ifndef SENK_GRAPH_HPP
#define SENK_GRAPH_HPP

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "senk_utils.hpp"

namespace senk {
namespace graph {

namespace detail {

// Row-block graph: blocks[b*bs .. b*bs+bs-1] are the rows of block b (sorted);
// adjacency lists the distinct blocks touched by those rows' columns.
struct BlockGraph {
    std::vector<int> rows;   // N entries
    std::vector<int> rptr;   // nblocks + 1
    std::vector<int> cind;
};

inline void block_adjacency(const int *cind, const int *rptr, const std::vector<int> &block_of, BlockGraph &g,
                            int nb, int bs)
{
    g.rptr.assign(nb + 1, 0);
    g.cind.clear();
    std::vector<int> touched;
    for (int b = 0; b < nb; b++) {
        touched.clear();
        for (int q = 0; q < bs; q++) {
            const int r = g.rows[(size_t)b * bs + q];
            for (int j = rptr[r]; j < rptr[r + 1]; j++) touched.push_back(block_of[cind[j]]);
        }
        std::sort(touched.begin(), touched.end());
        touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
        g.cind.insert(g.cind.end(), touched.begin(), touched.end());
        g.rptr[b + 1] = (int)g.cind.size();
    }
}

// senk_graph.hpp:27-66: block b = rows [b*bs, (b+1)*bs).
inline void simple_blocking(const int *cind, const int *rptr, int N, int bs, BlockGraph &g)
{
    g.rows.resize(N);
    std::vector<int> block_of(N);
    for (int i = 0; i < N; i++) { g.rows[i] = i; block_of[i] = i / bs; }
    block_adjacency(cind, rptr, block_of, g, N / bs, bs);
}

// senk_graph.hpp:77-139: blocks are filled in breadth-first order from the
// lowest unvisited row; when a search runs dry before the block is full, the
// next unvisited row seeds the same block; a full block ends the search.
inline bool connected_blocking(const int *cind, const int *rptr, int N, int bs, BlockGraph &g)
{
    g.rows.assign(N, 0);
    std::vector<int> block_of(N, 0);
    std::vector<char> seen(N, 0);
    std::vector<int> queue;
    int count = 0, fill = 0;
    auto take = [&](int r) {
        g.rows[count] = r;
        block_of[r] = count / bs;
        seen[r] = 1;
        count++;
        return ++fill == bs;
    };
    for (int seed = 0; seed < N; seed++) {
        if (seen[seed]) continue;
        if (take(seed)) { fill = 0; continue; }
        queue.assign(1, seed);
        size_t head = 0;
        bool full = false;
        while (!full && head < queue.size()) {
            const int q = queue[head++];
            for (int j = rptr[q]; j < rptr[q + 1]; j++) {
                const int c = cind[j];
                if (seen[c]) continue;
                if (take(c)) { fill = 0; full = true; break; }
                queue.push_back(c);
            }
        }
    }
    if (count != N) return false;
    for (int b = 0; b < N / bs; b++) std::sort(g.rows.begin() + (size_t)b * bs, g.rows.begin() + (size_t)(b + 1) * bs);
    block_adjacency(cind, rptr, block_of, g, N / bs, bs);
    return true;
}

// senk_graph.hpp:150-209: the pattern itself, or the sorted union of A and A^T.
inline void adjacency(const int *cind, const int *rptr, int N, bool isSym, std::vector<int> &ar,
                      std::vector<int> &ac)
{
    const int nnz = rptr[N];
    ar.assign(rptr, rptr + N + 1);
    ac.assign(cind, cind + nnz);
    if (isSym) return;
    std::vector<int> tr(N + 1, 0), tc(nnz);
    for (int j = 0; j < nnz; j++) tr[cind[j] + 1]++;
    for (int i = 0; i < N; i++) tr[i + 1] += tr[i];
    std::vector<int> at(tr.begin(), tr.end() - 1);
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++) tc[at[cind[j]]++] = i;
    std::vector<int> ur(N + 1, 0), uc;
    uc.reserve((size_t)nnz * 2);
    for (int i = 0; i < N; i++) {
        int a = rptr[i], b = tr[i];
        while (a < rptr[i + 1] || b < tr[i + 1]) {
            const int ca = a < rptr[i + 1] ? cind[a] : N;
            const int cb = b < tr[i + 1] ? tc[b] : N;
            if (ca <= cb) { uc.push_back(ca); a++; if (ca == cb) b++; }
            else { uc.push_back(cb); b++; }
        }
        ur[i + 1] = (int)uc.size();
    }
    ar.swap(ur);
    ac.swap(uc);
}

// senk_graph.hpp:218-238: colour c is one index-order sweep that takes every
// uncoloured vertex with no neighbour already holding colour c. Returns colours
// 1..num (0-based colour = value - 1).
inline std::vector<int> greedy_colours(const std::vector<int> &ar, const std::vector<int> &ac, int N, int *num)
{
    std::vector<int> colour(N, 0), mark(N, 0);
    int c = 1, done = 0;
    while (done < N) {
        for (int i = 0; i < N; i++) {
            if (colour[i] != 0 || mark[i] == c) continue;
            colour[i] = c;
            done++;
            for (int j = ar[i]; j < ar[i + 1]; j++) mark[ac[j]] = c;
        }
        c++;
    }
    *num = c - 1;
    return colour;
}

}  // namespace detail

/**
 * AMC ordering (senk_graph.hpp:250-277): LP lists the rows colour by colour in
 * index order; size_color[c] is the first row of colour c (N+1 style pointer in
 * rows, num_color+1 entries).
 */
inline void GetAMCPermutation(int *cind, int *rptr, int *num_color, int **size_color, int **LP, int **RP, int N,
                              bool isSym)
{
    std::vector<int> ar, ac;
    detail::adjacency(cind, rptr, N, isSym, ar, ac);
    std::vector<int> colour = detail::greedy_colours(ar, ac, N, num_color);
    *LP = utils::SafeMalloc<int>(N);
    *RP = utils::SafeMalloc<int>(N);
    *size_color = utils::SafeMalloc<int>(*num_color + 1);
    (*size_color)[0] = 0;
    int at = 0;
    for (int c = 1; c <= *num_color; c++) {
        for (int i = 0; i < N; i++)
            if (colour[i] == c) (*LP)[at++] = i;
        (*size_color)[c] = at;
    }
    for (int i = 0; i < N; i++) (*RP)[(*LP)[i]] = i;
}

/**
 * ABMC ordering (senk_graph.hpp:291-334): rows are grouped into blocks of bsize
 * ("simple": consecutive rows; "connect": breadth-first), the block graph (with
 * A + A^T unless isSym) is coloured, and LP lists the blocks colour by colour,
 * each block's rows in ascending order. size_color counts BLOCKS
 * (size_color[c] = first block of colour c). Prints an error and exits when N is
 * not a multiple of bsize or the method is unknown.
 */
inline void GetABMCPermutation(int *cind, int *rptr, int *num_color, int **size_color, int **LP, int **RP, int N,
                               int bsize, bool isSym, const char *bmethod)
{
    if (bsize <= 0 || N % bsize) {
        std::printf("Error: GetABMCPermutation\n");
        std::exit(1);
    }
    detail::BlockGraph g;
    if (std::strcmp(bmethod, "simple") == 0) {
        detail::simple_blocking(cind, rptr, N, bsize, g);
    } else if (std::strcmp(bmethod, "connect") == 0) {
        if (!detail::connected_blocking(cind, rptr, N, bsize, g)) std::exit(1);
    } else {
        std::printf("Error: GetABMCPermutation\n");
        std::printf("The blocking method is invalid\n");
        std::exit(1);
    }
    const int nb = N / bsize;
    std::vector<int> ar, ac;
    detail::adjacency(g.cind.data(), g.rptr.data(), nb, isSym, ar, ac);
    std::vector<int> colour = detail::greedy_colours(ar, ac, nb, num_color);
    *LP = utils::SafeMalloc<int>(N);
    *RP = utils::SafeMalloc<int>(N);
    *size_color = utils::SafeMalloc<int>(*num_color + 1);
    (*size_color)[0] = 0;
    int at = 0;
    for (int c = 1; c <= *num_color; c++) {
        for (int b = 0; b < nb; b++) {
            if (colour[b] != c) continue;
            for (int q = 0; q < bsize; q++) (*LP)[at++] = g.rows[(size_t)b * bsize + q];
        }
        (*size_color)[c] = at / bsize;
    }
    for (int i = 0; i < N; i++) (*RP)[(*LP)[i]] = i;
}

}  // namespace graph
}  // namespace senk

#endif
