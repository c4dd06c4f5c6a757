/**
 * @file senk_io.hpp
 * MatrixMarket input (senk_io.hpp:18-103 of the reference): the same function
 * and enum, host code. The file is read whole and its entries are parsed in
 * parallel (OpenMP over line-aligned chunks), then placed into CSR by a
 * counting pass over the rows; each row is sorted by column.
 *
 * Behaviour kept from the reference: the header line must name "symmetric"
 * (Shape Sym) or "general" (Unsym) and not "complex"; '%' lines before the
 * size line are skipped; entries are 1-based "row col value" triples; with
 * removeZeros, entries whose value is 0 are dropped; the lower triangle of a
 * symmetric file is returned as stored (senk::matrix::Expand makes the full
 * matrix); the stdout lines "# Readfile MatrixMarket" and "# N M nnz" and the
 * stderr messages are the reference's.
 *
 * Differences, each an input the reference does not handle: a missing size
 * line, fewer entries than announced, an unparsable token, or an index outside
 * 1..N / 1..M return false with a message (the reference reads garbage or
 * writes out of bounds); the entries of a row come out sorted by column with
 * equal columns in file order (the reference's quicksort leaves duplicate
 * entries in an unspecified order).
 */
#ifndef SENK_IO_HPP
#define SENK_IO_HPP

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "senk_utils.hpp"

namespace senk {

namespace io {

enum Shape {
    Sym,
    Unsym
};

namespace detail {

// Parses one "row col value" triple starting at p (skipping blanks and line
// breaks); returns the position after it, or nullptr if the tokens are not
// two integers and a number.
inline const char *parse_entry(const char *p, const char *end, long long *r, long long *c, double *v)
{
    char *q = nullptr;
    auto skip = [&]() {
        while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) p++;
    };
    skip();
    if (p >= end) return nullptr;
    *r = std::strtoll(p, &q, 10);
    if (q == p) return nullptr;
    p = q;
    skip();
    if (p >= end) return nullptr;
    *c = std::strtoll(p, &q, 10);
    if (q == p) return nullptr;
    p = q;
    skip();
    if (p >= end) return nullptr;
    *v = std::strtod(p, &q);
    if (q == p) return nullptr;
    return q;
}

}  // namespace detail

inline bool ReadMatrixMarket(std::string filename, double **val, int **cind, int **rptr, int *N, int *M,
                             Shape *shape, bool removeZeros)
{
    std::cout << "# Readfile MatrixMarket" << std::endl;
    std::ifstream ifs(filename, std::ios::binary);
    if (!ifs) {
        std::cerr << "# Could not open input file." << std::endl;
        return false;
    }
    std::string text((std::istreambuf_iterator<char>(ifs)), std::istreambuf_iterator<char>());
    // text must end in a byte strtod/strtoll stop at
    text.push_back('\n');
    const char *p = text.data(), *end = text.data() + text.size();
    const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
    const std::string header(p, nl ? nl : end);
    if (header.find("complex") != std::string::npos) {
        std::cerr << "# Header line is not valid." << std::endl;
        return false;
    }
    if (header.find("symmetric") != std::string::npos) shape[0] = Sym;
    else if (header.find("general") != std::string::npos) shape[0] = Unsym;
    else {
        std::cerr << "# Header line is not valid." << std::endl;
        return false;
    }
    p = nl ? nl + 1 : end;
    // comment lines, then the size line
    long long n = -1, m = -1, pe = -1;
    while (p < end) {
        const char *e = static_cast<const char *>(std::memchr(p, '\n', (size_t)(end - p)));
        if (!e) e = end;
        if (*p != '%') {
            const std::string line(p, e);
            if (std::sscanf(line.c_str(), "%lld %lld %lld", &n, &m, &pe) != 3) n = -1;
            p = e + (e < end ? 1 : 0);
            break;
        }
        p = e + (e < end ? 1 : 0);
    }
    if (n < 0 || m < 0 || pe < 0 || n > 0x7fffffff || m > 0x7fffffff || pe > 0x7fffffff) {
        std::cerr << "# Size line is not valid." << std::endl;
        return false;
    }
    N[0] = (int)n;
    M[0] = (int)m;
    std::cout << "# " << N[0] << " " << M[0] << " " << pe << std::endl;

    // Line-aligned chunks, one per thread: each parses its triples; the chunks
    // are joined in file order. As in the reference, the first `nnz` triples
    // of the file are the matrix (later ones are ignored) and, with
    // removeZeros, zero values among them are dropped.
    const size_t body = (size_t)(end - p);
    int nt = 1;
#ifdef _OPENMP
    nt = std::max(1, std::min(omp_get_max_threads(), (int)(body / (1 << 20)) + 1));
#endif
    std::vector<const char *> cut(nt + 1);
    cut[0] = p;
    cut[nt] = end;
    for (int t = 1; t < nt; t++) {
        const char *c = p + body * t / nt;
        const char *e = static_cast<const char *>(std::memchr(c, '\n', (size_t)(end - c)));
        cut[t] = std::max(cut[t - 1], e ? e + 1 : end);
    }
    struct Triple {
        int r, c;
        double v;
    };
    std::vector<std::vector<Triple>> part(nt);
    std::vector<int> bad(nt, 0);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; t++) {
        const char *q = cut[t], *qe = cut[t + 1];
        long long r, c;
        double v;
        while (q < qe) {
            const char *s = q;
            while (s < qe && (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r')) s++;
            if (s >= qe) break;
            const char *after = detail::parse_entry(s, qe, &r, &c, &v);
            if (!after) {
                bad[t] = 1;
                break;
            }
            q = after;
            if (r < 1 || r > n || c < 1 || c > m) {
                bad[t] = 2;
                break;
            }
            part[t].push_back({(int)(r - 1), (int)(c - 1), v});
        }
    }
    size_t held = 0;
    for (int t = 0; t < nt; t++) {
        // an error after the announced entries would not be read by the reference
        if (bad[t] && (long long)held + (long long)part[t].size() < pe) {
            std::cerr << (bad[t] == 1 ? "# Entry is not valid." : "# Entry index out of range.") << std::endl;
            return false;
        }
        held += part[t].size();
    }
    if ((long long)held < pe) {
        std::cerr << "# Fewer entries than the size line announces." << std::endl;
        return false;
    }
    size_t total = 0, seen = 0;
    for (int t = 0; t < nt; t++) {
        if (seen + part[t].size() > (size_t)pe) part[t].resize((size_t)pe > seen ? (size_t)pe - seen : 0);
        seen += part[t].size();
        if (removeZeros)
            part[t].erase(std::remove_if(part[t].begin(), part[t].end(), [](const Triple &e) { return e.v == 0; }),
                          part[t].end());
        total += part[t].size();
    }
    const int nnz = (int)total;
    *val = utils::SafeMalloc<double>(std::max(nnz, 1));
    *cind = utils::SafeMalloc<int>(std::max(nnz, 1));
    *rptr = utils::SafeMalloc<int>(N[0] + 1);
    std::vector<int> cnt(N[0] + 1, 0);
    for (int t = 0; t < nt; t++)
        for (const Triple &e : part[t]) cnt[e.r + 1]++;
    for (int i = 0; i < N[0]; i++) cnt[i + 1] += cnt[i];
    std::copy(cnt.begin(), cnt.end(), *rptr);
    for (int t = 0; t < nt; t++)
        for (const Triple &e : part[t]) {
            const int at = cnt[e.r]++;
            (*val)[at] = e.v;
            (*cind)[at] = e.c;
        }
    // sort each row by column, equal columns in file order
#pragma omp parallel
    {
        std::vector<std::pair<int, double>> row;
#pragma omp for schedule(dynamic, 1024)
        for (int i = 0; i < N[0]; i++) {
            const int b = (*rptr)[i], e = (*rptr)[i + 1];
            bool sorted = true;
            for (int j = b + 1; j < e && sorted; j++) sorted = (*cind)[j - 1] <= (*cind)[j];
            if (sorted) continue;
            row.clear();
            for (int j = b; j < e; j++) row.push_back({(*cind)[j], (*val)[j]});
            std::stable_sort(row.begin(), row.end(),
                             [](const std::pair<int, double> &a, const std::pair<int, double> &c) {
                                 return a.first < c.first;
                             });
            for (int j = b; j < e; j++) {
                (*cind)[j] = row[j - b].first;
                (*val)[j] = row[j - b].second;
            }
        }
    }
    return true;
}

}  // namespace io

}  // namespace senk

#endif
