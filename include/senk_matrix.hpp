/**
 * @file senk_matrix.hpp
 * @brief Host-side matrix setup of the SenK API (drop-in for
 *        include/senk_matrix.hpp of sapporosaburo/SenK): format conversions,
 *        ILU(0)/ILU(p)/ILUB factorisation patterns, splitting and reordering.
 *
 * These run once on the host before a solve. They reproduce the reference's
 * output arrays exactly (same sparsity, same entry order, same floating-point
 * operations in the same order for the factorisations), which the GPU sweeps
 * depend on. Output arrays are malloc'd; release them with free().
 */
#ifndef SENK_MATRIX_HPP
#define SENK_MATRIX_HPP

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "senk_class.hpp"
#include "senk_helper.hpp"
#include "senk_utils.hpp"

namespace senk {
namespace matrix {

/** Drops explicit zeros, in place (senk_matrix.hpp:29-43). */
template <typename T>
void RemoveZeros(T **val, int **cind, int *rptr, int N)
{
    int w = 0, r0 = rptr[0];
    for (int i = 0; i < N; i++) {
        const int e = rptr[i + 1];
        for (int j = r0; j < e; j++) {
            if ((*val)[j] == 0) continue;
            (*val)[w] = (*val)[j];
            (*cind)[w] = (*cind)[j];
            w++;
        }
        r0 = e;
        rptr[i + 1] = w;
    }
    *val = utils::SafeRealloc<T>(*val, w);
    *cind = utils::SafeRealloc<int>(*cind, w);
}

/** True when every row holds its diagonal entry (senk_matrix.hpp:45-56). */
template <typename T>
bool CheckStructure(T *val, int *cind, int *rptr, int N)
{
    (void)val;
    for (int i = 0; i < N; i++) {
        bool found = false;
        for (int j = rptr[i]; j < rptr[i + 1] && !found; j++) found = (cind[j] == i);
        if (!found) return false;
    }
    return true;
}

/** CSR (N x M) -> CSC, rows ascending within each column (senk_matrix.hpp:58-88). */
template <typename T>
void Csr2Csc(T *val, int *cind, int *rptr, T **cval, int **crind, int **ccptr, int N, int M)
{
    const int nnz = rptr[N];
    *cval = utils::SafeMalloc<T>(nnz);
    *crind = utils::SafeMalloc<int>(nnz);
    *ccptr = utils::SafeMalloc<int>(M + 1);
    std::vector<int> fill(M + 1, 0);
    for (int j = 0; j < nnz; j++) fill[cind[j] + 1]++;
    for (int c = 0; c < M; c++) fill[c + 1] += fill[c];
    std::copy(fill.begin(), fill.end(), *ccptr);
    for (int i = 0; i < N; i++) {
        for (int j = rptr[i]; j < rptr[i + 1]; j++) {
            const int at = fill[cind[j]]++;
            (*crind)[at] = i;
            (*cval)[at] = val[j];
        }
    }
}

/**
 * CSR -> SELL-c (senk_matrix.hpp:90-142): slice s (rows s*size ..) has
 * s_len[s+1]-s_len[s] columns stored column-major with row stride equal to the
 * slice's row count; short rows are padded with zeros (column 0). Returns the
 * number of stored elements.
 */
template <typename T>
int Csr2Sell(T *val, int *cind, int *rptr, T **s_val, int **s_cind, int **s_len, int size, int N)
{
    const int ns = (N + size - 1) / size;
    *s_len = utils::SafeMalloc<int>(ns + 1);
    (*s_len)[0] = 0;
    int total = 0;
    for (int s = 0; s < ns; s++) {
        const int rows = std::min(size, N - s * size);
        int w = 0;
        for (int r = s * size; r < s * size + rows; r++) w = std::max(w, rptr[r + 1] - rptr[r]);
        (*s_len)[s + 1] = (*s_len)[s] + w;
        total += w * rows;
    }
    *s_val = utils::SafeMalloc<T>(total);
    *s_cind = utils::SafeMalloc<int>(total);
    for (int s = 0; s < ns; s++) {
        const int rows = std::min(size, N - s * size);
        const int w = (*s_len)[s + 1] - (*s_len)[s];
        const int base = (*s_len)[s] * size;
        for (int r = 0; r < rows; r++) {
            const int row = s * size + r, len = rptr[row + 1] - rptr[row];
            for (int k = 0; k < w; k++) {
                const int at = base + k * rows + r;
                (*s_val)[at] = k < len ? val[rptr[row] + k] : T(0);
                (*s_cind)[at] = k < len ? cind[rptr[row] + k] : 0;
            }
        }
    }
    return total;
}

/**
 * CSR -> BCSR with bnl x bnw blocks (senk_matrix.hpp:144-211). A block row holds,
 * in ascending order, every block column touched by one of its rows; block
 * values are column-major (bval[blk*bnl*bnw + c*bnl + r]) and zero where the CSR
 * has no entry. Columns must ascend within each row. Exits when N is not a
 * multiple of bnl and bnw.
 *
 * An empty row takes one entry: the reference's row cursor starts at rptr[row]
 * and is only found finished after it has copied the entry there, which is the
 * first entry of the next non-empty row (senk_matrix.hpp:159-177, 196-203). An
 * L factor's row 0, and in ABMC order the first row of many blocks, so carries a
 * value on or near the diagonal, and the ILUB sweeps read it. Kept, since the
 * sweeps' results depend on it. Where no entry follows (trailing empty rows) the
 * reference reads past the arrays; here such a row stays empty.
 */
template <typename T>
void Csr2Bcsr(T *val, int *cind, int *rptr, T **bval, int **bcind, int **brptr, int N, int bnl, int bnw)
{
    if (N % bnl || N % bnw) {
        std::printf("Error: Csr2Bcsr\n");
        std::exit(EXIT_FAILURE);
    }
    const int nbr = N / bnl, nnz = rptr[N];
    // entries [rptr[row], row_end(row)) of a row, the one borrowed entry included
    auto row_end = [&](int row) {
        return rptr[row + 1] > rptr[row] ? rptr[row + 1] : std::min(rptr[row] + 1, nnz);
    };
    *brptr = utils::SafeMalloc<int>(nbr + 1);
    (*brptr)[0] = 0;
    std::vector<int> cols;
    std::vector<int> bc;
    for (int br = 0; br < nbr; br++) {
        cols.clear();
        for (int r = br * bnl; r < (br + 1) * bnl; r++)
            for (int j = rptr[r]; j < row_end(r); j++) cols.push_back(cind[j] / bnw);
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        bc.insert(bc.end(), cols.begin(), cols.end());
        (*brptr)[br + 1] = (int)bc.size();
    }
    const int nblk = (int)bc.size();
    *bcind = utils::SafeMalloc<int>(nblk);
    std::copy(bc.begin(), bc.end(), *bcind);
    *bval = utils::SafeCalloc<T>(nblk * bnl * bnw);
    for (int br = 0; br < nbr; br++) {
        for (int r = 0; r < bnl; r++) {
            const int row = br * bnl + r;
            int blk = (*brptr)[br];
            for (int j = rptr[row]; j < row_end(row); j++) {
                while ((*bcind)[blk] != cind[j] / bnw) blk++;
                (*bval)[(size_t)blk * bnl * bnw + (cind[j] % bnw) * bnl + r] = val[j];
            }
        }
    }
}

/** BCSR -> CSR keeping every block entry, zeros included (senk_matrix.hpp:213-241). */
template <typename T>
int Bcsr2Csr(T *bval, int *bcind, int *brptr, T **val, int **cind, int **rptr, int N, int bnl, int bnw)
{
    const int bs = bnl * bnw, nblk = brptr[N / bnl];
    *val = utils::SafeMalloc<T>(nblk * bs);
    *cind = utils::SafeMalloc<int>(nblk * bs);
    *rptr = utils::SafeMalloc<int>(N + 1);
    (*rptr)[0] = 0;
    int at = 0;
    for (int i = 0; i < N; i++) {
        const int br = i / bnl, r = i % bnl;
        for (int blk = brptr[br]; blk < brptr[br + 1]; blk++) {
            for (int c = 0; c < bnw; c++) {
                (*cind)[at] = bcind[blk] * bnw + c;
                (*val)[at] = bval[(size_t)blk * bs + c * bnl + r];
                at++;
            }
        }
        (*rptr)[i + 1] = at;
    }
    return at;
}

/** Pads N up to a multiple of `size` with unit diagonal rows (senk_matrix.hpp:243-255). */
template <typename T>
void Padding(T **val, int **cind, int **rptr, int size, int *N)
{
    const int extra = (*N % size == 0) ? 0 : size - *N % size;
    const int nnz = (*rptr)[*N];
    *val = utils::SafeRealloc<T>(*val, nnz + extra);
    *cind = utils::SafeRealloc<int>(*cind, nnz + extra);
    *rptr = utils::SafeRealloc<int>(*rptr, *N + 1 + extra);
    for (int k = 0; k < extra; k++) {
        (*val)[nnz + k] = 1;
        (*cind)[nnz + k] = *N + k;
        (*rptr)[*N + 1 + k] = (*rptr)[*N + k] + 1;
    }
    *N += extra;
}

/**
 * Splits A into L (strictly lower), D and U (strictly upper) by `key`
 * (senk_matrix.hpp:257-333): "LD-U" (diagonal ends each L row), "L-DU" (diagonal
 * starts each U row), "L-D-U" (diagonal in *diag), "LU-D" (off-diagonals in L,
 * diagonal in *diag). invDiag stores 1/a_ii. Exits on an unknown key.
 */
template <typename T>
void Split(T *val, int *cind, int *rptr, T **lval, int **lcind, int **lrptr, T **uval, int **ucind, int **urptr,
           T **diag, int N, const char *key, bool invDiag)
{
    int mode;
    if (std::strcmp(key, "LD-U") == 0) mode = 0;
    else if (std::strcmp(key, "L-DU") == 0) mode = 1;
    else if (std::strcmp(key, "L-D-U") == 0) mode = 2;
    else if (std::strcmp(key, "LU-D") == 0) mode = 3;
    else { std::printf("Split: Keyword is not valid."); std::exit(1); }
    int nl = 0, nu = 0, nd = 0;
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++) (cind[j] < i ? nl : cind[j] > i ? nu : nd)++;
    const int lsz = nl + (mode == 0 ? nd : 0) + (mode == 3 ? nu : 0);
    const int usz = mode == 3 ? 0 : nu + (mode == 1 ? nd : 0);
    *lval = utils::SafeMalloc<T>(lsz);
    *lcind = utils::SafeMalloc<int>(lsz);
    *lrptr = utils::SafeMalloc<int>(N + 1);
    if (usz != 0) {
        *uval = utils::SafeMalloc<T>(usz);
        *ucind = utils::SafeMalloc<int>(usz);
        *urptr = utils::SafeMalloc<int>(N + 1);
    }
    const bool sep = (mode == 2 || mode == 3);
    if (sep && nd == N) *diag = utils::SafeMalloc<T>(N);
    int lc = 0, uc = 0, dc = 0;
    (*lrptr)[0] = 0;
    if (usz) (*urptr)[0] = 0;
    for (int i = 0; i < N; i++) {
        for (int j = rptr[i]; j < rptr[i + 1]; j++) {
            const int c = cind[j];
            if (c < i || (mode == 3 && c > i)) {
                (*lval)[lc] = val[j];
                (*lcind)[lc++] = c;
            } else if (c > i) {
                (*uval)[uc] = val[j];
                (*ucind)[uc++] = c;
            } else {
                const T d = invDiag ? 1 / val[j] : val[j];
                if (mode == 0) { (*lval)[lc] = d; (*lcind)[lc++] = c; }
                else if (mode == 1) { (*uval)[uc] = d; (*ucind)[uc++] = c; }
                else { if (nd == N) (*diag)[dc] = d; dc++; }
            }
        }
        (*lrptr)[i + 1] = lc;
        if (usz) (*urptr)[i + 1] = uc;
    }
}

/**
 * Symmetric storage (lower "L" or upper "U" triangle incl. diagonal) -> full
 * matrix, rows sorted (senk_matrix.hpp:335-371).
 */
template <typename T>
void Expand(T *tval, int *tcind, int *trptr, T **val, int **cind, int **rptr, int N, const char *key)
{
    const bool lower = std::strcmp(key, "L") == 0;
    if (!lower && std::strcmp(key, "U") != 0) { std::printf("Expand: Keyword is not valid."); std::exit(1); }
    T *cv; int *cr, *cp;
    Csr2Csc<T>(tval, tcind, trptr, &cv, &cr, &cp, N, N);
    // lower part (incl. diagonal) from the lower-stored matrix, upper part
    // (excluding diagonal) from the other orientation
    const T *lv = lower ? tval : cv; const int *lc = lower ? tcind : cr; const int *lr = lower ? trptr : cp;
    const T *uv = lower ? cv : tval; const int *uc = lower ? cr : tcind; const int *ur = lower ? cp : trptr;
    const int nnz = trptr[N] * 2 - N;
    *val = utils::SafeMalloc<T>(nnz);
    *cind = utils::SafeMalloc<int>(nnz);
    *rptr = utils::SafeMalloc<int>(N + 1);
    int at = 0;
    (*rptr)[0] = 0;
    for (int i = 0; i < N; i++) {
        for (int j = lr[i]; j < lr[i + 1]; j++) { (*val)[at] = lv[j]; (*cind)[at++] = lc[j]; }
        for (int j = ur[i] + 1; j < ur[i + 1]; j++) { (*val)[at] = uv[j]; (*cind)[at++] = uc[j]; }
        (*rptr)[i + 1] = at;
    }
    std::free(cv); std::free(cr); std::free(cp);
}

/** Deep copy of a CSR matrix (senk_matrix.hpp:373-389). */
template <typename T>
void Duplicate(T *tval, int *tcind, int *trptr, T **val, int **cind, int **rptr, int N)
{
    const int nnz = trptr[N];
    *val = utils::SafeMalloc<T>(nnz);
    *cind = utils::SafeMalloc<int>(nnz);
    *rptr = utils::SafeMalloc<int>(N + 1);
    std::memcpy(*val, tval, sizeof(T) * (size_t)nnz);
    std::memcpy(*cind, tcind, sizeof(int) * (size_t)nnz);
    std::memcpy(*rptr, trptr, sizeof(int) * (size_t)(N + 1));
}

/** diag[i] = a_ii (senk_matrix.hpp:391-404). */
template <typename T>
void GetDiag(T *val, int *cind, int *rptr, T **diag, int N)
{
    *diag = utils::SafeMalloc<T>(N);
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++)
            if (cind[j] == i) { (*diag)[i] = val[j]; break; }
}

/** a_ij <- ld_i * a_ij * rd_j (senk_matrix.hpp:406-416). */
template <typename T>
void Scaling(T *val, int *cind, int *rptr, T *ld, T *rd, int N)
{
    for (int i = 0; i < N; i++) {
        const T l = ld[i];
        for (int j = rptr[i]; j < rptr[i + 1]; j++) val[j] = l * val[j] * rd[cind[j]];
    }
}

namespace detail {
// Position of the diagonal of row i, or -1.
inline int diag_pos(const int *cind, const int *rptr, int i)
{
    for (int j = rptr[i]; j < rptr[i + 1]; j++)
        if (cind[j] == i) return j;
    return -1;
}
}  // namespace detail

namespace detail {
// ILU(0) body; returns -1, or the row whose zero pivot stopped it.
template <typename T>
int ilu0(T *val, const int *cind, const int *rptr, int N)
{
    for (int i = 1; i < N; i++) {
        const int end = rptr[i + 1];
        for (int k = rptr[i]; k < end && cind[k] < i; k++) {
            const int p = cind[k];
            const int d = diag_pos(cind, rptr, p);
            if (d >= 0) {
                if (val[d] == 0) return p;
                val[k] = val[k] / val[d];
            }
            int l = rptr[p];
            const int pend = rptr[p + 1];
            for (int j = k + 1; j < end; j++) {
                while (l < pend && cind[l] < cind[j]) l++;
                if (l < pend && cind[l] == cind[j]) {
                    val[j] -= val[k] * val[l];
                    l++;
                }
            }
        }
    }
    return -1;
}
}  // namespace detail

/**
 * In-place ILU(0) on the pattern of A (senk_matrix.hpp:418-448): row by row,
 * each strictly-lower entry a_ik becomes a_ik / u_kk and is used to eliminate
 * the remaining entries of row i that row k also holds. Columns must be sorted.
 * Prints "Error: Ilu0, 0 pivot" and exits on a zero pivot.
 */
template <typename T>
void Ilu0(T *val, int *cind, int *rptr, int N)
{
    if (detail::ilu0(val, cind, rptr, N) >= 0) {
        std::printf("Error: Ilu0, 0 pivot\n");
        std::exit(1);
    }
}

namespace detail {
/*
 * Level-of-fill incomplete factorisation shared by Ilup (numeric) and
 * AllocLevelZero (pattern only) — senk_matrix.hpp:450-650. Row i starts as
 * A's row with level 0; every kept lower entry k (level <= p, in column order)
 * becomes a pivot (value a_ik/u_kk, level reset to 0 in the row) and is merged
 * with the finished upper part of row k: shared columns are updated and take
 * min(level, lev_ik + lev_kj + 1); new columns enter as fill with level
 * lev_ik + lev_kj + 1. Entries above level p stay in the working row (they are
 * still updated) but are neither pivots nor stored.
 */
template <typename T, bool NUMERIC>
void level_fill(T **val, int **cind, int **rptr, int N, int p)
{
    const T *va = *val;
    const int *ci = *cind, *rp = *rptr;
    std::vector<T> nv;
    std::vector<int> nc, nl, nr(N + 1, 0);
    for (int j = rp[0]; j < rp[1]; j++) { nv.push_back(va[j]); nc.push_back(ci[j]); nl.push_back(0); }
    nr[1] = (int)nc.size();
    struct E { T v; int lev; int col; };
    std::vector<E> cur, nxt;
    T pivot = 0;
    int pivot_lev = 0;
    for (int i = 1; i < N; i++) {
        cur.clear();
        for (int j = rp[i]; j < rp[i + 1]; j++) cur.push_back({va[j], 0, ci[j]});
        int count = 0;
        while (count < (int)cur.size() && cur[count].col < i) {
            if (cur[count].lev > p) { count++; continue; }
            const int k = cur[count].col;
            nxt.assign(cur.begin(), cur.begin() + count);
            int j = nr[k];
            for (; j < nr[k + 1]; j++) {
                if (nc[j] == k) {
                    pivot = NUMERIC ? cur[count].v / nv[j] : cur[count].v;
                    pivot_lev = cur[count].lev;
                    break;
                }
            }
            j++;
            int a = count + 1;
            nxt.push_back({pivot, 0, k});
            const int kend = nr[k + 1];
            while (a < (int)cur.size() || j < kend) {
                const int c1 = a < (int)cur.size() ? cur[a].col : N + 1;
                const int c2 = j < kend ? nc[j] : N + 1;
                if (c1 < c2) {
                    nxt.push_back(cur[a++]);
                } else if (c1 == c2) {
                    const int fl = pivot_lev + nl[j] + 1;
                    nxt.push_back({NUMERIC ? cur[a].v - pivot * nv[j] : cur[a].v, std::min(cur[a].lev, fl), cur[a].col});
                    a++;
                    j++;
                } else {
                    nxt.push_back({NUMERIC ? -pivot * nv[j] : T(0), pivot_lev + nl[j] + 1, nc[j]});
                    j++;
                }
            }
            count++;
            cur.swap(nxt);
        }
        for (const E &e : cur) {
            if (e.lev <= p) { nv.push_back(e.v); nc.push_back(e.col); nl.push_back(e.lev); }
        }
        nr[i + 1] = (int)nc.size();
    }
    const int nnz = (int)nc.size();
    *val = utils::SafeMalloc<T>(nnz);
    *cind = utils::SafeMalloc<int>(nnz);
    *rptr = utils::SafeMalloc<int>(N + 1);
    std::copy(nv.begin(), nv.end(), *val);
    std::copy(nc.begin(), nc.end(), *cind);
    std::copy(nr.begin(), nr.end(), *rptr);
}
}  // namespace detail

/**
 * ILU(p) by level of fill (senk_matrix.hpp:450-549). Replaces *val/*cind/*rptr
 * with newly allocated arrays; like the reference it does not free the old ones.
 */
template <typename T>
void Ilup(T **val, int **cind, int **rptr, int N, int p)
{
    detail::level_fill<T, true>(val, cind, rptr, N, p);
}

/**
 * The ILU(p) pattern with A's values and zero fill (senk_matrix.hpp:551-650);
 * Ilu0 on the result gives the ILU(p) factors. Old arrays are not freed.
 */
template <typename T>
void AllocLevelZero(T **val, int **cind, int **rptr, int N, int p)
{
    detail::level_fill<T, false>(val, cind, rptr, N, p);
}

/**
 * ILUB pattern: pads A's pattern with explicit zeros to full bnl x bnw blocks
 * (CSR -> BCSR -> CSR, senk_matrix.hpp:652-666). Frees the old arrays.
 */
template <typename T>
void AllocBlockZero(T **val, int **cind, int **rptr, int N, int bnl, int bnw)
{
    T *bv; int *bc, *br;
    Csr2Bcsr<T>(*val, *cind, *rptr, &bv, &bc, &br, N, bnl, bnw);
    std::free(*val); std::free(*cind); std::free(*rptr);
    Bcsr2Csr<T>(bv, bc, br, val, cind, rptr, N, bnl, bnw);
    std::free(bv); std::free(bc); std::free(br);
}

/**
 * Keeps only entries inside the bnum diagonal blocks of N/bnum rows (the
 * block-Jacobi pattern, senk_matrix.hpp:668-689); reallocates the arrays.
 */
template <typename T>
void RemoveOffDiagonal(T **val, int **cind, int **rptr, int N, int bnum)
{
    const int bs = N / bnum;
    int w = 0, r0 = (*rptr)[0];
    for (int i = 0; i < N; i++) {
        const int lo = i / bs * bs, hi = lo + bs, e = (*rptr)[i + 1];
        for (int j = r0; j < e; j++) {
            const int c = (*cind)[j];
            if (c < lo || c >= hi) continue;
            (*val)[w] = (*val)[j];
            (*cind)[w++] = c;
        }
        r0 = e;
        (*rptr)[i + 1] = w;
    }
    *val = utils::SafeRealloc<T>(*val, w);
    *cind = utils::SafeRealloc<int>(*cind, w);
}

namespace detail {
template <typename T>
void sort_row(int *c, T *v, int n)
{
    helper::QuickSort<int, T>(c, v, 0, n - 1);
}
}  // namespace detail

/** Columns renumbered by RP and each row re-sorted (senk_matrix.hpp:691-701). */
template <typename T>
void Reordering(T *val, int *cind, int *rptr, int *RP, int N)
{
    for (int i = 0; i < N; i++) {
        for (int j = rptr[i]; j < rptr[i + 1]; j++) cind[j] = RP[cind[j]];
        detail::sort_row(cind + rptr[i], val + rptr[i], rptr[i + 1] - rptr[i]);
    }
}

/**
 * Symmetric permutation A' = P A P^T (senk_matrix.hpp:703-730): row i of A' is
 * row LP[i] of A (LP: new -> old) with columns mapped through RP (old -> new)
 * and re-sorted. In place. Works for any value type (the reference's version
 * compiles only for double).
 */
template <typename T>
void Reordering(T *val, int *cind, int *rptr, int *LP, int *RP, int N)
{
    const int nnz = rptr[N];
    std::vector<T> tv(nnz);
    std::vector<int> tc(nnz), tr(N + 1, 0);
    for (int i = 0; i < N; i++) tr[i + 1] = tr[i] + (rptr[LP[i] + 1] - rptr[LP[i]]);
    for (int i = 0; i < N; i++) {
        const int src = rptr[LP[i]], len = rptr[LP[i] + 1] - src;
        for (int j = 0; j < len; j++) {
            tv[tr[i] + j] = val[src + j];
            tc[tr[i] + j] = RP[cind[src + j]];
        }
        detail::sort_row(tc.data() + tr[i], tv.data() + tr[i], len);
    }
    std::copy(tv.begin(), tv.end(), val);
    std::copy(tc.begin(), tc.end(), cind);
    std::copy(tr.begin(), tr.end(), rptr);
}

}  // namespace matrix
}  // namespace senk

#endif
