/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of SenK's preconditioned Krylov path (sapporosaburo/SenK,
 * header-only C++/OpenMP).  It is the CPU checker for the CUDA path and the CPU
 * baseline that bench.py times beside it.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product library never does.
 *
 * Each function names the reference file:line it restates.  Parity of this
 * restatement is pinned against the reference itself: oracle/Makefile also
 * compiles the reference headers into oracle/_ref/libsenk_ref.so (ref_shim.cpp),
 * and tests/test_oracle_pin.py compares the two on the same inputs, and against
 * the golden fixtures under tests/golden/ that the reference produced.
 *
 * Errors are returned as codes instead of the reference's exit(1).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_OP_CSR 0
#define ORACLE_OP_BCSR 1

#define ORACLE_PC_NONE 0
#define ORACLE_PC_ILU 1
#define ORACLE_PC_ILU_AMC 2
#define ORACLE_PC_ILU_ABMC 3
#define ORACLE_PC_ILU_BJ 4
#define ORACLE_PC_ILUB 5
#define ORACLE_PC_ILUB_ABMC 6

typedef struct {
    int iters;
    int converged;
    double res;
} oracle_result;

void oracle_free(void *p) { free(p); }

/* Thread count for the OpenMP regions. OpenMP reductions combine per-thread
 * partial sums in a run-dependent order, so parity checks run with one thread
 * (the reference's sequential semantics); the CPU baseline uses all cores. */
#ifdef _OPENMP
#include <omp.h>
void oracle_set_threads(int n) { omp_set_num_threads(n); }
int oracle_get_threads(void) { return omp_get_max_threads(); }
#else
void oracle_set_threads(int n) { (void)n; }
int oracle_get_threads(void) { return 1; }
#endif

/* -------------------------------------------- typed kernels and solvers --- */
#define T double
#define SFX(n) n##_d
#define SQRT sqrt
#define FABS fabs
#include "oracle_typed.h"
#undef T
#undef SFX
#undef SQRT
#undef FABS

#define T float
#define SFX(n) n##_s
#define SQRT sqrtf
#define FABS fabsf
#include "oracle_typed.h"
#undef T
#undef SFX
#undef SQRT
#undef FABS

/* include/senk_utils.hpp:103-110  Convert (FP64 -> FP32) */
void oracle_convert_d2s(const double *in, float *out, int n)
{
    #pragma omp parallel for
    for (int i = 0; i < n; i++) out[i] = (float)in[i];
}

/* --------------------------------------------------------- matrix setup --- */

/* include/senk_matrix.hpp:45-56  every row holds its diagonal */
int oracle_check_structure(const int *cind, const int *rptr, int N)
{
    for (int i = 0; i < N; i++) {
        int ok = 0;
        for (int j = rptr[i]; j < rptr[i + 1]; j++)
            if (cind[j] == i) { ok = 1; break; }
        if (!ok) return 0;
    }
    return 1;
}

/* include/senk_matrix.hpp:58-88  Csr2Csc (stable counting transpose) */
void oracle_csr2csc(const double *val, const int *cind, const int *rptr,
                    double **cval, int **crind, int **ccptr, int N, int M)
{
    int nnz = rptr[N];
    *cval = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    *crind = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    *ccptr = (int *)malloc(sizeof(int) * (M + 1));
    int *num = (int *)calloc(M > 0 ? M : 1, sizeof(int));
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++) num[cind[j]]++;
    (*ccptr)[0] = 0;
    for (int i = 0; i < M; i++) { (*ccptr)[i + 1] = (*ccptr)[i] + num[i]; num[i] = 0; }
    for (int i = 0; i < N; i++) {
        for (int j = rptr[i]; j < rptr[i + 1]; j++) {
            int at = (*ccptr)[cind[j]] + num[cind[j]]++;
            (*crind)[at] = i;
            (*cval)[at] = val[j];
        }
    }
    free(num);
}

/* include/senk_matrix.hpp:90-142  Csr2Sell: slice s holds s_len[s+1]-s_len[s]
 * columns; element (row j of the slice, column c) sits at s_len[s]*size +
 * c*rows + j where rows = size except for a short last slice. Returns the padded
 * element count. */
int oracle_csr2sell(const double *val, const int *cind, const int *rptr,
                    double **s_val, int **s_cind, int **s_len, int size, int N)
{
    int nslice = (N + size - 1) / size;
    *s_len = (int *)malloc(sizeof(int) * (nslice + 1));
    int nnz = 0;
    (*s_len)[0] = 0;
    for (int s = 0; s < nslice; s++) {
        int rows = (s == nslice - 1 && N % size != 0) ? N % size : size;
        int wmax = 0;
        for (int j = 0; j < rows; j++) {
            int r = s * size + j;
            if (wmax < rptr[r + 1] - rptr[r]) wmax = rptr[r + 1] - rptr[r];
        }
        (*s_len)[s + 1] = (*s_len)[s] + wmax;
        nnz += wmax * rows;
    }
    int cap = (*s_len)[nslice] * size;
    *s_val = (double *)calloc(cap > 0 ? cap : 1, sizeof(double));
    *s_cind = (int *)calloc(cap > 0 ? cap : 1, sizeof(int));
    for (int s = 0; s < nslice; s++) {
        int rows = (s == nslice - 1 && N % size != 0) ? N % size : size;
        int w = (*s_len)[s + 1] - (*s_len)[s];
        for (int j = 0; j < rows; j++) {
            int r = s * size + j, c = 0;
            for (int k = rptr[r]; k < rptr[r + 1]; k++, c++) {
                (*s_val)[(*s_len)[s] * size + c * rows + j] = val[k];
                (*s_cind)[(*s_len)[s] * size + c * rows + j] = cind[k];
            }
            for (; c < w; c++) {
                (*s_val)[(*s_len)[s] * size + c * rows + j] = 0;
                (*s_cind)[(*s_len)[s] * size + c * rows + j] = 0;
            }
        }
    }
    return nnz;
}

/* include/senk_matrix.hpp:144-211  Csr2Bcsr: a bnl-row block row is swept by
 * repeatedly taking the smallest remaining column and consuming every entry of
 * that bnw-wide block column; missing block entries are zero. Block storage is
 * column-major: bval[blk*bnl*bnw + c*bnl + r]. Returns 0, or -1 if N is not a
 * multiple of bnl and bnw. */
int oracle_csr2bcsr(const double *val, const int *cind, const int *rptr,
                    double **bval, int **bcind, int **brptr, int N, int bnl, int bnw)
{
    if (N % bnl || N % bnw) return -1;
    *brptr = (int *)malloc(sizeof(int) * (N / bnl + 1));
    int *ptr = (int *)malloc(sizeof(int) * bnl);
    int cnt = 0;
    (*brptr)[0] = 0;
    for (int pass = 0; pass < 2; pass++) {
        if (pass == 1) {
            *bcind = (int *)malloc(sizeof(int) * (cnt > 0 ? cnt : 1));
            *bval = (double *)calloc((size_t)(cnt > 0 ? cnt : 1) * bnl * bnw, sizeof(double));
            cnt = 0;
        }
        for (int i = 0; i < N; i += bnl) {
            for (int r = 0; r < bnl; r++) ptr[r] = rptr[i + r];
            for (;;) {
                int mn = N;
                for (int r = 0; r < bnl; r++)
                    if (ptr[r] != -1 && cind[ptr[r]] < mn) mn = cind[ptr[r]];
                if (mn == N) break;
                for (int r = 0; r < bnl; r++) {
                    if (ptr[r] == -1) continue;
                    while (cind[ptr[r]] / bnw == mn / bnw) {
                        if (pass == 1)
                            (*bval)[(size_t)cnt * bnl * bnw + (cind[ptr[r]] % bnw) * bnl + r] = val[ptr[r]];
                        ptr[r]++;
                        if (ptr[r] >= rptr[i + r + 1]) { ptr[r] = -1; break; }
                    }
                }
                if (pass == 1) (*bcind)[cnt] = mn / bnw;
                cnt++;
            }
            if (pass == 0) (*brptr)[i / bnl + 1] = cnt;
        }
    }
    free(ptr);
    return 0;
}

/* include/senk_matrix.hpp:213-241  Bcsr2Csr: every block entry becomes a CSR
 * entry (zeros included). Returns nnz. */
int oracle_bcsr2csr(const double *bval, const int *bcind, const int *brptr,
                    double **val, int **cind, int **rptr, int N, int bnl, int bnw)
{
    int bs = bnl * bnw;
    int nblk = brptr[N / bnl];
    *val = (double *)malloc(sizeof(double) * ((size_t)nblk * bs > 0 ? (size_t)nblk * bs : 1));
    *cind = (int *)malloc(sizeof(int) * ((size_t)nblk * bs > 0 ? (size_t)nblk * bs : 1));
    *rptr = (int *)malloc(sizeof(int) * (N + 1));
    (*rptr)[0] = 0;
    int cnt = 0;
    for (int i = 0; i < N; i++) {
        int br = i / bnl, r = i % bnl;
        for (int blk = brptr[br]; blk < brptr[br + 1]; blk++) {
            for (int c = 0; c < bnw; c++) {
                (*cind)[cnt] = bcind[blk] * bnw + c;
                (*val)[cnt] = bval[(size_t)blk * bs + c * bnl + r];
                cnt++;
            }
        }
        (*rptr)[i + 1] = cnt;
    }
    return cnt;
}

/* include/senk_matrix.hpp:257-333  Split with keys "LD-U", "L-DU", "L-D-U",
 * "LU-D"; invDiag stores 1/a_ii. Outputs are malloc'd (u arrays only when the
 * key gives U its own storage, diag only when the diagonal is separate).
 * Returns -1 for an unknown key. */
int oracle_split(const double *val, const int *cind, const int *rptr,
                 double **lval, int **lcind, int **lrptr,
                 double **uval, int **ucind, int **urptr,
                 double **diag, int N, const char *key, int invDiag)
{
    int which; /* 0 LD-U, 1 L-DU, 2 L-D-U, 3 LU-D */
    if (!strcmp(key, "LD-U")) which = 0;
    else if (!strcmp(key, "L-DU")) which = 1;
    else if (!strcmp(key, "L-D-U")) which = 2;
    else if (!strcmp(key, "LU-D")) which = 3;
    else return -1;
    int nL = 0, nU = 0, nD = 0;
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++) {
            if (cind[j] < i) nL++;
            else if (cind[j] > i) nU++;
            else nD++;
        }
    int lN = nL, uN = nU;
    if (which == 0) lN += nD;
    if (which == 1) uN += nD;
    if (which == 3) { lN += nU; uN = 0; }
    *lval = (double *)malloc(sizeof(double) * (lN > 0 ? lN : 1));
    *lcind = (int *)malloc(sizeof(int) * (lN > 0 ? lN : 1));
    *lrptr = (int *)malloc(sizeof(int) * (N + 1));
    if (uN != 0) {
        *uval = (double *)malloc(sizeof(double) * uN);
        *ucind = (int *)malloc(sizeof(int) * uN);
        *urptr = (int *)malloc(sizeof(int) * (N + 1));
    }
    int sepD = (which == 2 || which == 3);
    if (sepD && nD == N && diag) *diag = (double *)malloc(sizeof(double) * N);
    int lc = 0, uc = 0, dc = 0;
    int *lp = &lc, *up = (which == 3) ? &lc : &uc;
    double *lv = *lval, *uv = (which == 3) ? *lval : (uN ? *uval : NULL);
    int *lci = *lcind, *uci = (which == 3) ? *lcind : (uN ? *ucind : NULL);
    int *lr = *lrptr, *ur = (which == 3) ? *lrptr : (uN ? *urptr : NULL);
    lr[0] = 0;
    if (ur) ur[0] = 0;
    for (int i = 0; i < N; i++) {
        for (int j = rptr[i]; j < rptr[i + 1]; j++) {
            double v = val[j];
            if (cind[j] < i) { lv[*lp] = v; lci[*lp] = cind[j]; (*lp)++; }
            else if (cind[j] > i) { uv[*up] = v; uci[*up] = cind[j]; (*up)++; }
            else {
                double d = invDiag ? 1 / v : v;
                if (which == 0) { lv[lc] = d; lci[lc] = cind[j]; lc++; }
                else if (which == 1) { uv[uc] = d; uci[uc] = cind[j]; uc++; }
                else { if (diag && *diag) (*diag)[dc] = d; dc++; }
            }
        }
        lr[i + 1] = *lp;
        if (ur) ur[i + 1] = *up;
    }
    return 0;
}

/* include/senk_matrix.hpp:335-371  Expand: full matrix from the stored
 * triangle (key 'L': lower incl. diagonal stored; 'U': upper). Row i takes the
 * lower-oriented row's entries, then the upper-oriented row's entries after
 * its first (the diagonal). Returns -1 for another key. */
int oracle_expand(const double *tval, const int *tcind, const int *trptr,
                  double **val, int **cind, int **rptr, int N, char key)
{
    if (key != 'L' && key != 'U') return -1;
    double *cv; int *cr, *cp;
    oracle_csr2csc(tval, tcind, trptr, &cv, &cr, &cp, N, N);
    const double *lv = key == 'L' ? tval : cv, *uv = key == 'L' ? cv : tval;
    const int *lc = key == 'L' ? tcind : cr, *uc = key == 'L' ? cr : tcind;
    const int *lr = key == 'L' ? trptr : cp, *ur = key == 'L' ? cp : trptr;
    int nnz = trptr[N] * 2 - N;
    *val = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    *cind = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    *rptr = (int *)malloc(sizeof(int) * (N + 1));
    int at = 0;
    (*rptr)[0] = 0;
    for (int i = 0; i < N; i++) {
        for (int j = lr[i]; j < lr[i + 1]; j++) { (*val)[at] = lv[j]; (*cind)[at] = lc[j]; at++; }
        for (int j = ur[i] + 1; j < ur[i + 1]; j++) { (*val)[at] = uv[j]; (*cind)[at] = uc[j]; at++; }
        (*rptr)[i + 1] = at;
    }
    free(cv); free(cr); free(cp);
    return 0;
}

/* include/senk_io.hpp:41-103  ReadMatrixMarket: header with "symmetric"
 * (*sym = 1) or "general" (0), not "complex"; '%' lines skipped up to the
 * size line "N M PE"; PE triples "row col value" (1-based), zero values dropped
 * when remove_zeros; CSR with rows in order and each row sorted by column
 * (entries of equal row and column keep file order here). Returns -1 for a
 * file the reference would reject or read out of bounds. */
int oracle_read_matrix_market(const char *path, double **val, int **cind, int **rptr,
                              int *N, int *M, int *sym, int remove_zeros)
{
    FILE *f = fopen(path, "r");
    if (!f) return -1;
    char line[4096];
    if (!fgets(line, sizeof line, f) || strstr(line, "complex")) { fclose(f); return -1; }
    if (strstr(line, "symmetric")) *sym = 1;
    else if (strstr(line, "general")) *sym = 0;
    else { fclose(f); return -1; }
    long long n = -1, m = -1, pe = -1;
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '%') continue;
        if (sscanf(line, "%lld %lld %lld", &n, &m, &pe) != 3) n = -1;
        break;
    }
    if (n < 0 || m < 0 || pe < 0) { fclose(f); return -1; }
    int *row = (int *)malloc(sizeof(int) * (pe > 0 ? pe : 1));
    int *col = (int *)malloc(sizeof(int) * (pe > 0 ? pe : 1));
    double *v = (double *)malloc(sizeof(double) * (pe > 0 ? pe : 1));
    long long k = 0;
    for (long long e = 0; e < pe; e++) {
        long long r, c;
        double x;
        if (fscanf(f, "%lld %lld %lf", &r, &c, &x) != 3 || r < 1 || r > n || c < 1 || c > m) {
            free(row); free(col); free(v); fclose(f);
            return -1;
        }
        if (remove_zeros && x == 0) continue;
        row[k] = (int)(r - 1); col[k] = (int)(c - 1); v[k] = x; k++;
    }
    fclose(f);
    *N = (int)n;
    *M = (int)m;
    *rptr = (int *)calloc((size_t)n + 1, sizeof(int));
    *cind = (int *)malloc(sizeof(int) * (k > 0 ? k : 1));
    *val = (double *)malloc(sizeof(double) * (k > 0 ? k : 1));
    for (long long e = 0; e < k; e++) (*rptr)[row[e] + 1]++;
    for (long long i = 0; i < n; i++) (*rptr)[i + 1] += (*rptr)[i];
    int *at = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    memcpy(at, *rptr, sizeof(int) * ((size_t)n + 1));
    for (long long e = 0; e < k; e++) {
        int p = at[row[e]]++;
        (*cind)[p] = col[e];
        (*val)[p] = v[e];
    }
    /* insertion sort of each row by column (stable) */
    for (long long i = 0; i < n; i++) {
        for (int j = (*rptr)[i] + 1; j < (*rptr)[i + 1]; j++) {
            int c = (*cind)[j];
            double x = (*val)[j];
            int q = j - 1;
            while (q >= (*rptr)[i] && (*cind)[q] > c) { (*cind)[q + 1] = (*cind)[q]; (*val)[q + 1] = (*val)[q]; q--; }
            (*cind)[q + 1] = c;
            (*val)[q + 1] = x;
        }
    }
    free(at); free(row); free(col); free(v);
    return 0;
}

/* include/senk_matrix.hpp:391-404  GetDiag */
void oracle_get_diag(const double *val, const int *cind, const int *rptr, double *diag, int N)
{
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++)
            if (cind[j] == i) { diag[i] = val[j]; break; }
}

/* include/senk_matrix.hpp:406-416  Scaling: val_ij = ld_i * val_ij * rd_j */
void oracle_scaling(double *val, const int *cind, const int *rptr,
                    const double *ld, const double *rd, int N)
{
    for (int i = 0; i < N; i++) {
        double left = ld[i];
        for (int j = rptr[i]; j < rptr[i + 1]; j++) val[j] = left * val[j] * rd[cind[j]];
    }
}

/* include/senk_matrix.hpp:418-448  Ilu0: in-place IKJ ILU(0) on a CSR pattern
 * with sorted columns. Returns -1 on a zero pivot (the reference exits). */
int oracle_ilu0(double *val, const int *cind, const int *rptr, int N)
{
    for (int i = 1; i < N; i++) {
        for (int k = rptr[i]; k < rptr[i + 1]; k++) {
            int kc = cind[k];
            if (kc >= i) break;
            for (int l = rptr[kc]; l < rptr[kc + 1]; l++) {
                if (cind[l] == kc) {
                    if (val[l] == 0) return -1;
                    val[k] = val[k] / val[l];
                    break;
                }
            }
            int pos = rptr[kc];
            for (int j = k + 1; j < rptr[i + 1]; j++) {
                for (int l = pos; l < rptr[kc + 1]; l++) {
                    if (cind[l] < cind[j]) continue;
                    pos = l;
                    if (cind[l] == cind[j]) { val[j] -= val[k] * val[l]; pos++; }
                    break;
                }
            }
        }
    }
    return 0;
}

/* Growable (value, level, column) row: the role of sparse::SpVec
 * (include/senk_class.hpp:23-123) in Ilup/AllocLevelZero. */
typedef struct { double *v; int *lev; int *idx; int len, cap; } orow;
static void orow_push(orow *r, double v, int lev, int idx)
{
    if (r->len == r->cap) {
        r->cap = r->cap ? r->cap * 2 : 8;
        r->v = (double *)realloc(r->v, sizeof(double) * r->cap);
        r->lev = (int *)realloc(r->lev, sizeof(int) * r->cap);
        r->idx = (int *)realloc(r->idx, sizeof(int) * r->cap);
    }
    r->v[r->len] = v; r->lev[r->len] = lev; r->idx[r->len] = idx; r->len++;
}

/* include/senk_matrix.hpp:450-549 Ilup (numeric=1) and 551-650 AllocLevelZero
 * (numeric=0: same level-of-fill pattern, values untouched and fill-ins zero).
 * Row i is merged, pivot by pivot, with the already finished upper part of the
 * pivot row; entries whose level exceeds p are carried but not kept. Replaces
 * the val, cind and rptr arrays with malloc'd ones; the caller frees the old ones. */
static void oracle_level_fill(double **val, int **cind, int **rptr, int N, int p, int numeric)
{
    const int *rp = *rptr, *ci = *cind;
    const double *va = *val;
    int first = rp[1] - rp[0];
    int cap = first > 0 ? first : 1;
    double *nv = (double *)malloc(sizeof(double) * cap);
    int *nc = (int *)malloc(sizeof(int) * cap);
    int *nl = (int *)calloc(cap, sizeof(int));
    int *nr = (int *)malloc(sizeof(int) * (N + 1));
    memcpy(nv, va, sizeof(double) * first);
    memcpy(nc, ci, sizeof(int) * first);
    nr[0] = 0;
    nr[1] = first;
    int nlen = first;
    orow a = {0}, b = {0};
    double pivot = 0;
    int pivot_lev = 0;
    for (int i = 1; i < N; i++) {
        a.len = 0;
        for (int j = rp[i]; j < rp[i + 1]; j++) orow_push(&a, va[j], 0, ci[j]);
        int count = 0;
        while (count < a.len && a.idx[count] < i) {
            int kp = count;
            if (a.lev[kp] > p) { count++; continue; }
            int k = a.idx[kp];
            b.len = 0;
            for (int j = 0; j < count; j++) orow_push(&b, a.v[j], a.lev[j], a.idx[j]);
            int j;
            for (j = nr[k]; j < nr[k + 1]; j++) {
                if (nc[j] == k) {
                    pivot = numeric ? a.v[kp] / nv[j] : a.v[kp];
                    pivot_lev = a.lev[kp];
                    break;
                }
            }
            j++;
            kp++;
            orow_push(&b, pivot, 0, k);
            while (kp < a.len || j < nr[k + 1]) {
                int c1 = (kp < a.len) ? a.idx[kp] : N + 1;
                int c2 = (j < nr[k + 1]) ? nc[j] : N + 1;
                if (c1 < c2) {
                    orow_push(&b, a.v[kp], a.lev[kp], a.idx[kp]);
                    kp++;
                } else if (c1 == c2) {
                    double v = numeric ? a.v[kp] - pivot * nv[j] : a.v[kp];
                    int lev = a.lev[kp];
                    if (lev > pivot_lev + nl[j] + 1) lev = pivot_lev + nl[j] + 1;
                    orow_push(&b, v, lev, a.idx[kp]);
                    kp++;
                    j++;
                } else {
                    orow_push(&b, numeric ? -pivot * nv[j] : 0.0, pivot_lev + nl[j] + 1, nc[j]);
                    j++;
                }
            }
            count++;
            orow t = a; a = b; b = t; /* a <- merged row */
        }
        if (nlen + a.len > cap) {
            while (nlen + a.len > cap) cap *= 2;
            nv = (double *)realloc(nv, sizeof(double) * cap);
            nc = (int *)realloc(nc, sizeof(int) * cap);
            nl = (int *)realloc(nl, sizeof(int) * cap);
        }
        for (int j = 0; j < a.len; j++) {
            if (a.lev[j] <= p) { nv[nlen] = a.v[j]; nc[nlen] = a.idx[j]; nl[nlen] = a.lev[j]; nlen++; }
        }
        nr[i + 1] = nlen;
    }
    free(a.v); free(a.lev); free(a.idx); free(b.v); free(b.lev); free(b.idx);
    free(nl);
    *val = nv;
    *cind = nc;
    *rptr = nr;
}
void oracle_ilup(double **val, int **cind, int **rptr, int N, int p) { oracle_level_fill(val, cind, rptr, N, p, 1); }
void oracle_alloc_level_zero(double **val, int **cind, int **rptr, int N, int p) { oracle_level_fill(val, cind, rptr, N, p, 0); }

/* include/senk_matrix.hpp:652-666  AllocBlockZero: CSR -> BCSR -> CSR pads the
 * pattern with explicit zeros to full bnl x bnw blocks. New malloc'd arrays;
 * returns nnz or -1. */
int oracle_alloc_block_zero(double **val, int **cind, int **rptr, int N, int bnl, int bnw)
{
    double *bv; int *bc, *br;
    if (oracle_csr2bcsr(*val, *cind, *rptr, &bv, &bc, &br, N, bnl, bnw)) return -1;
    int nnz = oracle_bcsr2csr(bv, bc, br, val, cind, rptr, N, bnl, bnw);
    free(bv); free(bc); free(br);
    return nnz;
}

/* include/senk_matrix.hpp:668-689  RemoveOffDiagonal (block Jacobi pattern), in
 * place; returns the new nnz. */
int oracle_remove_off_diagonal(double *val, int *cind, int *rptr, int N, int bnum)
{
    int bs = N / bnum, off = 0;
    for (int i = 0; i < N; i++) {
        int start = rptr[i] + off;
        int lo = i / bs * bs, hi = lo + bs;
        for (int j = start; j < rptr[i + 1]; j++) {
            if (cind[j] < lo || hi <= cind[j]) { off++; continue; }
            val[j - off] = val[j];
            cind[j - off] = cind[j];
        }
        rptr[i + 1] -= off;
    }
    return rptr[N];
}

/* Insertion sort of one row by column (columns are distinct in a row, so every
 * correct sort gives the reference QuickSort's result). */
static void sort_row(int *c, double *v, int n)
{
    for (int a = 1; a < n; a++) {
        int kc = c[a]; double kv = v[a]; int b = a - 1;
        while (b >= 0 && c[b] > kc) { c[b + 1] = c[b]; v[b + 1] = v[b]; b--; }
        c[b + 1] = kc; v[b + 1] = kv;
    }
}

/* include/senk_matrix.hpp:703-730  Reordering(LP,RP): A' = P A P^T, row i of A'
 * is row LP[i] of A with columns mapped through RP and re-sorted. In place. */
void oracle_reordering(double *val, int *cind, int *rptr, const int *LP, const int *RP, int N)
{
    int nnz = rptr[N];
    double *tv = (double *)malloc(sizeof(double) * (nnz > 0 ? nnz : 1));
    int *tc = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    int *tr = (int *)malloc(sizeof(int) * (N + 1));
    tr[0] = 0;
    for (int i = 0; i < N; i++) tr[i + 1] = tr[i] + (rptr[LP[i] + 1] - rptr[LP[i]]);
    #pragma omp parallel for
    for (int i = 0; i < N; i++) {
        int id = LP[i], n = rptr[id + 1] - rptr[id];
        for (int j = 0; j < n; j++) {
            tv[tr[i] + j] = val[rptr[id] + j];
            tc[tr[i] + j] = RP[cind[rptr[id] + j]];
        }
        sort_row(&tc[tr[i]], &tv[tr[i]], n);
    }
    memcpy(val, tv, sizeof(double) * nnz);
    memcpy(cind, tc, sizeof(int) * nnz);
    memcpy(rptr, tr, sizeof(int) * (N + 1));
    free(tv); free(tc); free(tr);
}

/* include/senk_matrix.hpp:691-701  Reordering(RP): columns only (symmetric use). */
void oracle_reordering_cols(double *val, int *cind, const int *rptr, const int *RP, int N)
{
    for (int i = 0; i < N; i++) {
        for (int j = rptr[i]; j < rptr[i + 1]; j++) cind[j] = RP[cind[j]];
        sort_row(&cind[rptr[i]], &val[rptr[i]], rptr[i + 1] - rptr[i]);
    }
}

/* ---------------------------------------------------------------- graph --- */

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* include/senk_graph.hpp:27-66  SimpleBlocking: block i = rows [i*bs,(i+1)*bs);
 * block adjacency by merging the rows' column streams block column by block
 * column. */
static void simple_blocking(const int *cind, const int *rptr, int **b_cind, int **b_rptr,
                            int **block, int N, int bs)
{
    *block = (int *)malloc(sizeof(int) * N);
    for (int i = 0; i < N; i++) (*block)[i] = i;
    *b_rptr = (int *)malloc(sizeof(int) * (N / bs + 1));
    *b_cind = (int *)malloc(sizeof(int) * (rptr[N] > 0 ? rptr[N] : 1));
    int *ptr = (int *)malloc(sizeof(int) * bs);
    int cnt = 0;
    (*b_rptr)[0] = 0;
    for (int i = 0; i < N; i += bs) {
        for (int j = 0; j < bs; j++) ptr[j] = rptr[(*block)[i + j]];
        for (;;) {
            int mn = N;
            for (int j = 0; j < bs; j++)
                if (ptr[j] != -1 && cind[ptr[j]] < mn) mn = cind[ptr[j]];
            if (mn == N) break;
            (*b_cind)[cnt] = mn / bs;
            for (int j = 0; j < bs; j++) {
                if (ptr[j] == -1) continue;
                while (cind[ptr[j]] / bs == mn / bs) {
                    ptr[j]++;
                    if (ptr[j] >= rptr[(*block)[i + j] + 1]) { ptr[j] = -1; break; }
                }
            }
            cnt++;
        }
        (*b_rptr)[i / bs + 1] = cnt;
    }
    free(ptr);
}

/* include/senk_graph.hpp:77-139  ConnectedBlocking: BFS from the lowest
 * unvisited row fills blocks of bs rows (a new seed starts whenever the queue
 * empties); each block's rows are then sorted, and the block graph is the set of
 * distinct blocks touched by its rows' columns. Returns -1 on the queue fault the
 * reference exits on. */
static int connected_blocking(const int *cind, const int *rptr, int **b_cind, int **b_rptr,
                              int **block, int N, int bs)
{
    *block = (int *)calloc(N, sizeof(int));
    int *inv = (int *)calloc(N, sizeof(int));
    int *vis = (int *)calloc(N, sizeof(int));
    int *queue = (int *)calloc(bs + 1, sizeof(int));
    int count = 0, tcnt = 0;
    for (int i = 0; i < N; i++) {
        if (vis[i]) continue;
        int qs = 0, qe = 0;
        (*block)[count] = i; count++; tcnt++;
        inv[i] = (count - 1) / bs;
        vis[i] = 1;
        if (tcnt == bs) { tcnt = 0; continue; }
        queue[qe++] = i;
        int full = 0;
        while (!full) {
            int q = queue[qs++];
            for (int j = rptr[q]; j < rptr[q + 1]; j++) {
                int c = cind[j];
                if (vis[c]) continue;
                (*block)[count] = c; count++; tcnt++;
                inv[c] = (count - 1) / bs;
                vis[c] = 1;
                if (tcnt == bs) { tcnt = 0; full = 1; break; }
                queue[qe++] = c;
            }
            if (qs > qe) { free(inv); free(vis); free(queue); return -1; }
            if (qs == qe) break;
        }
    }
    for (int i = 0; i < N; i += bs) qsort(&(*block)[i], bs, sizeof(int), cmp_int);
    *b_rptr = (int *)malloc(sizeof(int) * (N / bs + 1));
    *b_cind = (int *)malloc(sizeof(int) * (rptr[N] > 0 ? rptr[N] : 1));
    int *tmp = (int *)malloc(sizeof(int) * (rptr[N] > 0 ? rptr[N] : 1));
    int cnt = 0;
    (*b_rptr)[0] = 0;
    for (int i = 0; i < N; i += bs) {
        int len = 0;
        for (int j = 0; j < bs; j++) {
            int r = (*block)[i + j];
            for (int k = rptr[r]; k < rptr[r + 1]; k++) tmp[len++] = inv[cind[k]];
        }
        qsort(tmp, len, sizeof(int), cmp_int);
        (*b_cind)[cnt++] = tmp[0];
        int prev = tmp[0];
        for (int j = 1; j < len; j++) {
            if (tmp[j] == prev) continue;
            (*b_cind)[cnt++] = tmp[j];
            prev = tmp[j];
        }
        (*b_rptr)[i / bs + 1] = cnt;
    }
    free(vis); free(queue); free(inv); free(tmp);
    return 0;
}

/* include/senk_graph.hpp:150-209  GetAdjacency: the pattern itself (isSym) or
 * the sorted union of the rows of A and A^T. */
static void get_adjacency(const int *cind, const int *rptr, int **am_cind, int **am_rptr,
                          int N, int isSym)
{
    int nnz = rptr[N];
    *am_rptr = (int *)malloc(sizeof(int) * (N + 1));
    if (isSym) {
        *am_cind = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
        memcpy(*am_cind, cind, sizeof(int) * nnz);
        memcpy(*am_rptr, rptr, sizeof(int) * (N + 1));
        return;
    }
    int *rind = (int *)malloc(sizeof(int) * (nnz > 0 ? nnz : 1));
    int *cptr = (int *)malloc(sizeof(int) * (N + 1));
    int *len = (int *)calloc(N > 0 ? N : 1, sizeof(int));
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++) len[cind[j]]++;
    cptr[0] = 0;
    for (int i = 0; i < N; i++) { cptr[i + 1] = cptr[i] + len[i]; len[i] = 0; }
    for (int i = 0; i < N; i++)
        for (int j = rptr[i]; j < rptr[i + 1]; j++) rind[cptr[cind[j]] + len[cind[j]]++] = i;
    *am_cind = (int *)malloc(sizeof(int) * (2 * nnz > 0 ? 2 * nnz : 1));
    (*am_rptr)[0] = 0;
    int cnt = 0;
    for (int i = 0; i < N; i++) {
        int a = rptr[i], b = cptr[i];
        while (a < rptr[i + 1] || b < cptr[i + 1]) {
            int ca = (a < rptr[i + 1]) ? cind[a] : N;
            int cb = (b < cptr[i + 1]) ? rind[b] : N;
            if (ca < cb) { (*am_cind)[cnt] = ca; a++; }
            else if (ca == cb) { (*am_cind)[cnt] = ca; a++; b++; }
            else { (*am_cind)[cnt] = cb; b++; }
            cnt++;
        }
        (*am_rptr)[i + 1] = cnt;
    }
    free(rind); free(cptr); free(len);
}

/* include/senk_graph.hpp:218-238  Coloring: colour `now` is assigned by one
 * index-order sweep that takes every uncoloured vertex not adjacent to a vertex
 * already given colour `now` (a maximal independent set per colour). */
static int *coloring(const int *cind, const int *rptr, int *num_color, int N)
{
    int *color = (int *)calloc(N > 0 ? N : 1, sizeof(int));
    int *visit = (int *)calloc(N > 0 ? N : 1, sizeof(int));
    int now = 1, cnt = 0;
    while (cnt < N) {
        for (int i = 0; i < N; i++) {
            if (visit[i] == now || color[i] != 0) continue;
            color[i] = now;
            cnt++;
            for (int j = rptr[i]; j < rptr[i + 1]; j++) visit[cind[j]] = now;
        }
        now++;
    }
    *num_color = now - 1;
    free(visit);
    return color;
}

/* include/senk_graph.hpp:250-277  GetAMCPermutation: LP lists rows colour by
 * colour in index order; size_color counts rows; RP = LP^-1. */
void oracle_amc_permutation(const int *cind, const int *rptr, int *num_color,
                            int **size_color, int **LP, int **RP, int N, int isSym)
{
    int *ac, *ar;
    get_adjacency(cind, rptr, &ac, &ar, N, isSym);
    int *color = coloring(ac, ar, num_color, N);
    *LP = (int *)malloc(sizeof(int) * N);
    *RP = (int *)malloc(sizeof(int) * N);
    *size_color = (int *)malloc(sizeof(int) * (*num_color + 1));
    (*size_color)[0] = 0;
    int cnt = 0;
    for (int c = 0; c < *num_color; c++) {
        int n = 0;
        for (int j = 0; j < N; j++)
            if (color[j] - 1 == c) { (*LP)[cnt++] = j; n++; }
        (*size_color)[c + 1] = (*size_color)[c] + n;
    }
    for (int i = 0; i < N; i++) (*RP)[(*LP)[i]] = i;
    free(ac); free(ar); free(color);
}

/* include/senk_graph.hpp:291-334  GetABMCPermutation: rows are grouped into
 * blocks of bsize ("simple" or "connect"), the block graph is coloured, and LP
 * lists the blocks colour by colour (block rows in their sorted order);
 * size_color counts blocks. Returns -1 where the reference exits (N%bsize, bad
 * method, BFS queue fault). */
int oracle_abmc_permutation(const int *cind, const int *rptr, int *num_color,
                            int **size_color, int **LP, int **RP, int N, int bsize,
                            int isSym, const char *bmethod)
{
    if (bsize <= 0 || N % bsize) return -1;
    int *bc, *br, *block;
    if (!strcmp(bmethod, "simple")) simple_blocking(cind, rptr, &bc, &br, &block, N, bsize);
    else if (!strcmp(bmethod, "connect")) {
        if (connected_blocking(cind, rptr, &bc, &br, &block, N, bsize)) return -1;
    } else return -1;
    int nb = N / bsize;
    int *ac, *ar;
    get_adjacency(bc, br, &ac, &ar, nb, isSym);
    int *color = coloring(ac, ar, num_color, nb);
    *LP = (int *)malloc(sizeof(int) * N);
    *RP = (int *)malloc(sizeof(int) * N);
    *size_color = (int *)malloc(sizeof(int) * (*num_color + 1));
    (*size_color)[0] = 0;
    int cnt = 0;
    for (int c = 0; c < *num_color; c++) {
        for (int j = 0; j < nb; j++) {
            if (color[j] - 1 != c) continue;
            for (int k = 0; k < bsize; k++) (*LP)[cnt++] = block[j * bsize + k];
        }
        (*size_color)[c + 1] = cnt / bsize;
    }
    for (int i = 0; i < N; i++) (*RP)[(*LP)[i]] = i;
    free(bc); free(br); free(block); free(ac); free(ar); free(color);
    return 0;
}

/* include/senk_test.hpp:11-22  ||b - A x|| / ||b|| in FP64 */
double oracle_relative_residual(const double *val, const int *cind, const int *rptr,
                                const double *b, const double *x, int N)
{
    double *t = (double *)malloc(sizeof(double) * N);
    oracle_spmv_csr_d(val, cind, rptr, x, t, N);
    oracle_axpby_d(1, b, -1, t, N);
    double r = oracle_nrm2_d(t, N) / oracle_nrm2_d(b, N);
    free(t);
    return r;
}
