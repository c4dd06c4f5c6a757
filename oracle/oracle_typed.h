/*
 * Type-generic body of the oracle (test infrastructure, see senk_oracle.c).
 * Included twice by senk_oracle.c: once with T=double / SFX(name)=name##_d and
 * once with T=float / SFX(name)=name##_s.  Each function restates one reference
 * function of SenK's Krylov path and cites the reference file:line it follows.
 * The loop structure, operation order and OpenMP pragmas follow the reference so
 * that the oracle is both a parity checker and a faithful CPU baseline.
 */

/* ---------------------------------------------------------------- sparse --- */

/* include/senk_sparse.hpp:25-35  SpmvCsr */
void SFX(oracle_spmv_csr)(const T *val, const int *cind, const int *rptr,
                          const T *x, T *y, int N)
{
    #pragma omp parallel for
    for (int i = 0; i < N; i++) {
        T acc = 0;
        for (int j = rptr[i]; j < rptr[i + 1]; j++) acc += val[j] * x[cind[j]];
        y[i] = acc;
    }
}

/* include/senk_sparse.hpp:47-57  SpmvCsr with a separately stored diagonal */
void SFX(oracle_spmv_csr_diag)(const T *val, const int *cind, const int *rptr,
                               const T *diag, const T *x, T *y, int N)
{
    #pragma omp parallel for
    for (int i = 0; i < N; i++) {
        T acc = x[i] * diag[i];
        for (int j = rptr[i]; j < rptr[i + 1]; j++) acc += val[j] * x[cind[j]];
        y[i] = acc;
    }
}

/* include/senk_sparse.hpp:70-91  SpmvBcsr<T,bnl,bnw>; block stored column-major */
void SFX(oracle_spmv_bcsr)(const T *bval, const int *bcind, const int *brptr,
                           const T *x, T *y, int N, int bnl, int bnw)
{
    const int bs = bnl * bnw;
    #pragma omp parallel for
    for (int i = 0; i < N; i += bnl) {
        int br = i / bnl;
        for (int r = 0; r < bnl; r++) y[i + r] = 0;
        for (int blk = brptr[br]; blk < brptr[br + 1]; blk++) {
            int xc = bcind[blk] * bnw;
            for (int c = 0; c < bnw; c++) {
                int off = blk * bs + c * bnl;
                for (int r = 0; r < bnl; r++) y[i + r] += bval[off + r] * x[xc + c];
            }
        }
    }
}

/* include/senk_sparse.hpp:103-121  SpmvSell (reference SELL-c layout, incl. its
 * tail test `i==len-1`, which is only meaningful when N%len==0) */
void SFX(oracle_spmv_sell)(const T *val, const int *cind, const int *wid, int len,
                           const T *x, T *y, int N)
{
    int nslice = (N + len - 1) / len;
    #pragma omp parallel for
    for (int s = 0; s < nslice; s++) {
        int start = wid[s] * len;
        int rows = (s == len - 1 && N % len != 0) ? N % len : len;
        for (int k = 0; k < rows; k++) y[s * len + k] = val[start + k] * x[cind[start + k]];
        for (int c = 1; c < wid[s + 1] - wid[s]; c++) {
            int off = start + c * len;
            for (int k = 0; k < rows; k++) y[s * len + k] += val[off + k] * x[cind[off + k]];
        }
    }
}

/* include/senk_sparse.hpp:132-143  SptrsvCsr_l, sequential, unit lower */
void SFX(oracle_sptrsv_l)(const T *val, const int *cind, const int *rptr,
                          const T *x, T *y, int N)
{
    for (int i = 0; i < N; i++) {
        T t = x[i];
        for (int j = rptr[i]; j < rptr[i + 1]; j++) t -= val[j] * y[cind[j]];
        y[i] = t;
    }
}

/* include/senk_sparse.hpp:154-167  SptrsvCsr_u, sequential; the inverted diagonal
 * is the first entry of each row */
void SFX(oracle_sptrsv_u)(const T *val, const int *cind, const int *rptr,
                          const T *x, T *y, int N)
{
    for (int i = N - 1; i >= 0; i--) {
        T t = x[i];
        int j;
        for (j = rptr[i + 1] - 1; j >= rptr[i] + 1; j--) t -= val[j] * y[cind[j]];
        y[i] = t * val[j];
    }
}

/* include/senk_sparse.hpp:180-201  SptrsvCsr_l, AMC: colours in order, rows of a
 * colour independent */
void SFX(oracle_sptrsv_l_amc)(const T *val, const int *cind, const int *rptr,
                              const T *x, T *y, int N, const int *cptr, int cnum)
{
    (void)N;
    #pragma omp parallel
    {
        for (int k = 0; k < cnum; k++) {
            #pragma omp for
            for (int i = cptr[k]; i < cptr[k + 1]; i++) {
                T t = x[i];
                for (int j = rptr[i]; j < rptr[i + 1]; j++) t -= val[j] * y[cind[j]];
                y[i] = t;
            }
        }
    }
}

/* include/senk_sparse.hpp:214-236  SptrsvCsr_u, AMC: colours in reverse */
void SFX(oracle_sptrsv_u_amc)(const T *val, const int *cind, const int *rptr,
                              const T *x, T *y, int N, const int *cptr, int cnum)
{
    (void)N;
    #pragma omp parallel
    {
        for (int k = cnum - 1; k >= 0; k--) {
            #pragma omp for
            for (int i = cptr[k + 1] - 1; i >= cptr[k]; i--) {
                T t = x[i];
                int j;
                for (j = rptr[i + 1] - 1; j >= rptr[i] + 1; j--) t -= val[j] * y[cind[j]];
                y[i] = t * val[j];
            }
        }
    }
}

/* include/senk_sparse.hpp:250-275  SptrsvCsr_l, ABMC: cptr counts blocks of bsize
 * rows; the rows of one block are solved in order */
void SFX(oracle_sptrsv_l_abmc)(const T *val, const int *cind, const int *rptr,
                               const T *x, T *y, int N, const int *cptr, int cnum,
                               int bsize)
{
    (void)N;
    #pragma omp parallel
    {
        for (int k = 0; k < cnum; k++) {
            #pragma omp for
            for (int b = cptr[k]; b < cptr[k + 1]; b++) {
                for (int l = 0; l < bsize; l++) {
                    int i = b * bsize + l;
                    T t = x[i];
                    for (int j = rptr[i]; j < rptr[i + 1]; j++) t -= val[j] * y[cind[j]];
                    y[i] = t;
                }
            }
        }
    }
}

/* include/senk_sparse.hpp:289-315  SptrsvCsr_u, ABMC */
void SFX(oracle_sptrsv_u_abmc)(const T *val, const int *cind, const int *rptr,
                               const T *x, T *y, int N, const int *cptr, int cnum,
                               int bsize)
{
    (void)N;
    #pragma omp parallel
    {
        for (int k = cnum - 1; k >= 0; k--) {
            #pragma omp for
            for (int b = cptr[k + 1] - 1; b >= cptr[k]; b--) {
                for (int l = bsize - 1; l >= 0; l--) {
                    int i = b * bsize + l;
                    T t = x[i];
                    int j;
                    for (j = rptr[i + 1] - 1; j >= rptr[i] + 1; j--) t -= val[j] * y[cind[j]];
                    y[i] = t * val[j];
                }
            }
        }
    }
}

/* include/senk_sparse.hpp:328-346  SptrsvCsr_l, block Jacobi (bnum equal blocks) */
void SFX(oracle_sptrsv_l_bj)(const T *val, const int *cind, const int *rptr,
                             const T *x, T *y, int N, int bnum)
{
    int bs = N / bnum;
    #pragma omp parallel for num_threads(bnum)
    for (int k = 0; k < bnum; k++) {
        for (int i = k * bs; i < (k + 1) * bs; i++) {
            T t = x[i];
            for (int j = rptr[i]; j < rptr[i + 1]; j++) t -= val[j] * y[cind[j]];
            y[i] = t;
        }
    }
}

/* include/senk_sparse.hpp:359-379  SptrsvCsr_u, block Jacobi */
void SFX(oracle_sptrsv_u_bj)(const T *val, const int *cind, const int *rptr,
                             const T *x, T *y, int N, int bnum)
{
    int bs = N / bnum;
    #pragma omp parallel for num_threads(bnum)
    for (int k = 0; k < bnum; k++) {
        for (int i = (k + 1) * bs - 1; i >= k * bs; i--) {
            T t = x[i];
            int j;
            for (j = rptr[i + 1] - 1; j >= rptr[i] + 1; j--) t -= val[j] * y[cind[j]];
            y[i] = t * val[j];
        }
    }
}

/* One bnl-row block row of the BCSR lower sweep (senk_sparse.hpp:399-415).
 * The reference's row loop is `omp simd` and g++ -O3 builds it from vectors of
 * two doubles: y[xc + c] is read again for every pair of rows (r, r+1), after
 * the pairs before have been updated. This differs from a row-by-row loop
 * (re-read for every row) and from a single read when the block holds a value
 * on the diagonal: Csr2Bcsr (senk_matrix.hpp:144-211) gives an empty L row the
 * next row's first entry. The pairwise reading reproduces the reference's
 * output bit for bit on every block shape it instantiates. */
#define ORACLE_BCSR_LANES 2
static void SFX(bcsr_l_row)(const T *bval, const int *bcind, const int *brptr,
                            const T *x, T *y, int i, int bnl, int bnw)
{
    const int bs = bnl * bnw;
    int br = i / bnl;
    for (int r = 0; r < bnl; r++) y[i + r] = x[i + r];
    for (int blk = brptr[br]; blk < brptr[br + 1]; blk++) {
        int xc = bcind[blk] * bnw;
        for (int c = 0; c < bnw; c++) {
            int off = blk * bs + c * bnl;
            for (int r0 = 0; r0 < bnl; r0 += ORACLE_BCSR_LANES) {
                const T yc = y[xc + c];
                const int r1 = r0 + ORACLE_BCSR_LANES < bnl ? r0 + ORACLE_BCSR_LANES : bnl;
                for (int r = r0; r < r1; r++) y[i + r] -= bval[off + r] * yc;
            }
        }
    }
}

/* One bnl-row block row of the BCSR upper sweep (senk_sparse.hpp:436-464): the
 * off-diagonal blocks after the bnl/bnw leading (diagonal-square) blocks, then a
 * dense back-substitution on the square whose diagonal holds inverses. */
static void SFX(bcsr_u_row)(const T *bval, const int *bcind, const int *brptr,
                            const T *x, T *y, int i, int bnl, int bnw)
{
    const int bs = bnl * bnw;
    const int rem = bnl / bnw;
    int br = i / bnl;
    for (int r = 0; r < bnl; r++) y[i + r] = x[i + r];
    for (int blk = brptr[br + 1] - 1; blk >= brptr[br] + rem; blk--) {
        int xc = bcind[blk] * bnw;
        for (int c = 0; c < bnw; c++) {
            int off = blk * bs + c * bnl;
            for (int r = 0; r < bnl; r++) y[i + r] -= bval[off + r] * y[xc + c];
        }
    }
    int pos = brptr[br] + rem - 1;
    for (int q = rem - 1; q >= 0; q--) {
        for (int c = bnw - 1; c >= 0; c--) {
            int off = pos * bs + c * bnl;
            int idx = q * bnw + c;
            y[i + idx] *= bval[off + idx];
            for (int l = q * bnw + c - 1; l >= 0; l--) y[i + l] -= bval[off + l] * y[i + idx];
        }
        pos--;
    }
}

/* include/senk_sparse.hpp:392-416  SptrsvBcsr_l, sequential */
void SFX(oracle_sptrsv_bcsr_l)(const T *bval, const int *bcind, const int *brptr,
                               const T *x, T *y, int N, int bnl, int bnw)
{
    for (int i = 0; i < N; i += bnl) SFX(bcsr_l_row)(bval, bcind, brptr, x, y, i, bnl, bnw);
}

/* include/senk_sparse.hpp:429-465  SptrsvBcsr_u, sequential */
void SFX(oracle_sptrsv_bcsr_u)(const T *bval, const int *bcind, const int *brptr,
                               const T *x, T *y, int N, int bnl, int bnw)
{
    for (int i = N - bnl; i >= 0; i -= bnl) SFX(bcsr_u_row)(bval, bcind, brptr, x, y, i, bnl, bnw);
}

/* include/senk_sparse.hpp:481-517  SptrsvBcsr_l, ABMC */
void SFX(oracle_sptrsv_bcsr_l_abmc)(const T *bval, const int *bcind, const int *brptr,
                                    const T *x, T *y, int N, const int *cptr, int cnum,
                                    int bsize, int bnl, int bnw)
{
    (void)N;
    #pragma omp parallel
    {
        for (int k = 0; k < cnum; k++) {
            #pragma omp for
            for (int b = cptr[k]; b < cptr[k + 1]; b++)
                for (int l = 0; l < bsize; l += bnl)
                    SFX(bcsr_l_row)(bval, bcind, brptr, x, y, b * bsize + l, bnl, bnw);
        }
    }
}

/* include/senk_sparse.hpp:533-581  SptrsvBcsr_u, ABMC */
void SFX(oracle_sptrsv_bcsr_u_abmc)(const T *bval, const int *bcind, const int *brptr,
                                    const T *x, T *y, int N, const int *cptr, int cnum,
                                    int bsize, int bnl, int bnw)
{
    (void)N;
    #pragma omp parallel
    {
        for (int k = cnum - 1; k >= 0; k--) {
            #pragma omp for
            for (int b = cptr[k + 1] - 1; b >= cptr[k]; b--)
                for (int l = bsize - bnl; l >= 0; l -= bnl)
                    SFX(bcsr_u_row)(bval, bcind, brptr, x, y, b * bsize + l, bnl, bnw);
        }
    }
}

/* ----------------------------------------------------------------- blas1 --- */

/* include/senk_blas1.hpp:26-30 */
void SFX(oracle_copy)(const T *x, T *y, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) y[i] = x[i];
}
/* include/senk_blas1.hpp:38-42 */
void SFX(oracle_scal)(T a, T *x, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) x[i] *= a;
}
/* include/senk_blas1.hpp:51-55 */
void SFX(oracle_axpy)(T a, const T *x, T *y, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) y[i] += a * x[i];
}
/* include/senk_blas1.hpp:65-69 */
void SFX(oracle_axpby)(T a, const T *x, T b, T *y, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) y[i] = a * x[i] + b * y[i];
}
/* include/senk_blas1.hpp:79-83 */
void SFX(oracle_axpyz)(T a, const T *x, const T *y, T *z, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) z[i] = a * x[i] + y[i];
}
/* include/senk_blas1.hpp:92-98 */
T SFX(oracle_dot)(const T *x, const T *y, int N)
{
    T res = 0;
    #pragma omp parallel for simd reduction(+ : res)
    for (int i = 0; i < N; i++) res += x[i] * y[i];
    return res;
}
/* include/senk_blas1.hpp:106-112 */
T SFX(oracle_nrm2)(const T *x, int N)
{
    T res = 0;
    #pragma omp parallel for simd reduction(+ : res)
    for (int i = 0; i < N; i++) res += x[i] * x[i];
    return SQRT(res);
}
/* include/senk_blas1.hpp:120-124 */
void SFX(oracle_hadprod)(const T *x, T *y, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) y[i] *= x[i];
}
/* include/senk_blas1.hpp:132-136 */
void SFX(oracle_haddiv)(const T *x, T *y, int N)
{
    #pragma omp parallel for simd
    for (int i = 0; i < N; i++) y[i] /= x[i];
}
/* include/senk_blas1.hpp:145-153  Givens generation */
T SFX(oracle_ggen)(T a, T b, T *c, T *s)
{
    T r = SQRT(a * a + b * b);
    *c = a / r;
    *s = -b / r;
    return r;
}
/* include/senk_blas1.hpp:162-168  Givens application */
void SFX(oracle_grot)(T c, T s, T *a, T *b)
{
    T t = *a;
    *a = c * t - s * *b;
    *b = s * t + c * *b;
}
/* include/senk_blas2.hpp:24-34  back-solve of the column-major Hessenberg (ld n) */
void SFX(oracle_trsv)(const T *U, const T *b, T *x, int n, int m)
{
    for (int i = m - 1; i >= 0; i--) {
        T t = b[i];
        for (int j = m - 1; j > i; j--) t -= U[j * n + i] * x[j];
        x[i] = t / U[i * n + i];
    }
}

/* -------------------------------------------------------------- solvers --- */

/* Operator: CSR (every solver but the block Gmresm) or BCSR
 * (senk_gmres.hpp:113-175). */
typedef struct {
    int kind; /* ORACLE_OP_CSR / ORACLE_OP_BCSR */
    const T *val; const int *cind; const int *rptr;
    int bnl, bnw;
} SFX(oracle_op);

/* Preconditioner applied as the reference's solvers apply it: L sweep into t,
 * then U sweep in place (senk_gmres.hpp:221-222, senk_gcr.hpp:328-329). */
typedef struct {
    int kind; /* ORACLE_PC_* */
    const T *lval; const int *lcind; const int *lrptr;
    const T *uval; const int *ucind; const int *urptr;
    const int *cptr; int cnum; int bsize; int bnum; int bnl, bnw;
} SFX(oracle_prec);

static void SFX(op_apply)(const SFX(oracle_op) *A, const T *x, T *y, int N)
{
    if (A->kind == ORACLE_OP_BCSR)
        SFX(oracle_spmv_bcsr)(A->val, A->cind, A->rptr, x, y, N, A->bnl, A->bnw);
    else
        SFX(oracle_spmv_csr)(A->val, A->cind, A->rptr, x, y, N);
}

static void SFX(prec_apply)(const SFX(oracle_prec) *P, const T *in, T *out, int N)
{
    switch (P->kind) {
    case ORACLE_PC_ILU:
        SFX(oracle_sptrsv_l)(P->lval, P->lcind, P->lrptr, in, out, N);
        SFX(oracle_sptrsv_u)(P->uval, P->ucind, P->urptr, out, out, N);
        break;
    case ORACLE_PC_ILU_AMC:
        SFX(oracle_sptrsv_l_amc)(P->lval, P->lcind, P->lrptr, in, out, N, P->cptr, P->cnum);
        SFX(oracle_sptrsv_u_amc)(P->uval, P->ucind, P->urptr, out, out, N, P->cptr, P->cnum);
        break;
    case ORACLE_PC_ILU_ABMC:
        SFX(oracle_sptrsv_l_abmc)(P->lval, P->lcind, P->lrptr, in, out, N, P->cptr, P->cnum, P->bsize);
        SFX(oracle_sptrsv_u_abmc)(P->uval, P->ucind, P->urptr, out, out, N, P->cptr, P->cnum, P->bsize);
        break;
    case ORACLE_PC_ILU_BJ:
        SFX(oracle_sptrsv_l_bj)(P->lval, P->lcind, P->lrptr, in, out, N, P->bnum);
        SFX(oracle_sptrsv_u_bj)(P->uval, P->ucind, P->urptr, out, out, N, P->bnum);
        break;
    case ORACLE_PC_ILUB:
        SFX(oracle_sptrsv_bcsr_l)(P->lval, P->lcind, P->lrptr, in, out, N, P->bnl, P->bnw);
        SFX(oracle_sptrsv_bcsr_u)(P->uval, P->ucind, P->urptr, out, out, N, P->bnl, P->bnw);
        break;
    case ORACLE_PC_ILUB_ABMC:
        SFX(oracle_sptrsv_bcsr_l_abmc)(P->lval, P->lcind, P->lrptr, in, out, N, P->cptr, P->cnum, P->bsize, P->bnl, P->bnw);
        SFX(oracle_sptrsv_bcsr_u_abmc)(P->uval, P->ucind, P->urptr, out, out, N, P->cptr, P->cnum, P->bsize, P->bnl, P->bnw);
        break;
    default: /* no preconditioner: K = I */
        SFX(oracle_copy)(in, out, N);
        break;
    }
}

/* GMRES(m) with MGS Arnoldi and Givens least squares.
 *  - P->kind == ORACLE_PC_NONE: include/senk_gmres.hpp:33-95 (CSR) and 113-175
 *    (BCSR), final update x += sum y_k V_k.
 *  - otherwise right-preconditioned: senk_gmres.hpp:197-270 (ILU), 293-367 (AMC),
 *    391-465 (ABMC), 487-561 (block Jacobi), 582-655 (ILUB), 679-753 (ABMC ILUB);
 *    final update V0 = y0 V0 + sum y_k V_k, t = K V0, x += t.
 * Convergence: |e_{j+1}| <= nrm_b*eps on the implicit residual. */
int SFX(oracle_gmres)(const SFX(oracle_op) *A, const SFX(oracle_prec) *P,
                      const T *b, T *x, T nrm_b, int outer, int m, int N, T eps,
                      int verbose, oracle_result *res)
{
    T *c = (T *)malloc(sizeof(T) * m);
    T *s = (T *)malloc(sizeof(T) * m);
    T *e = (T *)malloc(sizeof(T) * (m + 1));
    T *H = (T *)malloc(sizeof(T) * (size_t)(m + 1) * m);
    T *V = (T *)malloc(sizeof(T) * (size_t)N * (m + 1));
    T *y = (T *)malloc(sizeof(T) * m);
    T *t = (T *)malloc(sizeof(T) * N);
    if (!c || !s || !e || !H || !V || !y || !t) return -1;
    const int ld = m + 1;
    int flag = 0;
    res->iters = outer * m;
    res->res = -1;
    res->converged = 0;
    for (int i = 0; i < outer; i++) {
        SFX(op_apply)(A, x, &V[0], N);
        SFX(oracle_axpby)(1, b, -1, &V[0], N);
        e[0] = SFX(oracle_nrm2)(&V[0], N);
        SFX(oracle_scal)(1 / e[0], &V[0], N);
        int j;
        for (j = 0; j < m; j++) {
            T *vj = &V[(size_t)j * N], *w = &V[(size_t)(j + 1) * N];
            if (P->kind == ORACLE_PC_NONE) {
                SFX(op_apply)(A, vj, w, N);
            } else {
                SFX(prec_apply)(P, vj, t, N);
                SFX(op_apply)(A, t, w, N);
            }
            for (int k = 0; k <= j; k++) {
                H[j * ld + k] = SFX(oracle_dot)(&V[(size_t)k * N], w, N);
                SFX(oracle_axpy)(-H[j * ld + k], &V[(size_t)k * N], w, N);
            }
            H[j * ld + j + 1] = SFX(oracle_nrm2)(w, N);
            SFX(oracle_scal)(1 / H[j * ld + j + 1], w, N);
            for (int k = 0; k < j; k++)
                SFX(oracle_grot)(c[k], s[k], &H[j * ld + k], &H[j * ld + k + 1]);
            H[j * ld + j] = SFX(oracle_ggen)(H[j * ld + j], H[j * ld + j + 1], &c[j], &s[j]);
            H[j * ld + j + 1] = 0;
            e[j + 1] = s[j] * e[j];
            e[j] = c[j] * e[j];
            if (FABS(e[j + 1]) <= nrm_b * eps) {
                res->iters = i * m + j + 1;
                res->res = (double)(FABS(e[j + 1]) / nrm_b);
                res->converged = 1;
                if (verbose) {
                    printf("I iter %d\n", res->iters);
                    printf("# res %e\n", res->res);
                }
                j++;
                flag = 1;
                break;
            }
        }
        SFX(oracle_trsv)(H, e, y, m + 1, j);
        if (P->kind == ORACLE_PC_NONE) {
            for (int k = 0; k < j; k++) SFX(oracle_axpy)(y[k], &V[(size_t)k * N], x, N);
        } else {
            SFX(oracle_scal)(y[0], &V[0], N);
            for (int k = 1; k < j; k++) SFX(oracle_axpy)(y[k], &V[(size_t)k * N], &V[0], N);
            SFX(prec_apply)(P, &V[0], t, N);
            SFX(oracle_axpy)(1, t, x, N);
        }
        if (flag) break;
    }
    if (!flag && verbose) {
        printf("# iter %d\n", outer * m);
        printf("# res : Check by using senk::test\n");
    }
    free(c); free(s); free(e); free(H); free(V); free(y); free(t);
    return 0;
}

/* GCR(m): include/senk_gcr.hpp:30-72 (K = I), 93-142 (ILU), 163-212 (ILUB).
 * The residual is tested only at restart boundaries; iters = i*m there. */
int SFX(oracle_gcr)(const SFX(oracle_op) *A, const SFX(oracle_prec) *P,
                    const T *b, T *x, T nrm_b, int outer, int m, int N, T eps,
                    int verbose, oracle_result *res)
{
    T *r = (T *)malloc(sizeof(T) * N);
    T *Kr = (T *)malloc(sizeof(T) * N);
    T *p = (T *)malloc(sizeof(T) * (size_t)N * (m + 1));
    T *Ap = (T *)malloc(sizeof(T) * (size_t)N * (m + 1));
    T *AKr = (T *)malloc(sizeof(T) * N);
    T *dAp = (T *)malloc(sizeof(T) * (m + 1));
    if (!r || !Kr || !p || !Ap || !AKr || !dAp) return -1;
    T alpha, beta, nrm_r;
    res->iters = outer * m;
    res->res = -1;
    res->converged = 0;
    for (int i = 0; i < outer; i++) {
        SFX(op_apply)(A, x, r, N);
        SFX(oracle_axpby)(1, b, -1, r, N);
        SFX(prec_apply)(P, r, &p[0], N);
        nrm_r = SFX(oracle_nrm2)(r, N);
        res->res = (double)(nrm_r / nrm_b);
        if (verbose) printf("%d %e\n", i * m, res->res);
        if (nrm_r < nrm_b * eps) {
            res->iters = i * m;
            res->converged = 1;
            break;
        }
        SFX(op_apply)(A, &p[0], &Ap[0], N);
        for (int j = 0; j < m; j++) {
            T *pj = &p[(size_t)j * N], *Apj = &Ap[(size_t)j * N];
            T *pn = &p[(size_t)(j + 1) * N], *Apn = &Ap[(size_t)(j + 1) * N];
            dAp[j] = SFX(oracle_dot)(Apj, Apj, N);
            alpha = SFX(oracle_dot)(Apj, r, N) / dAp[j];
            SFX(oracle_axpy)(alpha, pj, x, N);
            SFX(oracle_axpy)(-alpha, Apj, r, N);
            SFX(prec_apply)(P, r, Kr, N);
            SFX(op_apply)(A, Kr, AKr, N);
            beta = -SFX(oracle_dot)(&Ap[0], AKr, N) / dAp[0];
            SFX(oracle_axpyz)(beta, &p[0], Kr, pn, N);
            SFX(oracle_axpyz)(beta, &Ap[0], AKr, Apn, N);
            for (int k = 1; k <= j; k++) {
                beta = -SFX(oracle_dot)(&Ap[(size_t)k * N], AKr, N) / dAp[k];
                SFX(oracle_axpy)(beta, &p[(size_t)k * N], pn, N);
                SFX(oracle_axpy)(beta, &Ap[(size_t)k * N], Apn, N);
            }
        }
    }
    free(r); free(Kr); free(p); free(Ap); free(AKr); free(dAp);
    return 0;
}

/* BiCGStab: include/senk_bicgstab.hpp:29-87 (K = I), 107-176 (ILU), 198-267 (ILUB).
 * The recursively updated residual is tested every iteration. */
int SFX(oracle_bicgstab)(const SFX(oracle_op) *A, const SFX(oracle_prec) *P,
                         const T *b, T *x, T nrm_b, int max_iter, int N, T eps,
                         int verbose, oracle_result *res)
{
    T *r = (T *)malloc(sizeof(T) * N), *rs = (T *)malloc(sizeof(T) * N);
    T *p = (T *)malloc(sizeof(T) * N), *Kp = (T *)malloc(sizeof(T) * N);
    T *AKp = (T *)malloc(sizeof(T) * N), *s = (T *)malloc(sizeof(T) * N);
    T *Ks = (T *)malloc(sizeof(T) * N), *AKs = (T *)malloc(sizeof(T) * N);
    T *tmp = (T *)malloc(sizeof(T) * N);
    if (!r || !rs || !p || !Kp || !AKp || !s || !Ks || !AKs || !tmp) return -1;
    T alpha, beta, omega, r_rs, prev;
    T nrm_r = nrm_b;
    int i, flag = 0;
    res->converged = 0;
    SFX(op_apply)(A, x, r, N);
    SFX(oracle_axpby)(1, b, -1, r, N);
    SFX(oracle_copy)(r, rs, N);
    SFX(oracle_copy)(r, p, N);
    r_rs = SFX(oracle_dot)(r, rs, N);
    for (i = 0; i < max_iter; i++) {
        SFX(prec_apply)(P, p, Kp, N);
        SFX(op_apply)(A, Kp, AKp, N);
        alpha = r_rs / SFX(oracle_dot)(AKp, rs, N);
        SFX(oracle_axpyz)(-alpha, AKp, r, s, N);
        SFX(prec_apply)(P, s, Ks, N);
        SFX(op_apply)(A, Ks, AKs, N);
        omega = SFX(oracle_dot)(AKs, s, N) / SFX(oracle_dot)(AKs, AKs, N);
        SFX(oracle_axpy)(alpha, Kp, x, N);
        SFX(oracle_axpy)(omega, Ks, x, N);
        SFX(oracle_axpyz)(-omega, AKs, s, r, N);
        nrm_r = SFX(oracle_nrm2)(r, N);
        if (verbose) printf("%d %e\n", i + 1, (double)(nrm_r / nrm_b));
        if (nrm_r < eps * nrm_b) {
            if (verbose) {
                printf("# iter %d\n", i + 1);
                printf("# res %e\n", (double)(nrm_r / nrm_b));
            }
            flag = 1;
            break;
        }
        prev = r_rs;
        r_rs = SFX(oracle_dot)(r, rs, N);
        beta = alpha / omega * r_rs / prev;
        SFX(oracle_axpyz)(-omega, AKp, p, tmp, N);
        SFX(oracle_axpyz)(beta, tmp, r, p, N);
    }
    res->iters = flag ? i + 1 : i;
    res->res = (double)(nrm_r / nrm_b);
    res->converged = flag;
    if (!flag && verbose) {
        printf("# iter %d (max)\n", i);
        printf("# res %e\n", (double)(nrm_r / nrm_b));
    }
    free(r); free(rs); free(p); free(Kp); free(AKp); free(s); free(Ks); free(AKs); free(tmp);
    return 0;
}
