/* CPU restatement of the reference's AMG setup.  TEST INFRASTRUCTURE ONLY.
 *
 * The oracle's own copy of helper::multigrid::get_amg_set (Ruge-Stueben
 * coarsening, direct interpolation, Galerkin product) with the level loop and
 * the data preparation of the intAMGflex and dfAMG constructors (row scaling of
 * the coarse levels, SOR split, exact LU of the coarsest level, fixed-point
 * conversion rules).  Each function cites the reference lines it follows.  It
 * lets the oracle build a hierarchy from a matrix without the product (the
 * CPU-baseline and reference legs of bench.py), and it is pinned bit for bit
 * against the reference hierarchies stored in tests/golden
 * (tests/test_oracle_setup.py).
 *
 * Every FP64 operation is written in the reference's order; the file is
 * compiled without FP contraction. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ------------------------------------------------------------ containers */

typedef struct { int n, m; int32_t *rptr, *cind; double *val; } dmat;
typedef struct { int n, m; int32_t *rptr, *cind; int32_t *val; int bit, dbit; } imat;

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) abort();
    return p;
}
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s);
    if (!p) abort();
    return p;
}
static void *xrealloc(void *p, size_t n) {
    p = realloc(p, n ? n : 1);
    if (!p) abort();
    return p;
}

static dmat dmat_new(int n, int m, int64_t nnz) {
    dmat A;
    A.n = n;
    A.m = m;
    A.rptr = (int32_t *)xcalloc((size_t)n + 1, sizeof(int32_t));
    A.cind = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)nnz);
    A.val = (double *)xmalloc(sizeof(double) * (size_t)nnz);
    return A;
}
static void dmat_free(dmat *A) {
    free(A->rptr); free(A->cind); free(A->val);
    A->rptr = A->cind = NULL;
    A->val = NULL;
}
static dmat dmat_copy(const dmat *A) {
    const int64_t nnz = A->rptr[A->n];
    dmat B = dmat_new(A->n, A->m, nnz);
    memcpy(B.rptr, A->rptr, sizeof(int32_t) * ((size_t)A->n + 1));
    memcpy(B.cind, A->cind, sizeof(int32_t) * (size_t)nnz);
    memcpy(B.val, A->val, sizeof(double) * (size_t)nnz);
    return B;
}
static void imat_free(imat *A) {
    free(A->rptr); free(A->cind); free(A->val);
    A->rptr = A->cind = A->val = NULL;
}

/* (int)(double) as g++ compiles it on x86-64 (cvttsd2si): truncation, INT_MIN
 * when out of range */
static int32_t cvt_i32(double v) {
    if (!(v > -2147483649.0 && v < 2147483648.0)) return (int32_t)0x80000000u;
    return (int32_t)v;
}

/* ---------------------------------------------- utils::QuickSort (sort.hpp:31-51) */

static void swap_i(int32_t *a, int i, int j) {
    const int32_t t = a[i];
    a[i] = a[j];
    a[j] = t;
}

/* key plus up to three companion arrays (NULL where unused), Hoare partition
 * around the middle key, the same swap sequence as the reference */
static void quicksort(int left, int right, int asc, int32_t *key, int32_t *c1, int32_t *c2, int32_t *c3) {
    int L = left, R = right;
    const int32_t pivot = key[(left + right) / 2];
    for (;;) {
        if (asc) {
            while (key[L] < pivot) L++;
            while (pivot < key[R]) R--;
        } else {
            while (key[L] > pivot) L++;
            while (pivot > key[R]) R--;
        }
        if (L >= R) break;
        swap_i(key, L, R);
        if (c1) swap_i(c1, L, R);
        if (c2) swap_i(c2, L, R);
        if (c3) swap_i(c3, L, R);
        L++;
        R--;
    }
    if (left < L - 1) quicksort(left, L - 1, asc, key, c1, c2, c3);
    if (R + 1 < right) quicksort(R + 1, right, asc, key, c1, c2, c3);
}

/* ------------------------------------------- get_amg_set (helper_multigrid.hpp) */

/* get_strong_weak_set (helper_multigrid.hpp:68-110): strong = off-diagonal
 * |a_ij| >= theta max_k!=i |a_ik|; everything else (the diagonal included) weak */
static void strong_weak(const dmat *A, double theta, dmat *S, dmat *W) {
    const int N = A->n;
    double *mx = (double *)xcalloc((size_t)N, sizeof(double));
    int64_t ns = 0;
    for (int i = 0; i < N; i++) {
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++)
            if (A->cind[j] != i && fabs(A->val[j]) > mx[i]) mx[i] = fabs(A->val[j]);
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++)
            if (A->cind[j] != i && fabs(A->val[j]) >= theta * mx[i]) ns++;
    }
    *S = dmat_new(N, N, ns);
    *W = dmat_new(N, N, (int64_t)A->rptr[N] - ns);
    int s = 0, w = 0;
    for (int i = 0; i < N; i++) {
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            if (A->cind[j] != i && fabs(A->val[j]) >= theta * mx[i]) {
                S->val[s] = A->val[j];
                S->cind[s++] = A->cind[j];
            } else {
                W->val[w] = A->val[j];
                W->cind[w++] = A->cind[j];
            }
        }
        S->rptr[i + 1] = s;
        W->rptr[i + 1] = w;
    }
    free(mx);
}

/* get_influence_set (helper_multigrid.hpp:113-136): the transpose pattern */
static void influence(const dmat *S, int32_t **trp, int32_t **tci) {
    const int N = S->n;
    int32_t *num = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    for (int i = 0; i < N; i++)
        for (int j = S->rptr[i]; j < S->rptr[i + 1]; j++) num[S->cind[j]]++;
    int32_t *rp = (int32_t *)xmalloc(sizeof(int32_t) * ((size_t)N + 1));
    int32_t *ci = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)S->rptr[N]);
    rp[0] = 0;
    for (int i = 0; i < N; i++) {
        rp[i + 1] = rp[i] + num[i];
        num[i] = 0;
    }
    for (int i = 0; i < N; i++)
        for (int j = S->rptr[i]; j < S->rptr[i + 1]; j++) {
            const int c = S->cind[j];
            ci[rp[c] + num[c]++] = i;
        }
    free(num);
    *trp = rp;
    *tci = ci;
}

#define UNSET (-38) /* a point neither pass has classified (helper_multigrid.hpp:155) */

/* first_pass (helper_multigrid.hpp:138-266) */
static int32_t *first_pass(const dmat *S, const int32_t *trp, const int32_t *tci) {
    const int N = S->n;
    int32_t *isc = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)N);
    int32_t *vis = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    int32_t *stc = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    int32_t *sc = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    int32_t *infl = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    int32_t *idx = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    int32_t *where = (int32_t *)xcalloc((size_t)N, sizeof(int32_t));
    for (int i = 0; i < N; i++) {
        stc[i] = trp[i + 1] - trp[i];
        sc[i] = S->rptr[i + 1] - S->rptr[i];
        idx[i] = i;
        if (stc[i] == 0 && sc[i] == 0) {
            isc[i] = 0;
            vis[i] = 1;
        } else {
            isc[i] = UNSET;
        }
        for (int j = trp[i]; j < trp[i + 1]; j++) infl[i] += S->rptr[tci[j] + 1] - S->rptr[tci[j]];
    }
    if (N > 0) quicksort(0, N - 1, 0, stc, sc, infl, idx);
    int maxc = N > 0 ? stc[0] : 0;
    int cap = maxc + 2;
    int32_t *cp = (int32_t *)xcalloc((size_t)cap, sizeof(int32_t));
    int ncp = maxc + 2;
    cp[maxc + 1] = 0;
    int strt = 0;
    for (int i = maxc; i >= 0; i--) {
        int num = 0, cut = 0;
        for (int j = strt; j < N; j++) {
            if (stc[j] == i) {
                num++;
            } else {
                cp[i] = cp[i + 1] + num;
                strt = j;
                cut = 1;
                break;
            }
        }
        if (cut) continue;
        cp[i] = cp[i + 1] + num;
    }
    for (int i = maxc; i >= 0; i--)
        if (cp[i] - cp[i + 1] > 1) quicksort(cp[i + 1], cp[i] - 1, 1, infl, idx, NULL, NULL);
    for (int i = 0; i < N; i++) where[idx[i]] = i;
    int pos = 0;
    while (pos < N) {
        while (pos < N && vis[idx[pos]]) pos++;
        if (pos >= N) break;
        const int c = idx[pos];
        vis[c] = 1;
        isc[c] = 1;
        for (int t = trp[c]; t < trp[c + 1]; t++) {
            const int f = tci[t];
            if (vis[f]) continue;
            vis[f] = 1;
            isc[f] = 0;
            for (int j = S->rptr[f]; j < S->rptr[f + 1]; j++) {
                if (vis[S->cind[j]]) continue;
                const int k = where[S->cind[j]];
                stc[k]++;
                int obj;
                if (stc[k] > maxc) {
                    maxc = stc[k];
                    obj = pos + 1;
                    if (ncp + 1 > cap) {
                        cap = 2 * (ncp + 1);
                        cp = (int32_t *)xrealloc(cp, sizeof(int32_t) * (size_t)cap);
                    }
                    cp[ncp++] = pos + 1; /* crdnl_ptr.push_back(pos+1) */
                    cp[maxc] = pos + 2;
                } else if (cp[stc[k]] > pos + 1) {
                    obj = cp[stc[k]];
                    cp[stc[k]] += 1;
                } else {
                    obj = pos + 1;
                    cp[stc[k]] = pos + 2;
                }
                swap_i(stc, k, obj);
                swap_i(idx, k, obj);
                swap_i(where, idx[k], idx[obj]);
            }
        }
        for (int j = S->rptr[c]; j < S->rptr[c + 1]; j++) {
            if (vis[S->cind[j]]) continue;
            const int k = where[S->cind[j]];
            if (stc[k] == 0) continue;
            stc[k]--;
            const int obj = cp[stc[k] + 1] - 1;
            cp[stc[k] + 1] -= 1;
            swap_i(stc, k, obj);
            swap_i(idx, k, obj);
            swap_i(where, idx[k], idx[obj]);
        }
        pos++;
    }
    free(vis); free(stc); free(sc); free(infl); free(idx); free(where); free(cp);
    return isc;
}

/* second_pass (helper_multigrid.hpp:378-417): a fine point with a strong fine
 * neighbour that shares no strong coarse point with it becomes coarse.
 * Returns -1 where the reference exits (an unclassified point). */
static int second_pass(const dmat *S, int32_t *isc) {
    const int N = S->n;
    for (int i = 0; i < N; i++) {
        if (isc[i] == UNSET) return -1;
        if (isc[i]) continue;
        for (int j = S->rptr[i]; j < S->rptr[i + 1]; j++) {
            const int f = S->cind[j];
            if (isc[f]) continue;
            int shared = 0, a = S->rptr[i], b = S->rptr[f];
            while (a < S->rptr[i + 1] && b < S->rptr[f + 1]) {
                if (S->cind[b] < S->cind[a]) {
                    b++;
                } else if (S->cind[b] == S->cind[a]) {
                    if (isc[S->cind[a]]) {
                        shared = 1;
                        break;
                    }
                    b++;
                    a++;
                } else {
                    a++;
                }
            }
            if (shared) continue;
            isc[i] = 1;
            break;
        }
    }
    return 0;
}

/* sepalate_strong_to_coarse_fine + get_interpolation_matrix
 * (helper_multigrid.hpp:419-532).  Returns -1 where the reference exits
 * ("2 amk = 0"); *warn counts its "1 amk = 0" messages. */
static int interpolation(const dmat *A, const dmat *S, const dmat *W, const int32_t *isc, dmat *P, long *warn) {
    const int N = A->n;
    int32_t *col = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)N);
    int count = 0;
    for (int i = 0; i < N; i++)
        if (isc[i]) col[i] = count++;
    /* strong coarse (C) and strong fine (F) entries of each row, in row order */
    int32_t *crp = (int32_t *)xcalloc((size_t)N + 1, sizeof(int32_t));
    int32_t *frp = (int32_t *)xcalloc((size_t)N + 1, sizeof(int32_t));
    for (int i = 0; i < N; i++) {
        crp[i + 1] = crp[i];
        frp[i + 1] = frp[i];
        for (int j = S->rptr[i]; j < S->rptr[i + 1]; j++) {
            if (isc[S->cind[j]]) crp[i + 1]++;
            else frp[i + 1]++;
        }
    }
    int32_t *cci = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)crp[N]);
    double *cv = (double *)xmalloc(sizeof(double) * (size_t)crp[N]);
    int32_t *fci = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)frp[N]);
    double *fv = (double *)xmalloc(sizeof(double) * (size_t)frp[N]);
    for (int i = 0; i < N; i++) {
        int a = crp[i], b = frp[i];
        for (int j = S->rptr[i]; j < S->rptr[i + 1]; j++) {
            if (isc[S->cind[j]]) {
                cci[a] = S->cind[j];
                cv[a++] = S->val[j];
            } else {
                fci[b] = S->cind[j];
                fv[b++] = S->val[j];
            }
        }
    }
    int64_t nnz = 0;
    for (int i = 0; i < N; i++) nnz += isc[i] ? 1 : crp[i + 1] - crp[i];
    *P = dmat_new(N, count, nnz);
    int q = 0, rc = 0;
    for (int i = 0; i < N && rc == 0; i++) {
        if (isc[i]) {
            P->val[q] = 1;
            P->cind[q++] = col[i];
        } else {
            double deno = 0;
            for (int j = W->rptr[i]; j < W->rptr[i + 1]; j++) deno += W->val[j];
            for (int j = crp[i]; j < crp[i + 1] && rc == 0; j++) {
                double aij = cv[j];
                for (int mm = frp[i]; mm < frp[i + 1]; mm++) {
                    const int m = fci[mm];
                    double amj = 0;
                    for (int l = A->rptr[m]; l < A->rptr[m + 1]; l++)
                        if (A->cind[l] == cci[j]) {
                            amj = A->val[l];
                            break;
                        }
                    int hit = 0;
                    double amk = 0;
                    int mp = A->rptr[m], kp = crp[i];
                    while (mp < A->rptr[m + 1] && kp < crp[i + 1]) {
                        if (A->cind[mp] < cci[kp]) {
                            mp++;
                        } else if (A->cind[mp] == cci[kp]) {
                            amk += A->val[mp];
                            hit = 1;
                            mp++;
                            kp++;
                        } else {
                            kp++;
                        }
                    }
                    if (amk == 0) {
                        if (hit) {
                            (*warn)++;
                            amk = 0.00001;
                        } else {
                            rc = -1;
                            break;
                        }
                    }
                    aij += fv[mm] * amj / amk;
                }
                P->val[q] = -aij / deno;
                P->cind[q++] = col[cci[j]];
            }
        }
        P->rptr[i + 1] = q;
    }
    free(col); free(crp); free(frp); free(cci); free(cv); free(fci); free(fv);
    if (rc) dmat_free(P);
    return rc;
}

/* transpose_interpolation_matrix (helper_multigrid.hpp:534-561) */
static dmat transpose(const dmat *P) {
    const int N = P->n, M = P->m;
    int32_t *num = (int32_t *)xcalloc((size_t)M, sizeof(int32_t));
    for (int i = 0; i < N; i++)
        for (int j = P->rptr[i]; j < P->rptr[i + 1]; j++) num[P->cind[j]]++;
    dmat R = dmat_new(M, N, P->rptr[N]);
    for (int i = 0; i < M; i++) {
        R.rptr[i + 1] = R.rptr[i] + num[i];
        num[i] = 0;
    }
    for (int i = 0; i < N; i++)
        for (int j = P->rptr[i]; j < P->rptr[i + 1]; j++) {
            const int c = P->cind[j];
            const int at = R.rptr[c] + num[c]++;
            R.val[at] = P->val[j];
            R.cind[at] = i;
        }
    free(num);
    return R;
}

static int cmp_i32(const void *a, const void *b) {
    const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return x < y ? -1 : x > y;
}

/* cscSpMM (helper_sparse.hpp:257-285): column i of the result is the sum over
 * the entries (k, alpha) of column i of r, in order, of alpha times column k
 * of l, each merge keeping y + alpha x and dropping exact zeros
 * (helper_sparse.hpp:213-240).  Written with a dense accumulator: every entry
 * receives the same additions in the same order (an entry that cancels to
 * zero and is hit again restarts from alpha x, which is 0 + alpha x), and the
 * exact zeros are dropped at the end; the column keeps its rows ascending. */
static void csc_spmm(const int32_t *lp, const int32_t *li, const double *lv, int L, const int32_t *rp,
                     const int32_t *ri, const double *rv, int R, int32_t **op, int32_t **oi, double **ov) {
    double *acc = (double *)xcalloc((size_t)L, sizeof(double));
    char *on = (char *)xcalloc((size_t)L, 1);
    int32_t *rows = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(L > 0 ? L : 1));
    int32_t *p = (int32_t *)xmalloc(sizeof(int32_t) * ((size_t)R + 1));
    size_t cap = 1024, len = 0;
    int32_t *idx = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    double *val = (double *)xmalloc(sizeof(double) * cap);
    p[0] = 0;
    for (int c = 0; c < R; c++) {
        int nr = 0;
        for (int e = rp[c]; e < rp[c + 1]; e++) {
            const int k = ri[e];
            const double alpha = rv[e];
            for (int t = lp[k]; t < lp[k + 1]; t++) {
                const int row = li[t];
                if (on[row]) {
                    acc[row] = acc[row] + alpha * lv[t];
                } else {
                    on[row] = 1;
                    acc[row] = alpha * lv[t];
                    rows[nr++] = row;
                }
            }
        }
        qsort(rows, (size_t)nr, sizeof(int32_t), cmp_i32);
        for (int t = 0; t < nr; t++) {
            const int row = rows[t];
            if (fabs(acc[row]) != 0.0) {
                if (len == cap) {
                    cap *= 2;
                    idx = (int32_t *)xrealloc(idx, sizeof(int32_t) * cap);
                    val = (double *)xrealloc(val, sizeof(double) * cap);
                }
                idx[len] = row;
                val[len++] = acc[row];
            }
            on[row] = 0;
        }
        p[c + 1] = (int32_t)len;
    }
    free(acc); free(on); free(rows);
    *op = p;
    *oi = idx;
    *ov = val;
}

/* get_coarse_matrix (helper_multigrid.hpp:564-586): C = P^T A P through two
 * CSC products; the CSC result read as CSR */
static dmat coarse_matrix(const dmat *A, const dmat *P, const dmat *R) {
    const int N = P->n, M = P->m;
    int32_t *tp, *ti, *cp, *ci;
    double *tv, *cv;
    csc_spmm(A->rptr, A->cind, A->val, N, R->rptr, R->cind, R->val, M, &tp, &ti, &tv);
    csc_spmm(P->rptr, P->cind, P->val, M, tp, ti, tv, M, &cp, &ci, &cv);
    free(tp); free(ti); free(tv);
    dmat C;
    C.n = C.m = M;
    C.rptr = cp;
    C.cind = ci;
    C.val = cv;
    return C;
}

/* get_amg_set (helper_multigrid.hpp:34-63) */
static int amg_set(const dmat *A, double theta, dmat *CA, dmat *P, dmat *R, long *warn) {
    dmat S, W;
    strong_weak(A, theta, &S, &W);
    int32_t *trp, *tci;
    influence(&S, &trp, &tci);
    int32_t *isc = first_pass(&S, trp, tci);
    int rc = second_pass(&S, isc);
    if (rc == 0) rc = interpolation(A, &S, &W, isc, P, warn);
    if (rc == 0) {
        *R = transpose(P);
        *CA = coarse_matrix(A, P, R);
    }
    dmat_free(&S); dmat_free(&W);
    free(trp); free(tci); free(isc);
    return rc;
}

/* ------------------------------------------------- constructor data */

/* SOR ctor (stationary.hpp:363-400; split "LD-U", helper_matrix.hpp:531-604):
 * LD = strict lower part + diagonal / omega (the diagonal last in its row),
 * U = (1 - 1/omega) diagonal first, then the strict upper part */
static void sor_split(const dmat *A, double omega, dmat *LD, dmat *U) {
    const int N = A->n;
    int64_t nl = 0, nu = 0;
    for (int i = 0; i < N; i++)
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            if (A->cind[j] <= i) nl++;
            else nu++;
        }
    *LD = dmat_new(N, A->m, nl);
    *U = dmat_new(N, A->m, nu + N);
    int l = 0, u = 0;
    for (int i = 0; i < N; i++) {
        const int u0 = u++;  /* the diagonal slot of U */
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            if (A->cind[j] <= i) {
                LD->val[l] = A->val[j];
                LD->cind[l++] = A->cind[j];
            } else {
                U->val[u] = A->val[j];
                U->cind[u++] = A->cind[j];
            }
        }
        const double d = LD->val[l - 1];
        U->val[u0] = (1 - 1.0 / omega) * d;
        U->cind[u0] = LD->cind[l - 1];
        LD->val[l - 1] = 1.0 / omega * d;
        LD->rptr[i + 1] = l;
        U->rptr[i + 1] = u;
    }
}

/* extractLDinv (helper_matrix.hpp:634-664): lower part with 1/diagonal */
static dmat extract_ldinv(const dmat *A) {
    const int N = A->n;
    int64_t nnz = 0;
    for (int i = 0; i < N; i++)
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) nnz += A->cind[j] <= i;
    dmat B = dmat_new(N, A->m, nnz);
    int q = 0;
    for (int i = 0; i < N; i++) {
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            if (A->cind[j] == i) {
                B.val[q] = 1 / A->val[j];
                B.cind[q++] = A->cind[j];
            } else if (A->cind[j] < i) {
                B.val[q] = A->val[j];
                B.cind[q++] = A->cind[j];
            }
        }
        B.rptr[i + 1] = q;
    }
    return B;
}

/* extractL (helper_matrix.hpp:606-632) and extractDinvU (698-728) */
static dmat extract_l(const dmat *A) {
    const int N = A->n;
    int64_t nnz = 0;
    for (int i = 0; i < N; i++)
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) nnz += A->cind[j] < i;
    dmat B = dmat_new(N, A->m, nnz);
    int q = 0;
    for (int i = 0; i < N; i++) {
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++)
            if (A->cind[j] < i) {
                B.val[q] = A->val[j];
                B.cind[q++] = A->cind[j];
            }
        B.rptr[i + 1] = q;
    }
    return B;
}
static dmat extract_dinvu(const dmat *A) {
    const int N = A->n;
    int64_t nnz = 0;
    for (int i = 0; i < N; i++)
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) nnz += A->cind[j] >= i;
    dmat B = dmat_new(N, A->m, nnz);
    int q = 0;
    for (int i = 0; i < N; i++) {
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            if (A->cind[j] == i) {
                B.val[q] = 1 / A->val[j];
                B.cind[q++] = A->cind[j];
            } else if (A->cind[j] > i) {
                B.val[q] = A->val[j];
                B.cind[q++] = A->cind[j];
            }
        }
        B.rptr[i + 1] = q;
    }
    return B;
}

/* helper::matrix::ilu (helper_matrix.hpp:978-1061): exact LU with fill, row by
 * row; each lower entry k of row i (in column order) is replaced by its
 * multiplier a_ik / u_kk and row i is merged with -multiplier times the upper
 * part of row k */
static dmat ilu(const dmat *A) {
    const int N = A->n;
    size_t cap = (size_t)A->rptr[N] + 16, len = 0;
    int32_t *nrp = (int32_t *)xmalloc(sizeof(int32_t) * ((size_t)N + 1));
    int32_t *nci = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    double *nv = (double *)xmalloc(sizeof(double) * cap);
    int32_t *tr = (int32_t *)xmalloc(sizeof(int32_t) * ((size_t)N + 1));
    double *tv = (double *)xmalloc(sizeof(double) * ((size_t)N + 1));
    int32_t *t2r = (int32_t *)xmalloc(sizeof(int32_t) * ((size_t)N + 1));
    double *t2v = (double *)xmalloc(sizeof(double) * ((size_t)N + 1));
    double pivot = 0; /* kept across rows, as the reference's */
    nrp[0] = 0;
    for (int i = 0; i < N; i++) {
        int tl = 0;
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            tr[tl] = A->cind[j];
            tv[tl++] = A->val[j];
        }
        int count = 0;
        while (i > 0 && count < tl && tr[count] < i) {
            const int k = tr[count];
            int kp = count, t2 = 0;
            for (int j = 0; j < count; j++) {
                t2r[t2] = tr[j];
                t2v[t2++] = tv[j];
            }
            int j;
            for (j = nrp[k]; j < nrp[k + 1]; j++)
                if (nci[j] == k) {
                    pivot = tv[kp] / nv[j];
                    break;
                }
            j++;
            kp++;
            t2r[t2] = k;
            t2v[t2++] = pivot;
            while (kp < tl || j < nrp[k + 1]) {
                const int c1 = kp < tl ? tr[kp] : N + 1;
                const int c2 = j < nrp[k + 1] ? nci[j] : N + 1;
                if (c1 < c2) {
                    t2v[t2] = tv[kp];
                    t2r[t2++] = tr[kp++];
                } else if (c1 == c2) {
                    t2v[t2] = tv[kp] - pivot * nv[j];
                    t2r[t2++] = tr[kp++];
                    j++;
                } else {
                    t2v[t2] = -pivot * nv[j];
                    t2r[t2++] = nci[j++];
                }
            }
            count++;
            memcpy(tr, t2r, sizeof(int32_t) * (size_t)t2);
            memcpy(tv, t2v, sizeof(double) * (size_t)t2);
            tl = t2;
        }
        if (len + (size_t)tl > cap) {
            while (len + (size_t)tl > cap) cap *= 2;
            nci = (int32_t *)xrealloc(nci, sizeof(int32_t) * cap);
            nv = (double *)xrealloc(nv, sizeof(double) * cap);
        }
        memcpy(nci + len, tr, sizeof(int32_t) * (size_t)tl);
        memcpy(nv + len, tv, sizeof(double) * (size_t)tl);
        len += (size_t)tl;
        nrp[i + 1] = (int32_t)len;
    }
    free(tr); free(tv); free(t2r); free(t2v);
    dmat F;
    F.n = F.m = N;
    F.rptr = nrp;
    F.cind = nci;
    F.val = nv;
    return F;
}

/* ---------------------------------------------------- conversion rules */

/* CSRflex (spmat.hpp:108): bit = max < 1 ? 30 : 32 - (ceil(log2(int(max)+1)) + 1) */
static int flex_bit(double mx) {
    if (mx < 1) return 30;
    return 32 - ((int)ceil(log2((double)(cvt_i32(mx) + 1))) + 1);
}
/* ltri / dutri::CSRflex (ltri.hpp:106-108, dutri.hpp:120-125): the largest
 * b <= 30 with max 2^b >= 2^30 */
static int while_bit(double mx) {
    int b = 0;
    while (b < 30 && mx * (double)(1 << b) < (double)(1 << 30)) b++;
    return b;
}

static imat quantize(const dmat *A, int bit, int dbit, int split_diag) {
    imat B;
    const int64_t nnz = A->rptr[A->n];
    B.n = A->n;
    B.m = A->m;
    B.bit = bit;
    B.dbit = dbit;
    B.rptr = (int32_t *)xmalloc(sizeof(int32_t) * ((size_t)A->n + 1));
    B.cind = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
    B.val = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnz ? nnz : 1));
    memcpy(B.rptr, A->rptr, sizeof(int32_t) * ((size_t)A->n + 1));
    memcpy(B.cind, A->cind, sizeof(int32_t) * (size_t)nnz);
    for (int i = 0; i < A->n; i++)
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            const int b = split_diag && A->cind[j] == i ? dbit : bit;
            B.val[j] = cvt_i32(A->val[j] * (double)(1 << b));
        }
    return B;
}
static double max_abs(const dmat *A, int which) { /* 0 all, 1 off-diagonal, 2 diagonal */
    double mx = 0;
    for (int i = 0; i < A->n; i++)
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) {
            const int d = A->cind[j] == i;
            if ((which == 1 && d) || (which == 2 && !d)) continue;
            if (fabs(A->val[j]) > mx) mx = fabs(A->val[j]);
        }
    return mx;
}
static imat to_flex(const dmat *A) { return quantize(A, flex_bit(max_abs(A, 0)), 0, 0); }
static imat to_ldtri_flex(const dmat *LDinv) {
    return quantize(LDinv, flex_bit(max_abs(LDinv, 1)), flex_bit(max_abs(LDinv, 2)), 1);
}
static imat to_ltri_flex(const dmat *L) { return quantize(L, while_bit(max_abs(L, 0)), 0, 0); }
static imat to_dutri_flex(const dmat *DU) {
    return quantize(DU, while_bit(max_abs(DU, 1)), while_bit(max_abs(DU, 2)), 1);
}

/* ------------------------------------------------------------ the setup */

struct or_setup {
    int depth;
    long warnings;
    /* integer hierarchy (intAMGflex) */
    imat A0, *CA, *P, *R, *LD, *U, LUL, LUU;
    or_csr_i32 *vCA, *vP, *vR, *vLD, *vU;
    /* FP64 hierarchy (dfAMG) */
    dmat dA0, *dCA, *dP, *dR, *dLD, *dU, dLUL, dLUU;
    or_csr_f64 *wCA, *wP, *wR, *wLD, *wU;
};

static or_csr_i32 iview(const imat *A) {
    or_csr_i32 v = {A->n, A->m, A->rptr, A->cind, A->val, A->bit, A->dbit};
    return v;
}
static or_csr_f64 dview(const dmat *A) {
    or_csr_f64 v = {A->n, A->m, A->rptr, A->cind, A->val};
    return v;
}

or_setup *or_setup_create(int n, const int32_t *rptr, const int32_t *cind, const double *val, double theta,
                          int max_levels, int coarse_limit, double omega, int *status) {
    *status = 0;
    if (n < 1 || !(theta > 0 && theta <= 1) || max_levels < 1) {
        *status = -2;
        return NULL;
    }
    dmat A;
    A.n = A.m = n;
    A.rptr = (int32_t *)rptr;
    A.cind = (int32_t *)cind;
    A.val = (double *)val;
    /* the level loop (INTAMG.hpp:38-51 and 162-195): CA[0] from A, then
     * while max_levels > depth and the last CA has more than coarse_limit rows */
    int cap = 4, D = 0;
    dmat *CA = (dmat *)xmalloc(sizeof(dmat) * (size_t)cap);
    dmat *P = (dmat *)xmalloc(sizeof(dmat) * (size_t)cap);
    dmat *R = (dmat *)xmalloc(sizeof(dmat) * (size_t)cap);
    long warn = 0;
    int rc = amg_set(&A, theta, &CA[0], &P[0], &R[0], &warn);
    if (rc == 0) D = 1;
    while (rc == 0 && max_levels > D && CA[D - 1].n > coarse_limit) {
        if (D == cap) {
            cap *= 2;
            CA = (dmat *)xrealloc(CA, sizeof(dmat) * (size_t)cap);
            P = (dmat *)xrealloc(P, sizeof(dmat) * (size_t)cap);
            R = (dmat *)xrealloc(R, sizeof(dmat) * (size_t)cap);
        }
        rc = amg_set(&CA[D - 1], theta, &CA[D], &P[D], &R[D], &warn);
        if (rc == 0) D++;
    }
    if (rc != 0) {
        for (int i = 0; i < D; i++) {
            dmat_free(&CA[i]); dmat_free(&P[i]); dmat_free(&R[i]);
        }
        free(CA); free(P); free(R);
        *status = rc;
        return NULL;
    }
    or_setup *s = (or_setup *)xcalloc(1, sizeof(or_setup));
    s->depth = D;
    s->warnings = warn;
    /* ---- dfAMG (INTAMG.hpp:57-73): unscaled operators; SOR<ldtri::CSR<double>>
     * holds extractLDinv of LD; LU<double> holds extractL / extractDinvU of ilu */
    s->dA0 = dmat_copy(&A);
    s->dCA = (dmat *)xcalloc((size_t)D, sizeof(dmat));
    s->dP = (dmat *)xcalloc((size_t)D, sizeof(dmat));
    s->dR = (dmat *)xcalloc((size_t)D, sizeof(dmat));
    s->dLD = (dmat *)xcalloc((size_t)D, sizeof(dmat));
    s->dU = (dmat *)xcalloc((size_t)D, sizeof(dmat));
    for (int l = 0; l < D; l++) {
        const dmat *Al = l == 0 ? &A : &CA[l - 1];
        dmat LD, U;
        sor_split(Al, omega, &LD, &U);
        s->dLD[l] = extract_ldinv(&LD);
        s->dU[l] = U;
        dmat_free(&LD);
        if (l < D - 1) s->dCA[l] = dmat_copy(&CA[l]);
        s->dP[l] = dmat_copy(&P[l]);
        s->dR[l] = dmat_copy(&R[l]);
    }
    {
        dmat F = ilu(&CA[D - 1]);
        s->dLUL = extract_l(&F);
        s->dLUU = extract_dinvu(&F);
        dmat_free(&F);
    }
    /* ---- intAMGflex (INTAMG.hpp:174-211): coarse operators and the
     * restrictions scaled by the coarse rows' maxima (prev: the level above's) */
    double *prev = (double *)xcalloc((size_t)n, sizeof(double));
    for (int l = 0; l < D; l++) {
        double *mx = (double *)xcalloc((size_t)CA[l].n, sizeof(double));
        for (int i = 0; i < CA[l].n; i++) {
            for (int j = CA[l].rptr[i]; j < CA[l].rptr[i + 1]; j++)
                if (fabs(CA[l].val[j]) > mx[i]) mx[i] = fabs(CA[l].val[j]);
            for (int j = CA[l].rptr[i]; j < CA[l].rptr[i + 1]; j++) CA[l].val[j] /= mx[i];
            for (int j = R[l].rptr[i]; j < R[l].rptr[i + 1]; j++) R[l].val[j] /= mx[i];
            /* in the loop, the first restriction keeps its own scale (INTAMG.hpp:190);
             * the last level always multiplies by prev (INTAMG.hpp:208-210) */
            if (l == 0 && l < D - 1) continue;
            for (int j = R[l].rptr[i]; j < R[l].rptr[i + 1]; j++) R[l].val[j] *= prev[R[l].cind[j]];
        }
        for (int i = 0; i < CA[l].n; i++) prev[i] = mx[i];
        free(mx);
    }
    free(prev);
    s->A0 = quantize(&A, 30, 0, 0); /* CSR<Fixed<30>> (spmat.hpp:62-70, array.hpp:43-49) */
    s->CA = (imat *)xcalloc((size_t)D, sizeof(imat));
    s->P = (imat *)xcalloc((size_t)D, sizeof(imat));
    s->R = (imat *)xcalloc((size_t)D, sizeof(imat));
    s->LD = (imat *)xcalloc((size_t)D, sizeof(imat));
    s->U = (imat *)xcalloc((size_t)D, sizeof(imat));
    for (int l = 0; l < D; l++) {
        const dmat *Al = l == 0 ? &A : &CA[l - 1];
        dmat LD, U;
        sor_split(Al, omega, &LD, &U); /* SOR<ldtri::CSRflex, CSRflex> (stationary.hpp:363-400) */
        dmat LDinv = extract_ldinv(&LD);
        s->LD[l] = to_ldtri_flex(&LDinv); /* ldtri.hpp:127-160 */
        s->U[l] = to_flex(&U);
        dmat_free(&LDinv); dmat_free(&LD); dmat_free(&U);
        if (l < D - 1) s->CA[l] = to_flex(&CA[l]);
        s->P[l] = to_flex(&P[l]);
        s->R[l] = to_flex(&R[l]);
    }
    {
        dmat F = ilu(&CA[D - 1]); /* LUflex (lu.hpp:71-95) on the scaled coarsest operator */
        dmat L = extract_l(&F), DU = extract_dinvu(&F);
        s->LUL = to_ltri_flex(&L);
        s->LUU = to_dutri_flex(&DU);
        dmat_free(&F); dmat_free(&L); dmat_free(&DU);
    }
    for (int i = 0; i < D; i++) {
        dmat_free(&CA[i]); dmat_free(&P[i]); dmat_free(&R[i]);
    }
    free(CA); free(P); free(R);
    /* views for the oracle's hierarchy structs */
    s->vCA = (or_csr_i32 *)xcalloc((size_t)D, sizeof(or_csr_i32));
    s->vP = (or_csr_i32 *)xcalloc((size_t)D, sizeof(or_csr_i32));
    s->vR = (or_csr_i32 *)xcalloc((size_t)D, sizeof(or_csr_i32));
    s->vLD = (or_csr_i32 *)xcalloc((size_t)D, sizeof(or_csr_i32));
    s->vU = (or_csr_i32 *)xcalloc((size_t)D, sizeof(or_csr_i32));
    s->wCA = (or_csr_f64 *)xcalloc((size_t)D, sizeof(or_csr_f64));
    s->wP = (or_csr_f64 *)xcalloc((size_t)D, sizeof(or_csr_f64));
    s->wR = (or_csr_f64 *)xcalloc((size_t)D, sizeof(or_csr_f64));
    s->wLD = (or_csr_f64 *)xcalloc((size_t)D, sizeof(or_csr_f64));
    s->wU = (or_csr_f64 *)xcalloc((size_t)D, sizeof(or_csr_f64));
    for (int l = 0; l < D; l++) {
        if (l < D - 1) {
            s->vCA[l] = iview(&s->CA[l]);
            s->wCA[l] = dview(&s->dCA[l]);
        }
        s->vP[l] = iview(&s->P[l]);
        s->vR[l] = iview(&s->R[l]);
        s->vLD[l] = iview(&s->LD[l]);
        s->vU[l] = iview(&s->U[l]);
        s->wP[l] = dview(&s->dP[l]);
        s->wR[l] = dview(&s->dR[l]);
        s->wLD[l] = dview(&s->dLD[l]);
        s->wU[l] = dview(&s->dU[l]);
    }
    return s;
}

int or_setup_depth(const or_setup *s) { return s->depth; }
long or_setup_warnings(const or_setup *s) { return s->warnings; }

void or_setup_amg_i32(const or_setup *s, or_amg_i32 *h) {
    memset(h, 0, sizeof(*h));
    h->depth = s->depth;
    h->A0 = iview(&s->A0);
    h->CA = s->vCA;
    h->P = s->vP;
    h->R = s->vR;
    h->LD = s->vLD;
    h->U = s->vU;
    h->smooth_iter = 1;
    h->LUL = iview(&s->LUL);
    h->LUU = iview(&s->LUU);
}

void or_setup_amg_f64(const or_setup *s, or_amg_f64 *h) {
    memset(h, 0, sizeof(*h));
    h->depth = s->depth;
    h->A0 = dview(&s->dA0);
    h->CA = s->wCA;
    h->P = s->wP;
    h->R = s->wR;
    h->LD = s->wLD;
    h->U = s->wU;
    h->smooth_iter = 1;
    h->LUL = dview(&s->dLUL);
    h->LUU = dview(&s->dLUU);
}

void or_setup_destroy(or_setup *s) {
    if (!s) return;
    const int D = s->depth;
    imat_free(&s->A0);
    imat_free(&s->LUL);
    imat_free(&s->LUU);
    dmat_free(&s->dA0);
    dmat_free(&s->dLUL);
    dmat_free(&s->dLUU);
    for (int l = 0; l < D; l++) {
        if (l < D - 1) {
            imat_free(&s->CA[l]);
            dmat_free(&s->dCA[l]);
        }
        imat_free(&s->P[l]); imat_free(&s->R[l]); imat_free(&s->LD[l]); imat_free(&s->U[l]);
        dmat_free(&s->dP[l]); dmat_free(&s->dR[l]); dmat_free(&s->dLD[l]); dmat_free(&s->dU[l]);
    }
    free(s->CA); free(s->P); free(s->R); free(s->LD); free(s->U);
    free(s->dCA); free(s->dP); free(s->dR); free(s->dLD); free(s->dU);
    free(s->vCA); free(s->vP); free(s->vR); free(s->vLD); free(s->vU);
    free(s->wCA); free(s->wP); free(s->wR); free(s->wLD); free(s->wU);
    free(s);
}
