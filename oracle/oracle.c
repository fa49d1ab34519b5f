/* CPU restatement of the reference solve phase.  TEST INFRASTRUCTURE ONLY.
 * See oracle.h for the contract.  Reference paths are relative to the
 * suzuki-hpc/SC23-AD tree (Library/...).
 */
#include "oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

void or_set_threads(int nthreads) { g_threads = nthreads > 0 ? nthreads : 1; }
int or_get_threads(void) { return g_threads; }

/* two's-complement helpers (the reference relies on g++'s wrap behaviour) */
static inline int32_t lo32(int64_t v) { return (int32_t)(uint32_t)(uint64_t)v; }
static inline int64_t wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
static inline int64_t wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
static inline int64_t wmul(int64_t a, int64_t b) { return (int64_t)((uint64_t)a * (uint64_t)b); }
static inline int64_t wshl(int64_t a, int s) { return (int64_t)((uint64_t)a << s); }
static inline int32_t add32(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t sub32(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
/* (int)(double) as compiled by g++ on x86-64 (cvttsd2si): truncation toward
 * zero, 0x80000000 when out of range or NaN. */
static inline int32_t d2i(double v) {
    if (!(v > -2147483649.0 && v < 2147483648.0)) return INT32_MIN;
    return (int32_t)v;
}
static inline int64_t d2l(double v) {
    if (!(v > -9223372036854775808.0 && v < 9223372036854775808.0)) return INT64_MIN;
    return (int64_t)v;
}

/* ===================================================================== int */

/* CSRflex::SpMV / CSR<Fixed<bit>>::SpMV (matrix/spmat.hpp:128-137, 77-86):
 * out_i = (int)((sum_j (long)val_j * (long)in_cj) >> bit). */
int or_spmv_i32(const or_csr_i32 *A, const int32_t *in, int32_t *out) {
    const int n = A->n, bit = A->bit;
    int ovf = 0;
#pragma omp parallel for num_threads(g_threads) reduction(| : ovf) schedule(static)
    for (int i = 0; i < n; i++) {
        int64_t t = 0;
        for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) t = wadd(t, (int64_t)A->val[j] * (int64_t)in[A->cind[j]]);
        int64_t s = t >> bit;
        out[i] = lo32(s);
        ovf |= (s != (int64_t)lo32(s));
    }
    return ovf;
}

/* ldtri::CSRflex::SpTRSV (matrix/trimat/ldtri.hpp:172-183): forward Gauss-Seidel
 * row with the inverse diagonal stored last in the row.  With bj != NULL the
 * same sweep runs inside each block independently (BJCSRflex, ldtri.hpp:511-525). */
static int ldtri_row(const or_csr_i32 *LD, int i, const int32_t *in, int32_t *out) {
    const int bit = LD->bit, dbit = LD->dbit;
    int64_t t = wshl((int64_t)in[i], bit);
    int j;
    for (j = LD->rptr[i]; j < LD->rptr[i + 1] - 1; j++) t = wsub(t, (int64_t)LD->val[j] * (int64_t)out[LD->cind[j]]);
    int64_t s = wmul(t >> bit, (int64_t)LD->val[j]) >> dbit;
    out[i] = lo32(s);
    return s != (int64_t)lo32(s);
}

static int ldtri_rows(const or_csr_i32 *LD, int r0, int r1, const int32_t *in, int32_t *out) {
    int ovf = 0;
    for (int i = r0; i < r1; i++) ovf |= ldtri_row(LD, i, in, out);
    return ovf;
}

int or_ldtri_order_i32(const or_csr_i32 *LD, const int32_t *order, const int32_t *in, int32_t *out) {
    int ovf = 0;
    for (int k = 0; k < LD->n; k++) ovf |= ldtri_row(LD, order[k], in, out);
    return ovf;
}

int or_ldtri_i32(const or_csr_i32 *LD, const int32_t *bj, int nbj, const int32_t *in, int32_t *out) {
    if (!bj) return ldtri_rows(LD, 0, LD->n, in, out);
    int ovf = 0;
#pragma omp parallel for num_threads(g_threads) reduction(| : ovf) schedule(static, 1)
    for (int b = 0; b < nbj; b++) ovf |= ldtri_rows(LD, bj[b], bj[b + 1], in, out);
    return ovf;
}

/* ltri::CSRflex::SpTRSV (matrix/trimat/ltri.hpp:125-133): unit lower solve. */
int or_ltri_i32(const or_csr_i32 *L, const int32_t *in, int32_t *out) {
    const int bit = L->bit;
    int ovf = 0;
    for (int i = 0; i < L->n; i++) {
        int64_t t = wshl((int64_t)in[i], bit);
        for (int j = L->rptr[i]; j < L->rptr[i + 1]; j++) t = wsub(t, (int64_t)L->val[j] * (int64_t)out[L->cind[j]]);
        int64_t s = t >> bit;
        out[i] = lo32(s);
        ovf |= (s != (int64_t)lo32(s));
    }
    return ovf;
}

/* dutri::CSRflex::SpTRSV (matrix/trimat/dutri.hpp:146-156): backward solve with
 * the inverse diagonal first in each row. */
int or_dutri_i32(const or_csr_i32 *U, const int32_t *in, int32_t *out) {
    const int bit = U->bit, dbit = U->dbit;
    int ovf = 0;
    for (int i = U->n - 1; i >= 0; i--) {
        int64_t t = wshl((int64_t)in[i], bit);
        int j;
        for (j = U->rptr[i + 1] - 1; j >= U->rptr[i] + 1; j--) t = wsub(t, (int64_t)U->val[j] * (int64_t)out[U->cind[j]]);
        int64_t s = wmul(t >> bit, (int64_t)U->val[j]) >> dbit;
        out[i] = lo32(s);
        ovf |= (s != (int64_t)lo32(s));
    }
    return ovf;
}

/* blas1::int32::lsqrt (blas/blas1.hpp:107-119): integer Newton square root. */
int64_t or_lsqrt(int64_t x) {
    int64_t s, t;
    if (x <= 0) return 0;
    s = 1;
    t = x;
    while (s < t) { s <<= 1; t >>= 1; }
    do {
        t = s;
        s = (x / s + s) >> 1;
    } while (s < t);
    return t;
}

/* blas1::int32::Dot (blas1.hpp:274-281) */
int64_t or_dot_i32(const int32_t *x, const int32_t *y, int n, int bit) {
    uint64_t res = 0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : res) schedule(static)
    for (int i = 0; i < n; i++) res += (uint64_t)((int64_t)x[i] * (int64_t)y[i]);
    return ((int64_t)res) >> bit;
}

/* blas1::int32::Nrm2 (blas1.hpp:283-290): lsqrt of the int64 sum of squares. */
int64_t or_nrm2_i32(const int32_t *x, int n) {
    uint64_t res = 0;
#pragma omp parallel for num_threads(g_threads) reduction(+ : res) schedule(static)
    for (int i = 0; i < n; i++) res += (uint64_t)((int64_t)x[i] * (int64_t)x[i]);
    return or_lsqrt((int64_t)res);
}

/* blas1::int32::Axpy (blas1.hpp:245-250): y += (int)(a*x >> bit) */
void or_axpy_i32(int64_t a, const int32_t *x, int32_t *y, int n, int bit) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < n; i++) y[i] = add32(y[i], lo32(wmul(a, (int64_t)x[i]) >> bit));
}

/* blas1::int32::Scal (blas1.hpp:230-235): x = (int)(a*x >> bit) */
void or_scal_i32(int64_t a, int32_t *x, int n, int bit) {
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < n; i++) x[i] = lo32(wmul(a, (int64_t)x[i]) >> bit);
}

/* blas1::int32::Axpy_D (blas1.hpp:252-258): y += a * (double)x * 2^-bit */
void or_axpy_d(double a, const int32_t *x, double *y, int n, int bit) {
    const double fact_inv = 1.0 / (double)((int64_t)1 << bit);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < n; i++) y[i] += a * (double)x[i] * fact_inv;
}

/* blas1::int32::Ggen (blas1.hpp:292-300) */
int64_t or_ggen_i32(int64_t a, int64_t b, int64_t *c, int64_t *s, int bit) {
    int64_t r = wadd(wmul(a, a), wmul(b, b));
    r = or_lsqrt(r);
    int64_t inv_r = (r == 0 ? 0 : (((int64_t)1 << 62) / r)) >> (62 - bit - bit);
    *c = wmul(a, inv_r) >> bit;
    *s = wsub(0, wmul(b, inv_r)) >> bit; /* -(b*inv_r) >> bit: negation binds first */
    return r;
}

/* blas1::int32::Grot (blas1.hpp:302-307) */
void or_grot_i32(int64_t c, int64_t s, int64_t *a, int64_t *b, int bit) {
    int64_t t = *a;
    *a = wsub(wmul(c, t), wmul(s, *b)) >> bit;
    *b = wadd(wmul(s, t), wmul(c, *b)) >> bit;
}

/* blas2::int32::Trsv (blas/blas2.hpp:366-376): FP64 back solve of the int64
 * Hessenberg factor; ld = m+1 is the column stride of H. */
void or_trsv_i32(const int64_t *H, double e0, const int64_t *e, double *y, int ld, int m, int bit) {
    const double fact = (double)((int64_t)1 << bit);
    for (int i = m - 1; i >= 0; i--) {
        double t = e0 * (double)e[i] / fact;
        for (int j = m - 1; j > i; j--) t -= (double)H[j * ld + i] / fact * y[j];
        y[i] = t / ((double)H[i * ld + i] / fact);
    }
}

/* SOR<ldtri::CSRflex,CSRflex>::Smooth / BlockSORflex::Smooth
 * (smoother/stationary.hpp:415-430, 997-1012):
 *   isInited: repeat iter times { tmp = in - U*out; out = LD^-1 tmp }
 *   else:     out = LD^-1 in; repeat iter-1 times { ... } */
static void sweep_i32(const or_amg_i32 *h, int l, const int32_t *in, int32_t *out) {
    const int32_t *order = h->order ? h->order[l] : NULL;
    if (order) or_ldtri_order_i32(&h->LD[l], order, in, out);
    else or_ldtri_i32(&h->LD[l], h->bj ? h->bj[l] : NULL, h->nbj, in, out);
}

void or_smooth_i32(const or_amg_i32 *h, int l, const int32_t *in, int32_t *out, int inited) {
    const or_csr_i32 *U = &h->U[l];
    const int n = h->LD[l].n;
    int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int k0 = 0;
    if (!inited) {
        sweep_i32(h, l, in, out);
        k0 = 1;
    }
    for (int k = k0; k < h->smooth_iter; k++) {
        or_spmv_i32(U, out, tmp);
#pragma omp parallel for num_threads(g_threads) schedule(static)
        for (int i = 0; i < n; i++) tmp[i] = sub32(in[i], tmp[i]); /* Axpby<int>(1,in,-1,tmp) */
        sweep_i32(h, l, tmp, out);
    }
    free(tmp);
}

/* direct::LUflex::Solve (solver/lu.hpp:91-94) */
void or_lu_i32(const or_amg_i32 *h, const int32_t *in, int32_t *out) {
    int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)h->LUL.n);
    or_ltri_i32(&h->LUL, in, tmp);
    or_dutri_i32(&h->LUU, tmp, out);
    free(tmp);
}

static void vsub32(const int32_t *x, int32_t *y, int n) { /* blas1::Sub (blas1.hpp:41-44) */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < n; i++) y[i] = sub32(x[i], y[i]);
}
static void vadd32(const int32_t *x, int32_t *y, int n) { /* blas1::Add (blas1.hpp:47-50) */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < n; i++) y[i] = add32(x[i], y[i]);
}

/* intAMGflex::Precondition (preconditioner/INTAMG.hpp:269-293): one V-cycle. */
void or_vcycle_i32(const or_amg_i32 *h, const int32_t *in, int32_t *out) {
    const int D = h->depth, N = h->A0.n;
    int32_t *r = (int32_t *)malloc(sizeof(int32_t) * (size_t)N);
    int32_t **rr = (int32_t **)malloc(sizeof(int32_t *) * (size_t)D);
    int32_t **ee = (int32_t **)malloc(sizeof(int32_t *) * (size_t)D);
    int32_t **xx = (int32_t **)malloc(sizeof(int32_t *) * (size_t)D);
    for (int i = 0; i < D; i++) {
        int len = h->R[i].n;
        rr[i] = (int32_t *)calloc((size_t)len, sizeof(int32_t));
        ee[i] = (int32_t *)calloc((size_t)len, sizeof(int32_t));
        xx[i] = (int32_t *)calloc((size_t)len, sizeof(int32_t));
    }
    or_smooth_i32(h, 0, in, out, 0);
    or_spmv_i32(&h->A0, out, r);
    vsub32(in, r, N);
    or_spmv_i32(&h->R[0], r, ee[0]);
    for (int i = 0; i < D - 1; i++) {
        or_smooth_i32(h, i + 1, ee[i], xx[i], 0);
        or_spmv_i32(&h->CA[i], xx[i], rr[i]);
        vsub32(ee[i], rr[i], h->CA[i].n);
        or_spmv_i32(&h->R[i + 1], rr[i], ee[i + 1]);
    }
    or_lu_i32(h, ee[D - 1], xx[D - 1]);
    for (int i = D - 2; i >= 0; i--) {
        or_spmv_i32(&h->P[i + 1], xx[i + 1], rr[i]);
        vadd32(rr[i], xx[i], h->CA[i].n);
        or_smooth_i32(h, i + 1, ee[i], xx[i], 1);
    }
    or_spmv_i32(&h->P[0], xx[0], r);
    vadd32(r, out, N);
    or_smooth_i32(h, 0, in, out, 1);
    for (int i = 0; i < D; i++) { free(rr[i]); free(ee[i]); free(xx[i]); }
    free(rr); free(ee); free(xx); free(r);
}

double or_nrm2_f64(const double *x, int n) { /* blas1::Nrm2<double> (blas1.hpp:63-68), sequential */
    double s = 0;
    for (int i = 0; i < n; i++) s += x[i] * x[i];
    return sqrt(s);
}

/* FGMRESflex::Solve (solver/gmres.hpp:307-353). */
/* early restart of the batched engine (0: off, the reference's FGMRESflex) */
static int g_cycle_bits = 0;
void or_set_cycle_bits(int bits) { g_cycle_bits = bits; }
static int64_t cycle_target(int bit) { return bit > g_cycle_bits ? (int64_t)1 << (bit - g_cycle_bits) : 1; }

int or_fgmres_i32_cycle(const or_csr_i32 *A, const or_amg_i32 *M, int m, double eps, int bit,
                        const double *r, double nrm_b, double *x,
                        int32_t *V, int32_t *Z, int64_t *H, int64_t *c, int64_t *s, int64_t *e,
                        double *y, const double *e0_in, int *converged, int print) {
    const int N = A->n;
    const double fact = (double)((int64_t)1 << bit);
    const size_t NN = (size_t)N;
    double e0 = e0_in ? *e0_in : or_nrm2_f64(r, N);
    double e_inv = 1.0 / e0;
    int64_t criteria = d2l(nrm_b * eps * e_inv * fact);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int k = 0; k < N; k++) V[k] = d2i(r[k] * e_inv * fact);
    e[0] = (int64_t)1 << bit;
    int flag = 0, j;
    for (j = 0; j < m; j++) {
        int32_t *vj = V + (size_t)j * NN, *zj = Z + (size_t)j * NN, *w = V + (size_t)(j + 1) * NN;
        or_vcycle_i32(M, vj, zj);
        or_spmv_i32(A, zj, w);
        int64_t *Hj = H + (size_t)j * (m + 1);
        for (int k = 0; k <= j; k++) {
            Hj[k] = or_dot_i32(V + (size_t)k * NN, w, N, bit);
            or_axpy_i32(-Hj[k], V + (size_t)k * NN, w, N, bit);
        }
        Hj[j + 1] = or_nrm2_i32(w, N);
        int64_t hinv = (Hj[j + 1] == 0 ? 0 : (((int64_t)1 << 62) / Hj[j + 1])) >> (62 - bit - bit);
        or_scal_i32(hinv, w, N, bit);
        for (int k = 0; k < j; k++) or_grot_i32(c[k], s[k], &Hj[k], &Hj[k + 1], bit);
        Hj[j] = or_ggen_i32(Hj[j], Hj[j + 1], &c[j], &s[j], bit);
        Hj[j + 1] = 0;
        e[j + 1] = wmul(s[j], e[j]) >> bit;
        e[j] = wmul(c[j], e[j]) >> bit;
        if (print) printf("# [%d] %e\n", j + 1, fabs(e0 * (double)e[j + 1] / fact) / nrm_b);
        if ((e[j + 1] < 0 ? -e[j + 1] : e[j + 1]) <= criteria) {
            if (print) printf("[Res] : %e\n", fabs(e0 * (double)e[j + 1] / fact) / nrm_b);
            j++;
            flag = 1;
            break;
        }
        /* the batched engine's early restart (no counterpart in the
         * reference): the cycle ends once the estimate has fallen 2^K below
         * its start e[0] = 2^bit, where the fixed-point basis stops gaining */
        if (g_cycle_bits > 0 && (e[j + 1] < 0 ? -e[j + 1] : e[j + 1]) <= cycle_target(bit)) {
            j++;
            *converged = 0;
            or_trsv_i32(H, e0, e, y, m + 1, j, bit);
            for (int k = 0; k < j; k++) or_axpy_d(y[k], Z + (size_t)k * NN, x, N, bit);
            return j;
        }
    }
    or_trsv_i32(H, e0, e, y, m + 1, j, bit);
    for (int k = 0; k < j; k++) or_axpy_d(y[k], Z + (size_t)k * NN, x, N, bit);
    *converged = flag;
    return flag ? j : m;
}

static void axpby_sub_f64(const double *b, double *r, int n) { /* Axpby<double>(1,b,-1,r) */
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int i = 0; i < n; i++) r[i] = 1.0 * b[i] + (-1.0) * r[i];
}

/* Restarted::Solve (solver/irsolver.hpp:61-77) around FGMRESflex. */
int or_ir_solve_i32(const or_csr_f64 *dA, const or_csr_i32 *A, const or_amg_i32 *M, int m, double eps,
                    int bit, const double *b, double nrm_b, double *x, int max_outer, int print) {
    const int N = A->n;
    const size_t NN = (size_t)N;
    double *r = (double *)malloc(sizeof(double) * NN);
    int32_t *V = (int32_t *)malloc(sizeof(int32_t) * NN * (size_t)(m + 1));
    int32_t *Z = (int32_t *)malloc(sizeof(int32_t) * NN * (size_t)(m + 1));
    int64_t *H = (int64_t *)calloc((size_t)(m + 1) * (size_t)m, sizeof(int64_t));
    int64_t *c = (int64_t *)calloc((size_t)m, sizeof(int64_t));
    int64_t *s = (int64_t *)calloc((size_t)m, sizeof(int64_t));
    int64_t *e = (int64_t *)calloc((size_t)m + 1, sizeof(int64_t));
    double *y = (double *)calloc((size_t)m, sizeof(double));
    double prev = 0;
    int iter = 0, result = 0;
    for (int i = 0; i < max_outer; i++) {
        or_spmv_f64(dA, x, r);
        axpby_sub_f64(b, r, N);
        double nrm_r = or_nrm2_f64(r, N);
        if (fabs(nrm_r - prev) / nrm_r < 1.0e-8) break;
        prev = nrm_r;
        int conv = 0;
        iter += or_fgmres_i32_cycle(A, M, m, eps, bit, r, nrm_b, x, V, Z, H, c, s, e, y, NULL, &conv, print);
        if (conv) { result = iter; break; }
    }
    free(r); free(V); free(Z); free(H); free(c); free(s); free(e); free(y);
    return result;
}

int or_ir_solve_i32x(const or_csr_f64 *dA, const or_csr_i32 *A, const or_amg_i32 *M, int m, double eps,
                     int bit, const double *b, double nrm_b, double *x, int max_outer, int explicit_stop,
                     double *res_out) {
    const int N = A->n;
    const size_t NN = (size_t)N;
    double *r = (double *)malloc(sizeof(double) * NN);
    int32_t *V = (int32_t *)malloc(sizeof(int32_t) * NN * (size_t)(m + 1));
    int32_t *Z = (int32_t *)malloc(sizeof(int32_t) * NN * (size_t)(m + 1));
    int64_t *H = (int64_t *)calloc((size_t)(m + 1) * (size_t)m, sizeof(int64_t));
    int64_t *c = (int64_t *)calloc((size_t)m, sizeof(int64_t));
    int64_t *s = (int64_t *)calloc((size_t)m, sizeof(int64_t));
    int64_t *e = (int64_t *)calloc((size_t)m + 1, sizeof(int64_t));
    double *y = (double *)calloc((size_t)m, sizeof(double));
    double prev = 0, nrm_r = 0;
    int iter = 0, result = 0, done = 0;
    for (int i = 0; i < max_outer && !done; i++) {
        or_spmv_f64(dA, x, r); /* irsolver.hpp:66-68 */
        axpby_sub_f64(b, r, N);
        nrm_r = or_nrm2_f64(r, N);
        if (explicit_stop && i > 0 && nrm_r <= eps * nrm_b) {
            result = iter;
            done = 1;
            break;
        }
        if (fabs(nrm_r - prev) / nrm_r < 1.0e-8) break;
        prev = nrm_r;
        int conv = 0;
        iter += or_fgmres_i32_cycle(A, M, m, eps, bit, r, nrm_b, x, V, Z, H, c, s, e, y, NULL, &conv, 0);
        if (conv && !explicit_stop) {
            result = iter;
            done = 1;
        }
    }
    or_spmv_f64(dA, x, r);
    axpby_sub_f64(b, r, N);
    nrm_r = or_nrm2_f64(r, N);
    if (explicit_stop && !done && nrm_r <= eps * nrm_b) result = iter;
    if (res_out) *res_out = nrm_r / nrm_b;
    free(r); free(V); free(Z); free(H); free(c); free(s); free(e); free(y);
    return result;
}

/* ====================================================== FP64 / FP32 siblings
 * One body per precision, instantiated by macro.  T is the vector type. */

#define DEFINE_FP(SFX, T)                                                                          \
    /* CSR<T>::SpMV (matrix/spmat.hpp:43-52) */                                                   \
    int or_spmv_##SFX(const or_csr_##SFX *A, const T *in, T *out) {                              \
        _Pragma("omp parallel for num_threads(g_threads) schedule(static)")                        \
        for (int i = 0; i < A->n; i++) {                                                            \
            T t = 0;                                                                                \
            for (int j = A->rptr[i]; j < A->rptr[i + 1]; j++) t += A->val[j] * in[A->cind[j]];      \
            out[i] = t;                                                                             \
        }                                                                                           \
        return 0;                                                                                   \
    }                                                                                               \
    /* ldtri::CSR<T>::SpTRSV (ldtri.hpp:49-58); BJCSR<T> (ldtri.hpp:398-412) */                  \
    static void ldtri_row_##SFX(const or_csr_##SFX *LD, int i, const T *in, T *out) {             \
        T t = in[i];                                                                                \
        int j;                                                                                      \
        for (j = LD->rptr[i]; j < LD->rptr[i + 1] - 1; j++) t -= LD->val[j] * out[LD->cind[j]];     \
        out[i] = t * LD->val[j];                                                                    \
    }                                                                                               \
    static void ldtri_rows_##SFX(const or_csr_##SFX *LD, int r0, int r1, const T *in, T *out) {   \
        for (int i = r0; i < r1; i++) ldtri_row_##SFX(LD, i, in, out);                              \
    }                                                                                               \
    int or_ldtri_order_##SFX(const or_csr_##SFX *LD, const int32_t *order, const T *in, T *out) { \
        for (int k = 0; k < LD->n; k++) ldtri_row_##SFX(LD, order[k], in, out);                     \
        return 0;                                                                                   \
    }                                                                                               \
    int or_ldtri_##SFX(const or_csr_##SFX *LD, const int32_t *bj, int nbj, const T *in, T *out) { \
        if (!bj) { ldtri_rows_##SFX(LD, 0, LD->n, in, out); return 0; }                             \
        _Pragma("omp parallel for num_threads(g_threads) schedule(static, 1)")                     \
        for (int b = 0; b < nbj; b++) ldtri_rows_##SFX(LD, bj[b], bj[b + 1], in, out);              \
        return 0;                                                                                   \
    }                                                                                               \
    /* ltri::CSR<T>::SpTRSV (ltri.hpp:45-53) */                                                   \
    int or_ltri_##SFX(const or_csr_##SFX *L, const T *in, T *out) {                               \
        for (int i = 0; i < L->n; i++) {                                                            \
            T t = in[i];                                                                            \
            for (int j = L->rptr[i]; j < L->rptr[i + 1]; j++) t -= L->val[j] * out[L->cind[j]];     \
            out[i] = t;                                                                             \
        }                                                                                           \
        return 0;                                                                                   \
    }                                                                                               \
    /* dutri::CSR<T>::SpTRSV (dutri.hpp:45-54) */                                                 \
    int or_dutri_##SFX(const or_csr_##SFX *U, const T *in, T *out) {                              \
        for (int i = U->n - 1; i >= 0; i--) {                                                       \
            T t = in[i];                                                                            \
            int j;                                                                                  \
            for (j = U->rptr[i + 1] - 1; j >= U->rptr[i] + 1; j--) t -= U->val[j] * out[U->cind[j]]; \
            out[i] = t * U->val[j];                                                                 \
        }                                                                                           \
        return 0;                                                                                   \
    }                                                                                               \
    /* SOR<ClassLD<T>,ClassU<T>>::Smooth (stationary.hpp:238-255) */                              \
    static void sweep_##SFX(const or_amg_##SFX *h, int l, const T *in, T *out) {                 \
        const int32_t *order = h->order ? h->order[l] : NULL;                                       \
        if (order) or_ldtri_order_##SFX(&h->LD[l], order, in, out);                                 \
        else or_ldtri_##SFX(&h->LD[l], h->bj ? h->bj[l] : NULL, h->nbj, in, out);                   \
    }                                                                                               \
    static void smooth_##SFX(const or_amg_##SFX *h, int l, const T *in, T *out, int inited) {     \
        const or_csr_##SFX *U = &h->U[l];                                                           \
        const int n = h->LD[l].n;                                                                   \
        T *tmp = (T *)malloc(sizeof(T) * (size_t)n);                                                \
        int k0 = 0;                                                                                 \
        if (!inited) { sweep_##SFX(h, l, in, out); k0 = 1; }                                        \
        for (int k = k0; k < h->smooth_iter; k++) {                                                 \
            or_spmv_##SFX(U, out, tmp);                                                             \
            for (int i = 0; i < n; i++) tmp[i] = (T)1 * in[i] + (T)(-1) * tmp[i];                   \
            sweep_##SFX(h, l, tmp, out);                                                            \
        }                                                                                           \
        free(tmp);                                                                                  \
    }                                                                                               \
    /* dfAMG::Precondition (INTAMG.hpp:108-133) with LU<T>::Solve (lu.hpp:30-33) */               \
    void or_vcycle_##SFX(const or_amg_##SFX *h, const T *in, T *out) {                            \
        const int D = h->depth, N = h->A0.n;                                                        \
        T *r = (T *)malloc(sizeof(T) * (size_t)N);                                                  \
        T **rr = (T **)malloc(sizeof(T *) * (size_t)D);                                             \
        T **ee = (T **)malloc(sizeof(T *) * (size_t)D);                                             \
        T **xx = (T **)malloc(sizeof(T *) * (size_t)D);                                             \
        for (int i = 0; i < D; i++) {                                                               \
            rr[i] = (T *)calloc((size_t)h->R[i].n, sizeof(T));                                      \
            ee[i] = (T *)calloc((size_t)h->R[i].n, sizeof(T));                                      \
            xx[i] = (T *)calloc((size_t)h->R[i].n, sizeof(T));                                      \
        }                                                                                           \
        smooth_##SFX(h, 0, in, out, 0);                                                             \
        or_spmv_##SFX(&h->A0, out, r);                                                              \
        for (int k = 0; k < N; k++) r[k] = in[k] - r[k];                                            \
        or_spmv_##SFX(&h->R[0], r, ee[0]);                                                          \
        for (int i = 0; i < D - 1; i++) {                                                           \
            smooth_##SFX(h, i + 1, ee[i], xx[i], 0);                                                \
            or_spmv_##SFX(&h->CA[i], xx[i], rr[i]);                                                 \
            for (int k = 0; k < h->CA[i].n; k++) rr[i][k] = ee[i][k] - rr[i][k];                   \
            or_spmv_##SFX(&h->R[i + 1], rr[i], ee[i + 1]);                                          \
        }                                                                                           \
        {                                                                                           \
            T *tmp = (T *)malloc(sizeof(T) * (size_t)h->LUL.n);                                     \
            or_ltri_##SFX(&h->LUL, ee[D - 1], tmp);                                                 \
            or_dutri_##SFX(&h->LUU, tmp, xx[D - 1]);                                                \
            free(tmp);                                                                              \
        }                                                                                           \
        for (int i = D - 2; i >= 0; i--) {                                                          \
            or_spmv_##SFX(&h->P[i + 1], xx[i + 1], rr[i]);                                          \
            for (int k = 0; k < h->CA[i].n; k++) xx[i][k] = rr[i][k] + xx[i][k];                    \
            smooth_##SFX(h, i + 1, ee[i], xx[i], 1);                                                \
        }                                                                                           \
        or_spmv_##SFX(&h->P[0], xx[0], r);                                                          \
        for (int k = 0; k < N; k++) out[k] = r[k] + out[k];                                         \
        smooth_##SFX(h, 0, in, out, 1);                                                             \
        for (int i = 0; i < D; i++) { free(rr[i]); free(ee[i]); free(xx[i]); }                      \
        free(rr); free(ee); free(xx); free(r);                                                      \
    }

DEFINE_FP(f64, double)
DEFINE_FP(f32, float)

/* blas1 generic kernels in precision T, sequential (blas1.hpp:16-68, 83-96) */
#define DEFINE_FP_BLAS(SFX, T, SQRT)                                                               \
    static T dot_##SFX(const T *x, const T *y, int n) {                                            \
        T s = 0;                                                                                    \
        for (int i = 0; i < n; i++) s += x[i] * y[i];                                               \
        return s;                                                                                   \
    }                                                                                               \
    static T ggen_##SFX(T a, T b, T *c, T *s) {                                                    \
        T r = SQRT(a * a + b * b);                                                                  \
        *c = a / r;                                                                                 \
        *s = -b / r;                                                                                \
        return r;                                                                                   \
    }                                                                                               \
    static void grot_##SFX(T c, T s, T *a, T *b) {                                                 \
        T t = *a;                                                                                   \
        *a = c * t - s * *b;                                                                        \
        *b = s * t + c * *b;                                                                        \
    }                                                                                               \
    /* blas2::Trsv (blas2.hpp:25-34) */                                                            \
    static void trsv_##SFX(const T *U, const T *b, T *x, int n, int m) {                           \
        for (int i = m - 1; i >= 0; i--) {                                                          \
            T t = b[i];                                                                             \
            for (int j = m - 1; j > i; j--) t -= U[j * n + i] * x[j];                               \
            x[i] = t / U[i * n + i];                                                                \
        }                                                                                           \
    }

DEFINE_FP_BLAS(f64, double, sqrt)
DEFINE_FP_BLAS(f32, float, sqrtf)

/* FGMRES<double>::Solve (gmres.hpp:130-170) */
static int fgmres_f64(const or_csr_f64 *A, const or_amg_f64 *M, int m, double eps, const double *r,
                      double nrm_b, double *x, double *V, double *Z, double *H, double *c, double *s,
                      double *e, double *y, int *converged, int print) {
    const int N = A->n;
    const size_t NN = (size_t)N;
    e[0] = or_nrm2_f64(r, N);
    double e_inv = 1.0 / e[0];
    for (int k = 0; k < N; k++) V[k] = r[k] * e_inv;
    int flag = 0, j;
    for (j = 0; j < m; j++) {
        double *w = V + (size_t)(j + 1) * NN, *Hj = H + (size_t)j * (m + 1);
        or_vcycle_f64(M, V + (size_t)j * NN, Z + (size_t)j * NN);
        or_spmv_f64(A, Z + (size_t)j * NN, w);
        for (int k = 0; k <= j; k++) {
            const double *vk = V + (size_t)k * NN;
            Hj[k] = dot_f64(vk, w, N);
            double a = -Hj[k];
            for (int i = 0; i < N; i++) w[i] += a * vk[i];
        }
        Hj[j + 1] = sqrt(dot_f64(w, w, N));
        double a = 1 / Hj[j + 1];
        for (int i = 0; i < N; i++) w[i] *= a;
        for (int k = 0; k < j; k++) grot_f64(c[k], s[k], &Hj[k], &Hj[k + 1]);
        Hj[j] = ggen_f64(Hj[j], Hj[j + 1], &c[j], &s[j]);
        Hj[j + 1] = 0;
        e[j + 1] = s[j] * e[j];
        e[j] = c[j] * e[j];
        if (print) printf("# [%d] %e\n", j + 1, fabs(e[j + 1] / nrm_b));
        if (fabs(e[j + 1]) <= nrm_b * eps) {
            if (print) printf("[Res] : %e\n", fabs(e[j + 1]) / nrm_b);
            j++;
            flag = 1;
            break;
        }
    }
    trsv_f64(H, e, y, m + 1, j);
    for (int k = 0; k < j; k++) {
        const double *zk = Z + (size_t)k * NN;
        for (int i = 0; i < N; i++) x[i] += y[k] * zk[i];
    }
    *converged = flag;
    return flag ? j : m;
}

int or_ir_solve_f64(const or_csr_f64 *dA, const or_amg_f64 *M, int m, double eps, const double *b,
                    double nrm_b, double *x, int max_outer, int print) {
    const int N = dA->n;
    const size_t NN = (size_t)N;
    double *r = (double *)malloc(sizeof(double) * NN);
    double *V = (double *)malloc(sizeof(double) * NN * (size_t)(m + 1));
    double *Z = (double *)malloc(sizeof(double) * NN * (size_t)(m + 1));
    double *H = (double *)calloc((size_t)(m + 1) * (size_t)m, sizeof(double));
    double *c = (double *)calloc((size_t)m, sizeof(double));
    double *s = (double *)calloc((size_t)m, sizeof(double));
    double *e = (double *)calloc((size_t)m + 1, sizeof(double));
    double *y = (double *)calloc((size_t)m, sizeof(double));
    double prev = 0;
    int iter = 0, result = 0;
    for (int i = 0; i < max_outer; i++) {
        or_spmv_f64(dA, x, r);
        axpby_sub_f64(b, r, N);
        double nrm_r = or_nrm2_f64(r, N);
        if (fabs(nrm_r - prev) / nrm_r < 1.0e-8) break;
        prev = nrm_r;
        int conv = 0;
        iter += fgmres_f64(dA, M, m, eps, r, nrm_b, x, V, Z, H, c, s, e, y, &conv, print);
        if (conv) { result = iter; break; }
    }
    free(r); free(V); free(Z); free(H); free(c); free(s); free(e); free(y);
    return result;
}

/* FGMRES<float>::Solve (gmres.hpp:212-252) inside Restarted with the FP64 A. */
static int fgmres_f32(const or_csr_f32 *A, const or_amg_f32 *M, int m, double eps, const double *r,
                      double nrm_b, double *x, float *V, float *Z, float *H, float *c, float *s,
                      float *e, float *y, int *converged, int print) {
    const int N = A->n;
    const size_t NN = (size_t)N;
    e[0] = (float)or_nrm2_f64(r, N);
    double e_inv = 1.0 / e[0];
    for (int k = 0; k < N; k++) V[k] = (float)(r[k] * e_inv);
    int flag = 0, j;
    for (j = 0; j < m; j++) {
        float *w = V + (size_t)(j + 1) * NN, *Hj = H + (size_t)j * (m + 1);
        or_vcycle_f32(M, V + (size_t)j * NN, Z + (size_t)j * NN);
        or_spmv_f32(A, Z + (size_t)j * NN, w);
        for (int k = 0; k <= j; k++) {
            const float *vk = V + (size_t)k * NN;
            Hj[k] = dot_f32(vk, w, N);
            float a = -Hj[k];
            for (int i = 0; i < N; i++) w[i] += a * vk[i];
        }
        Hj[j + 1] = sqrtf(dot_f32(w, w, N));
        float a = 1 / Hj[j + 1];
        for (int i = 0; i < N; i++) w[i] *= a;
        for (int k = 0; k < j; k++) grot_f32(c[k], s[k], &Hj[k], &Hj[k + 1]);
        Hj[j] = ggen_f32(Hj[j], Hj[j + 1], &c[j], &s[j]);
        Hj[j + 1] = 0;
        e[j + 1] = s[j] * e[j];
        e[j] = c[j] * e[j];
        if (print) printf("# [%d] %e\n", j + 1, fabs(e[j + 1] / nrm_b));
        if (fabsf(e[j + 1]) <= nrm_b * eps) {
            if (print) printf("[Res] : %e\n", fabsf(e[j + 1]) / nrm_b);
            j++;
            flag = 1;
            break;
        }
    }
    trsv_f32(H, e, y, m + 1, j);
    for (int k = 0; k < j; k++) {
        const float *zk = Z + (size_t)k * NN;
        for (int i = 0; i < N; i++) x[i] += (double)(y[k] * zk[i]); /* AxpyFD (blas1.hpp:98-101) */
    }
    *converged = flag;
    return flag ? j : m;
}

int or_ir_solve_f32(const or_csr_f64 *dA, const or_csr_f32 *fA, const or_amg_f32 *M, int m, double eps,
                    const double *b, double nrm_b, double *x, int max_outer, int print) {
    const int N = dA->n;
    const size_t NN = (size_t)N;
    double *r = (double *)malloc(sizeof(double) * NN);
    float *V = (float *)malloc(sizeof(float) * NN * (size_t)(m + 1));
    float *Z = (float *)malloc(sizeof(float) * NN * (size_t)(m + 1));
    float *H = (float *)calloc((size_t)(m + 1) * (size_t)m, sizeof(float));
    float *c = (float *)calloc((size_t)m, sizeof(float));
    float *s = (float *)calloc((size_t)m, sizeof(float));
    float *e = (float *)calloc((size_t)m + 1, sizeof(float));
    float *y = (float *)calloc((size_t)m, sizeof(float));
    double prev = 0;
    int iter = 0, result = 0;
    for (int i = 0; i < max_outer; i++) {
        or_spmv_f64(dA, x, r);
        axpby_sub_f64(b, r, N);
        double nrm_r = or_nrm2_f64(r, N);
        if (fabs(nrm_r - prev) / nrm_r < 1.0e-8) break;
        prev = nrm_r;
        int conv = 0;
        iter += fgmres_f32(fA, M, m, eps, r, nrm_b, x, V, Z, H, c, s, e, y, &conv, print);
        if (conv) { result = iter; break; }
    }
    free(r); free(V); free(Z); free(H); free(c); free(s); free(e); free(y);
    return result;
}
