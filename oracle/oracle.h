/* CPU restatement of the reference solve phase.  TEST INFRASTRUCTURE ONLY.
 *
 * This is the oracle: a plain-C re-statement of suzuki-hpc/SC23-AD's integer,
 * FP64 and FP32 AMG-preconditioned FGMRES solve phase (every function cites the
 * reference file:line it follows).  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it, and only as the checker or as the
 * timed CPU baseline; the product never links it.
 *
 * It is pinned against the reference itself: tests/golden/*.npz hold arrays and
 * kernel input/output pairs dumped by oracle/ref_harness.cpp, which drives the
 * reference's own classes (tests/test_oracle_golden.py checks this file against
 * them bit for bit).
 *
 * Integer semantics follow the reference compiled by g++ on a 64-bit target:
 * `long` is int64, `(int)` of an int64 keeps the low 32 bits, `>>` of a negative
 * value is an arithmetic shift, and integer sums wrap.  Those wraps are
 * undefined in C, so the code below does them on unsigned types explicitly.
 */
#ifndef SA_ORACLE_H
#define SA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int n, m; const int32_t *rptr, *cind, *val; int bit, dbit; } or_csr_i32;
typedef struct { int n, m; const int32_t *rptr, *cind; const double *val; } or_csr_f64;
typedef struct { int n, m; const int32_t *rptr, *cind; const float *val; } or_csr_f32;

/* Integer AMG hierarchy in the reference's own numbering (INTAMG.hpp:136-147):
 * depth coarse levels, CA[0..depth-2], P[0..depth-1] (Intrpl), R[0..depth-1]
 * (Intrpl_t), smoother of level l = (LD[l], U[l]) for l in 0..depth-1, with
 * optional block-Jacobi boundaries bj[l] (nbj blocks) for BlockSORflex, and the
 * coarsest LU factors (ltri LUL, dutri LUU).  order (optional, may be NULL or
 * hold NULL levels) gives, per level, the row order of the smoother's forward
 * sweep: the multicolour variant sweeps the rows colour by colour
 * (ldtri::MCCSR, matrix/trispmat.hpp:597-640, after the MC renumbering). */
typedef struct {
    int depth;
    or_csr_i32 A0;
    const or_csr_i32 *CA, *P, *R, *LD, *U;
    const int32_t *const *bj;
    int nbj;
    int smooth_iter;
    or_csr_i32 LUL, LUU;
    const int32_t *const *order;
} or_amg_i32;

typedef struct {
    int depth;
    or_csr_f64 A0;
    const or_csr_f64 *CA, *P, *R, *LD, *U;
    const int32_t *const *bj;
    int nbj;
    int smooth_iter;
    or_csr_f64 LUL, LUU;
    const int32_t *const *order;
} or_amg_f64;

typedef struct {
    int depth;
    or_csr_f32 A0;
    const or_csr_f32 *CA, *P, *R, *LD, *U;
    const int32_t *const *bj;
    int nbj;
    int smooth_iter;
    or_csr_f32 LUL, LUU;
    const int32_t *const *order;
} or_amg_f32;

/* Threads used by the parallel loops (SpMV rows, integer reductions).  FP
 * reductions stay sequential so that results do not depend on it. */
void or_set_threads(int nthreads);
int or_get_threads(void);

/* --- integer kernels --- */
int or_spmv_i32(const or_csr_i32 *A, const int32_t *in, int32_t *out);
int or_ldtri_i32(const or_csr_i32 *LD, const int32_t *bj, int nbj, const int32_t *in, int32_t *out);
/* the same forward sweep, rows visited in the given order (a permutation) */
int or_ldtri_order_i32(const or_csr_i32 *LD, const int32_t *order, const int32_t *in, int32_t *out);
int or_ltri_i32(const or_csr_i32 *L, const int32_t *in, int32_t *out);
int or_dutri_i32(const or_csr_i32 *U, const int32_t *in, int32_t *out);
int64_t or_lsqrt(int64_t x);
int64_t or_dot_i32(const int32_t *x, const int32_t *y, int n, int bit);
int64_t or_nrm2_i32(const int32_t *x, int n);
void or_axpy_i32(int64_t a, const int32_t *x, int32_t *y, int n, int bit);
void or_scal_i32(int64_t a, int32_t *x, int n, int bit);
void or_axpy_d(double a, const int32_t *x, double *y, int n, int bit);
int64_t or_ggen_i32(int64_t a, int64_t b, int64_t *c, int64_t *s, int bit);
void or_grot_i32(int64_t c, int64_t s, int64_t *a, int64_t *b, int bit);
void or_trsv_i32(const int64_t *H, double e0, const int64_t *e, double *y, int ld, int m, int bit);
void or_smooth_i32(const or_amg_i32 *h, int level, const int32_t *in, int32_t *out, int inited);
void or_lu_i32(const or_amg_i32 *h, const int32_t *in, int32_t *out);
void or_vcycle_i32(const or_amg_i32 *h, const int32_t *in, int32_t *out);

/* One call of FGMRESflex::Solve.  V, Z: (m+1)*n int32; H: (m+1)*m int64;
 * c, s: m; e: m+1; y: m doubles.  e0_in: if non-NULL, used instead of the FP64
 * norm of r.  Returns the iterations done; *converged set.  print: emit the
 * reference's per-iteration lines on stdout. */
int or_fgmres_i32_cycle(const or_csr_i32 *A, const or_amg_i32 *M, int m, double eps, int bit,
                        const double *r, double nrm_b, double *x,
                        int32_t *V, int32_t *Z, int64_t *H, int64_t *c, int64_t *s, int64_t *e,
                        double *y, const double *e0_in, int *converged, int print);

/* Restarted(FGMRESflex) (irsolver.hpp:61-77).  Returns total iterations if
 * converged, 0 otherwise (the reference's Converge.iter). */
int or_ir_solve_i32(const or_csr_f64 *dA, const or_csr_i32 *A, const or_amg_i32 *M, int m, double eps,
                    int bit, const double *b, double nrm_b, double *x, int max_outer, int print);

/* --- FP64 / FP32 siblings --- */
int or_spmv_f64(const or_csr_f64 *A, const double *in, double *out);
int or_ldtri_f64(const or_csr_f64 *LD, const int32_t *bj, int nbj, const double *in, double *out);
int or_ldtri_order_f64(const or_csr_f64 *LD, const int32_t *order, const double *in, double *out);
int or_ltri_f64(const or_csr_f64 *L, const double *in, double *out);
int or_dutri_f64(const or_csr_f64 *U, const double *in, double *out);
void or_vcycle_f64(const or_amg_f64 *h, const double *in, double *out);
int or_ir_solve_f64(const or_csr_f64 *dA, const or_amg_f64 *M, int m, double eps,
                    const double *b, double nrm_b, double *x, int max_outer, int print);

int or_spmv_f32(const or_csr_f32 *A, const float *in, float *out);
int or_ldtri_f32(const or_csr_f32 *LD, const int32_t *bj, int nbj, const float *in, float *out);
int or_ldtri_order_f32(const or_csr_f32 *LD, const int32_t *order, const float *in, float *out);
void or_vcycle_f32(const or_amg_f32 *h, const float *in, float *out);
int or_ir_solve_f32(const or_csr_f64 *dA, const or_csr_f32 *fA, const or_amg_f32 *M, int m, double eps,
                    const double *b, double nrm_b, double *x, int max_outer, int print);

double or_nrm2_f64(const double *x, int n);

/* Restarted(FGMRESflex) as or_ir_solve_i32 with a choice of stop: the
 * reference's (the inner solver's estimate, irsolver.hpp:38-40) or, with
 * explicit_stop, the explicit FP64 residual ||b - A x|| <= eps ||b|| checked
 * before every refinement step after the first.  *res_out (optional) = the
 * explicit relative residual at return.  Returns the iterations if converged,
 * else 0. */
int or_ir_solve_i32x(const or_csr_f64 *dA, const or_csr_i32 *A, const or_amg_i32 *M, int m, double eps,
                     int bit, const double *b, double nrm_b, double *x, int max_outer, int explicit_stop,
                     double *res_out);

/* The batched engine's early restart, which the reference lacks: with bits
 * = K > 0 a cycle of or_fgmres_i32_cycle also ends (not converged) once
 * |e_{j+1}| <= 2^(F-K), i.e. the estimate has fallen 2^K below its start
 * e_0 = 2^F.  0 (the default) is the reference's FGMRESflex. */
void or_set_cycle_bits(int bits);

/* --- the AMG setup (oracle_setup.c) ---
 * helper::multigrid::get_amg_set (helper_multigrid.hpp:34-63) in the level
 * loop of the AMG constructors (INTAMG.hpp:38-51, 162-195: a level is added
 * while max_levels > depth and the last coarse operator has more than
 * coarse_limit rows; the reference uses 2000), with the data both
 * constructors prepare: intAMGflex (coarse rows scaled by their maxima, SOR
 * split, exact LU, fixed-point conversions) and dfAMG (FP64).  The input is the
 * LMax1-scaled fine matrix (copied).  *status: 0, -1 where the reference exits
 * (an unclassified point, or "2 amk = 0"), -2 for invalid arguments. */
typedef struct or_setup or_setup;
or_setup *or_setup_create(int n, const int32_t *rptr, const int32_t *cind, const double *val, double theta,
                          int max_levels, int coarse_limit, double omega, int *status);
void or_setup_destroy(or_setup *s);
int or_setup_depth(const or_setup *s);
long or_setup_warnings(const or_setup *s); /* the reference's "1 amk = 0" messages */
/* hierarchy structs viewing the setup's arrays (valid while it lives) */
void or_setup_amg_i32(const or_setup *s, or_amg_i32 *h);
void or_setup_amg_f64(const or_setup *s, or_amg_f64 *h);

#ifdef __cplusplus
}
#endif
#endif
