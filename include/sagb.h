/* sagb.h -- C ABI of the GB300 solve phase of int-AMG-FGMRES(m)
 *
 * The reference (suzuki-hpc/SC23-AD, a header-only C++ library) has no FFI of
 * its own; its solve phase is reached through C++ objects.  Every entry point
 * below replaces one of those reference interfaces, cited as Library/<file>:line.
 * The C++ drop-in headers under include/senk/ are written on top of this ABI.
 *
 * Conventions
 *  - Every function returns SA_OK (0) or an SA_ERR_* code; none calls exit()
 *    or traps.  sa_last_error() returns a message for the calling thread.
 *  - Vector arguments may be host or device pointers (device = cudaMalloc'd or
 *    managed memory); host buffers are staged through device memory.
 *  - Integer vectors are int32 fixed point with `bits` fractional bits; the
 *    arithmetic is the reference's, bit for bit (int64 products and sums,
 *    arithmetic right shifts, int32 wrap-around), and any int32 overflow is
 *    reported through the status flags instead of being silent.
 *  - One context = one GPU and one CUDA stream; calls on a context are
 *    serialised by the caller.
 */
#ifndef SAGB_H
#define SAGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- codes */
#define SA_OK 0
#define SA_ERR_ARG 1      /* invalid argument                                  */
#define SA_ERR_CUDA 2     /* CUDA runtime error (no GPU, out of memory, ...)   */
#define SA_ERR_SETUP 3    /* the host setup rejected the matrix                */
#define SA_ERR_NUMERIC 4  /* a device status flag stopped the solve            */

/* device status flags (sa_ctx_flags) */
#define SA_FLAG_OVERFLOW 1u       /* an int32 result wrapped (the reference would silently wrap) */
#define SA_FLAG_TIMEOUT 2u        /* a bounded device-side wait ran out                          */
#define SA_FLAG_DIVZERO 4u        /* zero Hessenberg / Givens denominator                        */
#define SA_FLAG_NORM_OVERFLOW 8u  /* int64 sum of squares wrapped                                */
#define SA_FLAG_PRECOND_OVERFLOW 16u /* an int32 result wrapped inside the V-cycle (FGMRES continues) */

/* precisions */
#define SA_INT 0 /* int32 fixed point, int64 accumulation (FGMRESflex/intAMGflex) */
#define SA_F64 1 /* FP64 (FGMRES<double>/dfAMG<...,double>)                      */
#define SA_F32 2 /* FP32 (FGMRES<float>/dfAMG<...,float>)                        */

/* matrix kinds for sa_mat_create */
#define SA_MAT_FIXED 0 /* CSR<Fixed<bit>>: (int)(a * 2^bit)       Library/matrix/spmat.hpp:55-70  */
#define SA_MAT_FLEX 1  /* CSRflex: own bit from max|a|            Library/matrix/spmat.hpp:89-121 */
#define SA_MAT_F64 2   /* CSR<double>                             Library/matrix/spmat.hpp:21-36  */
#define SA_MAT_F32 3   /* CSR<float>                              Library/matrix/spmat.hpp:21-36  */

/* operators of a hierarchy (sa_amg_level_spmv, sa_setup_view, ...) */
#define SA_OP_A0 0  /* fine operator                                  */
#define SA_OP_CA 1  /* coarse operator C_A[level]                      */
#define SA_OP_P 2   /* interpolation Intrpl[level]                     */
#define SA_OP_R 3   /* restriction Intrpl_t[level]                     */
#define SA_OP_LD 4  /* smoother lower factor (D^-1 last in each row)   */
#define SA_OP_U 5   /* smoother upper part                             */
#define SA_OP_LUL 6 /* coarsest LU, unit lower factor (ltri)           */
#define SA_OP_LUU 7 /* coarsest LU, D^-1 U (dutri)                     */
#define SA_OP_BJ 8  /* block boundaries of a BlockSOR smoother (rptr)  */
#define SA_OP_COLOR 9 /* colour of each row of a multicolour smoother (view.rptr, n rows) */

/* synthetic systems for sa_gen */
#define SA_GEN_POISSON2D 0  /* 5-point, 4/-1                             */
#define SA_GEN_POISSON3D 1  /* 7-point, 6/-1                             */
#define SA_GEN_ANISO2D 2    /* 5-point, -u_xx - p*u_yy                   */
#define SA_GEN_STENCIL27 3  /* 27-point, diag 26+U[0.1,1], off -1        */
#define SA_GEN_CONVDIFF3D 4 /* 7-point upwinded convection-diffusion, Pe=p */
#define SA_GEN_VARCOEF3D 5  /* 7-point lognormal(0,p) harmonic-mean faces */

typedef struct sa_context *sa_ctx;
typedef struct sa_matrix *sa_mat;
typedef struct sa_multigrid *sa_amg;
typedef struct sa_krylov *sa_solver;
typedef struct sa_hierarchy *sa_setup;
typedef struct sa_host_csr *sa_hcsr;
typedef struct sa_timer *sa_event;

typedef struct {
    int n, m;
    int64_t nnz;
    const int32_t *rptr, *cind;
    const void *val; /* double for FP64 views, int32 for integer views, float for FP32 */
    int bit, dbit;
} sa_csr_view;

typedef struct {
    int max_levels;      /* AMGParam::level (20)                      Library/parameters.hpp:253-264 */
    double theta;        /* AMGParam::theta (0.8 in Work/main.cpp:32)                                */
    int smoother_blocks; /* 0: SOR, >0: BlockSOR with this many blocks  Library/parameters.hpp:223-241 */
    double omega;        /* SORParam::omega (1.0)                                                     */
    int smooth_iter;     /* SORParam::iter (1)                                                        */
    int multicolor;      /* 1: SOR in greedy-colour order (ldtri::MCCSR, matrix/trispmat.hpp:597-640,
                            colouring helper/helper_graph.hpp:191-219); 2: JacobiSORflex
                            (smoother/stationary.hpp:564-676: chunks of 1200 consecutive rows, GS
                            across chunks, Jacobi inside one; single-system setups only); 0: natural
                            order (default) */
    int max_colours;     /* multicolour: cap on the colours per level, rows beyond it join their least
                            conflicting colour (Jacobi-like inside it); 0: no cap (default) */
    int coarse_size;     /* coarsen while the coarsest level has more rows than this; 0: the
                            reference's 2000 (INTAMG.hpp:38-51) */
    int coarse_colours;  /* multicolour: the cap on the levels below the finest (0: max_colours) */
} sa_amg_params;

typedef struct {
    int m;                 /* restart length (FGMRES m)                Library/solver/gmres.hpp:276-297 */
    double eps;            /* relative tolerance (1e-10)                                                */
    int max_outer;         /* Restarted max cycles (1000/m)            Library/solver/irsolver.hpp:50-57 */
    int frac_bits;         /* F_G of the integer solver (FGMRESflex bit)                                */
    int verbose;           /* print the reference's "# [j] res" / "[Res]" lines                         */
    int overflow_fallback; /* int only: on an overflow flag, redo the cycle with F-1 (0: reference behaviour) */
    int explicit_stop;     /* 1: stop only when ||b - A x|| / ||b|| <= eps in FP64 (the reference stops on
                              the inner solver's implicit estimate, which can leave it above eps)      */
    int cycle_bits;        /* batched integer solver only (no counterpart in the reference): a pair's
                              restart cycle also ends, unconverged, once its estimate |e_{j+1}| has
                              fallen 2^cycle_bits below the cycle's start e_0 = 2^F; the FP64
                              refinement then restarts from the true residual.  An F-bit basis stops
                              gaining about 2^20 below its start, so the rest of a long cycle is
                              wasted.  0: the full m steps, as FGMRESflex (gmres.hpp:237-262)      */
} sa_solver_params;

/* ------------------------------------------------------------- library */
const char *sa_version(void);
const char *sa_last_error(void);

/* ------------------------------------------------------------- context */
int sa_ctx_create(int device, sa_ctx *out);
int sa_ctx_destroy(sa_ctx ctx);
#define SA_OPT_FP_EXACT 0 /* FP kernels in the reference's sequential order, no FMA (bit-exact) */
#define SA_OPT_GRAPHS 1   /* capture Arnoldi steps into CUDA graphs (default on)              */
#define SA_OPT_PDL 2      /* batched engine: start each V-cycle kernel while the one before it
                           * drains (programmatic dependent launch; default on)               */
#define SA_OPT_GPU_SETUP 3 /* sa_batch_create: the Ruge-Stueben chain of each system of at least
                            * this many rows on the GPU (same hierarchy bit for bit): 0 none, 1
                            * the default 2^20 (smaller systems build faster side by side on the
                            * host threads), >= 2 that many rows */
#define SA_OPT_CYCLE_GRAPH 4 /* batched engines: each restart cycle as one CUDA graph whose steps after
                              * the first run only while a pair is still active (the convergence test
                              * of gmres.hpp:257 on the device, no host round trip per step); off:
                              * one graph per step and a status read after each (default on) */
int sa_ctx_set_option(sa_ctx ctx, int option, int value);
int sa_ctx_flags(sa_ctx ctx, unsigned *flags, int clear);
int sa_ctx_launches(sa_ctx ctx, long long *count);
int sa_ctx_sync(sa_ctx ctx);
int sa_ctx_stream(sa_ctx ctx, void **stream); /* the cudaStream_t all work is queued on */

/* device memory and timing helpers (no library state) */
int sa_device_alloc(sa_ctx ctx, uint64_t bytes, void **ptr);
int sa_device_free(sa_ctx ctx, void *ptr);
int sa_memcpy(sa_ctx ctx, void *dst, const void *src, uint64_t bytes); /* any direction, synchronous */
int sa_host_alloc(uint64_t bytes, void **ptr); /* page-locked host memory (fast host<->device copies) */
int sa_host_free(void *ptr);
int sa_event_create(sa_event *out);
int sa_event_record(sa_ctx ctx, sa_event ev);
int sa_event_elapsed_ms(sa_event start, sa_event stop, float *ms);
int sa_event_destroy(sa_event ev);

/* ------------------------------------------------- host CSR and generators */
/* io::ReadMM(path, true, false)                      Library/io/mm.hpp:24-98 */
int sa_hcsr_read_mm(const char *path, sa_hcsr *out);
/* the same through a binary cache file: read when it records this very
 * Matrix Market file (size and modification time), else written after the
 * parse (an unwritable cache is skipped) */
int sa_hcsr_read_mm_cached(const char *mm_path, const char *cache_path, sa_hcsr *out);
/* a host CSR to / from the binary CSR file (header, rptr, cind, val) */
int sa_hcsr_save(sa_hcsr A, const char *path);
int sa_hcsr_load(const char *path, sa_hcsr *out);
int sa_hcsr_create(int n, int m, const int32_t *rptr, const int32_t *cind, const double *val, sa_hcsr *out);
int sa_hcsr_view(sa_hcsr A, sa_csr_view *out);
/* CSRMat::LMax1Scaling(b)                            Library/matrix/csrmat.hpp:70-80 */
int sa_hcsr_lmax1_scaling(sa_hcsr A, double *b);
/* x* ~ U[-1,1] (splitmix64 seed), b = A x* (row order) -- synthetic right-hand side */
int sa_hcsr_rhs(sa_hcsr A, uint64_t seed, double *xstar, double *b);
int sa_hcsr_destroy(sa_hcsr A);
int sa_gen(int kind, int nx, double param, uint64_t seed, sa_hcsr *out);

/* ------------------------------------------------------------ matrices */
/* CSR<Fixed<bit>>(CSRMat*) / CSRflex(CSRMat*) / CSR<double> / CSR<float>
 *                                   Library/matrix/spmat.hpp:28-36, 62-70, 96-121 */
int sa_mat_create(sa_ctx ctx, int kind, int bit, int n, int m, const int32_t *rptr, const int32_t *cind,
                  const double *val, sa_mat *out);
/* an already quantised int32 CSR with `bit` fractional bits */
int sa_mat_create_i32(sa_ctx ctx, int n, int m, const int32_t *rptr, const int32_t *cind, const int32_t *val,
                      int bit, sa_mat *out);
int sa_mat_destroy(sa_mat A);
int sa_mat_info(sa_mat A, int *n, int *m, int64_t *nnz, int *bit, int *precision);
/* SpMat<T>::SpMV(in, out)          Library/matrix/spmat.hpp:43-52, 77-86, 128-137 */
int sa_spmv(sa_ctx ctx, sa_mat A, const void *x, void *y);

/* --------------------------------------------------------- host AMG setup */
void sa_amg_params_default(sa_amg_params *p);
/* the hierarchy a dfAMG / intAMGflex constructor builds (host only, no GPU):
 *                                   Library/preconditioner/INTAMG.hpp:25-84, 149-245 */
int sa_setup_create(int precision, const sa_amg_params *p, int n, const int32_t *rptr, const int32_t *cind,
                    const double *val, sa_setup *out);
/* the same hierarchy, bit for bit, with the Ruge-Stueben levels' strength
 * split, transposes, interpolation and Galerkin products on the context's GPU
 * (the C/F splitting, smoother splits and quantisation stay on the host)
 *                                   Library/helper/helper_multigrid.hpp:34-586 */
int sa_setup_create_gpu(sa_ctx ctx, int precision, const sa_amg_params *p, int n, const int32_t *rptr,
                        const int32_t *cind, const double *val, sa_setup *out);
/* the hierarchy of another precision over the same coarsening (the Ruge-Stueben
 * chain does not depend on the precision; dfAMG and intAMGflex both build it from
 * the unscaled operators, Library/preconditioner/INTAMG.hpp:38-51, 162-173) */
int sa_setup_derive(sa_setup s, int precision, sa_setup *out);
int sa_setup_destroy(sa_setup s);
int sa_setup_depth(sa_setup s);
int sa_setup_view(sa_setup s, int op, int level, sa_csr_view *out);

/* ------------------------------------------------------------------ AMG */
/* dfAMG<...>(CSRMat*, SpMat<T>*, AMGParam*) / intAMGflex<...>(CSRMat*, SpMat<int>*, AMGParam*):
 * host setup + upload.             Library/preconditioner/INTAMG.hpp:25-84, 149-245 */
int sa_amg_create(sa_ctx ctx, int precision, const sa_amg_params *p, int n, const int32_t *rptr,
                  const int32_t *cind, const double *val, sa_amg *out);
int sa_amg_create_from_setup(sa_ctx ctx, sa_setup s, sa_amg *out);
int sa_amg_destroy(sa_amg M);
int sa_amg_depth(sa_amg M);
int sa_amg_precision(sa_amg M);
/* Preconditioner<T>::Precondition(in, out): one V-cycle
 *                                   Library/preconditioner/INTAMG.hpp:108-133, 269-293 */
int sa_amg_precondition(sa_ctx ctx, sa_amg M, const void *in, void *out);
/* Smoother<T>::Smooth(in, out, isInited) of level l
 *                                   Library/smoother/stationary.hpp:238-255, 415-430, 997-1012 */
int sa_amg_smooth(sa_ctx ctx, sa_amg M, int level, const void *in, void *out, int inited);
/* ldtri::SpMat<T>::SpTRSV of level l's smoother (one Gauss-Seidel sweep)
 *                                   Library/matrix/trimat/ldtri.hpp:49-58, 172-183, 398-412, 511-525 */
int sa_amg_sweep(sa_ctx ctx, sa_amg M, int level, const void *in, void *out);
/* No counterpart in the reference.  The same sweep as sa_amg_sweep, but it
 * allocates no device memory: for callers that cannot call cudaMalloc while
 * they solve -- their GPU memory is already claimed by another allocator (a
 * framework's caching allocator, a fixed pool), or they cannot afford the
 * device-wide synchronisation that allocating and freeing imply.  in and out
 * must be device buffers.  The fine-level sweep kernel's scratch comes from a
 * static device array sized for 262,144 rows (2 MiB, held by every GPU that
 * loads the library until the process exits); a level with more rows is
 * rejected with SA_ERR_ARG.  The first call on a device looks up that array's
 * address, so make the first call before any stream capture.  Every call
 * shares the array: calls that overlap on the GPU race. */
int sa_amg_sweep_noalloc(sa_ctx ctx, sa_amg M, int level, const void *in, void *out);
/* direct::LUflex::Solve / LU<T>::Solve   Library/solver/lu.hpp:30-33, 91-94 */
int sa_amg_coarse_solve(sa_ctx ctx, sa_amg M, const void *in, void *out);
/* SpMV with one operator of the hierarchy (SA_OP_A0, _CA, _P, _R, _U) */
int sa_amg_level_spmv(sa_ctx ctx, sa_amg M, int op, int level, const void *in, void *out);
/* sizes of an operator; nlev = number of dependency levels of a triangular sweep */
int sa_amg_level_info(sa_amg M, int op, int level, int *n, int *m, int64_t *nnz, int *bit, int *nlev);

/* --------------------------------------------------------------- solvers */
void sa_solver_params_default(sa_solver_params *p);
/* FGMRESflex(A, m, eps, M, bit) / FGMRES<T>(A, m, eps, M) inside Restarted(dA, inner, max, eps)
 *                                   Library/solver/gmres.hpp:110-129, 192-211, 276-297;
 *                                   Library/solver/irsolver.hpp:50-57 */
int sa_solver_create(sa_ctx ctx, int precision, sa_mat dA, sa_mat A, sa_amg M, const sa_solver_params *p,
                     sa_solver *out);
int sa_solver_destroy(sa_solver S);
/* Restarted::Solve(b, nrm_b, x): returns iterations (0 if not converged, as
 * Converge.iter)                    Library/solver/irsolver.hpp:61-77 */
int sa_solver_solve(sa_solver S, const double *b, double nrm_b, double *x, int *iters, int *converged);
/* one inner FGMRES*::Solve(r, nrm_b, x) call.  e0: optional injected norm of r;
 * dumps: optional host buffers {V, Z, H, c, s, e, y} (integer solver)
 *                                   Library/solver/gmres.hpp:130-170, 212-252, 307-353 */
int sa_solver_cycle(sa_solver S, const double *r, double nrm_b, double *x, const double *e0, int *iters,
                    int *converged, void *const *dumps);
int sa_solver_set_bits(sa_solver S, int frac_bits);
int sa_solver_bits(sa_solver S, int *frac_bits);
/* per-iteration residual estimates and status flags of the last solve */
int sa_solver_history(sa_solver S, double *hist, int cap, int *n, unsigned *flags);

/* Work/main.cpp:153-161: one FP64 V-cycle on b, F = rule(max|c| / ||b||) */
int sa_rule_bits(sa_ctx ctx, sa_amg M_f64, const double *b, double nrm_b, int *frac_bits);
/* the same V-cycle; *ratio = max|c| / ||b||, the number the rule maps to F */
int sa_rule_ratio(sa_ctx ctx, sa_amg M_f64, const double *b, double nrm_b, double *ratio);

/* ------------------------------------------------ learned bit selector
 * No counterpart in the reference, which picks F by the rule above or by a
 * manual sweep (Work/sub.cpp:36-102).  A 3-layer FP32 MLP (n_in -> hidden ->
 * hidden -> n_out, ReLU) maps SA_NUM_FEATURES matrix features to a predicted
 * cost (log2 iterations) for each candidate F = f_lo + k; the selector takes
 * the argmin.  Training and inference run in this library's own CUDA kernels.
 * Arrays are row-major (one sample per row); host or device pointers. */
#define SA_NUM_FEATURES 20
typedef struct sa_mlp_net *sa_mlp;
/* features of an integer setup; ratio = sa_rule_ratio's value */
int sa_setup_features(sa_setup s_int, double ratio, float *feat);
int sa_mlp_create(sa_ctx ctx, int n_in, int hidden, int n_out, uint64_t seed, sa_mlp *out);
int sa_mlp_destroy(sa_mlp m);
/* flat parameters W1[h][in] b1[h] W2[h][h] b2[h] W3[out][h] b3[out] */
int sa_mlp_nparams(sa_mlp m, int64_t *n);
int sa_mlp_get_params(sa_mlp m, float *out);
int sa_mlp_set_params(sa_mlp m, const float *in);
/* input standardisation x -> (x - mu) / sd applied before the first layer */
int sa_mlp_set_norm(sa_mlp m, const float *mu, const float *sd);
int sa_mlp_predict(sa_ctx ctx, sa_mlp m, const float *X, int n, float *Y);
/* masked MSE loss sum M (Y - T)^2 / sum M over all n rows and its gradient
 * with respect to the flat parameters (no update) */
int sa_mlp_gradient(sa_ctx ctx, sa_mlp m, const float *X, const float *T, const float *M, int n, float *grad,
                    float *loss);
/* mini-batch Adam (lr, beta 0.9/0.999, eps 1e-8), rows shuffled per epoch by
 * seed; loss_hist[epoch] (optional) = mean batch loss */
int sa_mlp_train(sa_ctx ctx, sa_mlp m, const float *X, const float *T, const float *M, int n, int epochs,
                 int batch, float lr, uint64_t seed, float *loss_hist);
/* argmin over the predicted costs of one feature row: *bits = f_lo + k */
int sa_mlp_select_bits(sa_ctx ctx, sa_mlp m, const float *feat, int f_lo, int *frac_bits);

/* ------------------------------------------------------ batched solver
 * No counterpart in the reference, which solves one system per process.  Many
 * independent systems (already LMax1-scaled, uneven sizes), nrhs right-hand
 * sides each (1, 2 or 4), are set up with the multicolour SOR smoother and
 * solved together: every operation of the V-cycle and of FGMRESflex is one
 * launch over the whole batch, each Arnoldi step is one CUDA graph.  Per
 * system and right-hand side the integer arithmetic is that of the
 * single-system solver with a multicolour setup (sa_amg_params.multicolor = 1).
 * Vectors (b, x, precondition in/out) hold the systems' rows one after the
 * other (sa_batch_offsets) with the right-hand sides interleaved:
 * v[(offset[s] + i) * nrhs + r].  Per-pair arrays are indexed s * nrhs + r. */
typedef struct sa_batch_set *sa_batch;
/* threads: host threads for the per-system setup (0: all) */
int sa_batch_create(sa_ctx ctx, int nsys, const int *n, const int32_t *const *rptr, const int32_t *const *cind,
                    const double *const *val, int nrhs, const sa_amg_params *p, int threads, sa_batch *out);
int sa_batch_destroy(sa_batch B);
int sa_batch_info(sa_batch B, int *nsys, int *nrhs, int *depth_max, int64_t *rows);
/* offsets[nsys + 1]: first row of each system in the batch vectors */
int sa_batch_offsets(sa_batch B, int64_t *offsets);
/* the integer setup of one system (a new handle sharing the batch's arrays;
 * release it with sa_setup_destroy) */
int sa_batch_system_setup(sa_batch B, int sys, sa_setup *out);
/* intAMGflex::Precondition of every system and right-hand side at once */
int sa_batch_precondition(sa_ctx ctx, sa_batch B, const int32_t *in, int32_t *out);
/* time every candidate lanes-per-row value of each level operator and keep the fastest */
int sa_batch_autotune(sa_ctx ctx, sa_batch B, int reps);
/* rebuild every system's multicolour SOR split with other colour caps: caps[l]
 * for level l (the last for all deeper levels; 0 = a proper colouring), the
 * coarsening kept.  The greedy colouring (Library/helper/helper_graph.hpp:191-219)
 * stops after the cap and the rows left join their least conflicting colour
 * (their couplings inside it act Jacobi-like).  Launch shapes fall back to
 * their defaults (autotune again); results of earlier solves are unaffected.
 * No counterpart in the reference, which colours without a cap. */
int sa_batch_set_colour_caps(sa_ctx ctx, sa_batch B, int ncaps, const int *caps, int threads);
/* the cap in force per level: *ncaps = depth, caps[l] for l < min(cap, depth) */
int sa_batch_colour_caps(sa_batch B, int cap, int *ncaps, int *caps);
/* the chosen lanes per row of one operator (op: 0 A, 1 LD sweep, 2 U, 3 P, 4 R) */
int sa_batch_group(sa_batch B, int level, int op, int *group);
/* sets the lanes per row of one operator (1, 2, 4, 8, 16, 32; 0 = tile-staged
 * stream, not for op 1); results do not depend on it */
int sa_batch_set_group(sa_batch B, int level, int op, int group);
/* the colour sweep's launch form at one level: 0 one launch per colour, 1 one
 * thread-block-cluster launch, 2 the same over a packed copy of LD, 3 one
 * launch per colour over LD packed in colour order; set >= 0 chooses it
 * (SA_ERR_ARG / an error if the level lacks that form), -1 reads it; results
 * do not depend on it */
int sa_batch_sweep_form(sa_batch B, int level, int set, int *form);
/* compressed column storage of a level's A (op 0) or U (op 2): 16-bit offsets
 * column - row, 6 bytes an entry instead of 8, kept when every offset fits;
 * set 1 / 0 chooses it (SA_ERR_ARG / an error if the operator has none), -1
 * reads it; results do not depend on it (the autotuner chooses per operator) */
int sa_batch_compressed(sa_batch B, int level, int op, int set, int *on);
/* ELL copy of a level's A (op 0) or U (op 2), kept when its rows have at most
 * 8 entries and at most a quarter of the slots would be empty (the finest
 * level of a stencil matrix): slot-major, 16-bit column offsets, so a row's
 * entries need no row pointers (the reference prototypes the same idea as
 * SELL, spmat.hpp:208-281); set 1 / 0 chooses it (for the level-0 A also in
 * the Arnoldi SpMV), -1 reads; results do not depend on it (the autotuner
 * chooses) */
int sa_batch_ell(sa_batch B, int level, int op, int set, int *on);
/* sweeps of the levels below the finest whose multicolour split kept one
 * colour (LD is the diagonal: ldtri.hpp:172-183 without off-diagonal terms),
 * fused into the SpMVs around them: the pre-smoothing sweep into the
 * restriction that produces the level's e, the post-smoothing one into its U
 * residual; set 1 / 0 turns it on / off (default on), -1 reads; *levels = the
 * levels fused; results do not depend on it */
int sa_batch_fused_sweeps(sa_batch B, int set, int *levels);
/* the V-cycle's persistent coarse tail: set = t >= 1 runs levels t .. depth-1
 * and the coarsest LU solves in one cooperative launch (a grid barrier between
 * steps), 0 turns it off, -1 reads; *from = the tail's first level (0: none).
 * The autotuner picks t by V-cycle time; results do not depend on it */
int sa_batch_tail(sa_batch B, int set, int *from);
/* failure detection of the tail's grid barrier: one tail launch from `level`
 * whose first barrier waits for one CTA more than the grid has, so its wait
 * (bounded by timeout_ms, at most 2000) runs out; *status = the bits raised
 * (SA_FLAG_TIMEOUT expected).  The context stays usable; the batch's status
 * words and tail setting are restored */
int sa_batch_tail_selftest(sa_ctx ctx, sa_batch B, int level, double timeout_ms, unsigned *status);
/* Work/main.cpp:153-161 per system and right-hand side: max|M_f64 b| / ||b|| */
int sa_batch_rule_ratios(sa_ctx ctx, sa_batch B, const double *b, const double *nrm_b, double *ratio);
/* one operator of one batch level on interleaved vectors: op 0 A, 2 U, 3 P,
 * 4 R (y = M x), or op 1 the multicolour sweep (out = LD^-1 in; out is read
 * and written) */
int sa_batch_level_op(sa_ctx ctx, sa_batch B, int level, int op, const int32_t *in, int32_t *out);
/* the batched coarsest LU solve on the batch's own level vectors (for timing) */
int sa_batch_coarse_solve(sa_ctx ctx, sa_batch B);
/* milliseconds per call of one operator as the solver runs it (max(reps, 5)
 * calls captured in one CUDA graph when graphs are on, else reps calls on the
 * stream): op 0..4 as sa_batch_level_op, 5 the coarsest LU (in/out unused), 6
 * the whole V-cycle (level unused); the autotuner times its candidates so */
int sa_batch_time_op(sa_ctx ctx, sa_batch B, int level, int op, const int32_t *in, int32_t *out, int reps, float *ms);
/* the same with the L2 flushed (a buffer three times its size read) before
 * every call and the flush's own time subtracted: the call reads its operator
 * from HBM, as it does inside a V-cycle, which streams ~1 GB between two uses */
int sa_batch_time_op_cold(sa_ctx ctx, sa_batch B, int level, int op, const int32_t *in, int32_t *out, int reps,
                          float *ms);
/* rows, columns, entries and colour count of one batch level operator */
int sa_batch_level_info(sa_batch B, int level, int op, int *n, int *m, int64_t *nnz, int *ncolours);
/* Restarted(FGMRESflex) per pair; bits: F_G per system; nrm_b per pair;
 * iters / converged / final_bits (after overflow fallbacks) per pair, optional */
int sa_batch_solve(sa_ctx ctx, sa_batch B, const sa_solver_params *p, const int *bits, const double *b,
                   const double *nrm_b, double *x, int *iters, int *converged, int *final_bits);

/* ---------------------------------- floating-point siblings of a batch
 * FP64-AMG-FGMRES and FP32-mixed AMG-FGMRES of the same systems, set up from an
 * integer batch's coarsening and smoother parameters and run by the same
 * batched GPU design (one launch per operation over all systems, CUDA-graph
 * Arnoldi steps, programmatic dependent launch, autotuned lanes per row), so
 * that the integer solver can be compared with an FP64 solver on equal terms.
 * Per system: dfAMG<CSR<T>, SOR<ldtri::CSR<T>, CSR<T>>, T> in the multicolour
 * order of the integer batch's colouring (Library/preconditioner/INTAMG.hpp:13-134),
 * FGMRES<double> (Library/solver/gmres.hpp:19-98) or FGMRES<float>
 * (gmres.hpp:101-180), Restarted (Library/solver/irsolver.hpp:27-43).
 * Vectors are laid out as the integer batch's; precondition in/out are
 * double (SA_F64) or float (SA_F32); b and x are double. */
typedef struct sa_batch_fp_set *sa_batch_fp;
/* precision: SA_F64 or SA_F32; threads: host threads for the per-system
 * dfAMG setups (0: all).  The integer batch must outlive the handle. */
int sa_batch_fp_create(sa_ctx ctx, sa_batch B, int precision, int threads, sa_batch_fp *out);
int sa_batch_fp_destroy(sa_batch_fp F);
/* dfAMG::Precondition (INTAMG.hpp:86-134) of every system and right-hand side */
int sa_batch_fp_precondition(sa_ctx ctx, sa_batch_fp F, const void *in, void *out);
/* lanes per row of each operator and the sweep form of each level, timed */
int sa_batch_fp_autotune(sa_ctx ctx, sa_batch_fp F, int reps);
/* milliseconds per V-cycle as the solver runs it */
int sa_batch_fp_time_vcycle(sa_ctx ctx, sa_batch_fp F, int reps, float *ms);
/* as sa_batch_fused_sweeps for the floating-point engine (default on) */
int sa_batch_fp_fused_sweeps(sa_batch_fp F, int set, int *levels);
/* Restarted(FGMRES<T>) per pair; nrm_b per pair; iters / converged per pair (optional) */
int sa_batch_fp_solve(sa_ctx ctx, sa_batch_fp F, const sa_solver_params *p, const double *b, const double *nrm_b,
                      double *x, int *iters, int *converged);
/* restart cycles of the last sa_batch_solve (F null) or sa_batch_fp_solve (B
 * null) that ran as one graph each (SA_OPT_CYCLE_GRAPH; 0 when the engine fell
 * back to one graph per step, e.g. where the driver refuses conditional nodes) */
int sa_batch_cycle_graphs(sa_batch B, sa_batch_fp F, int *cycles);

/* start (on = 1) or stop (0) the profiler's collection range: a profiler
 * started with collection off records only the launches in between */
int sa_profiler_range(int on);

#ifdef __cplusplus
}
#endif
#endif
