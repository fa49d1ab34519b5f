// Internal declarations shared by the CUDA translation units and the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "host/amg_setup.hpp"
#include "host/batch_setup.hpp"
#include "host/csr.hpp"
#include "host/schedule.hpp"

namespace sagb {

enum VType : int { VT_I32 = 0, VT_F64 = 1, VT_F32 = 2 };

inline size_t vt_size(int vt) { return vt == VT_F64 ? 8 : 4; }

struct CudaError {
    std::string msg;
};
void cuda_check(cudaError_t e, const char *what);
#define SAGB_CUDA(call) ::sagb::cuda_check((call), #call)

// One GPU, one stream.  All kernels of a context run on `stream`.
struct Ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    unsigned *d_flags = nullptr;     // device status bits (ST_* in common.cuh) of the current launches
    unsigned *d_flags_main = nullptr;  // word 0: everything outside the preconditioner
    unsigned *d_flags_prec = nullptr;  // word 1: the V-cycle's kernels (see PrecFlags)
    unsigned *h_flags = nullptr;     // pinned mirror
    bool fp_exact = false;           // FP kernels in sequential order without FMA
    bool use_graphs = true;
    bool use_pdl = true;             // batched V-cycle kernels chained by programmatic dependent launch
    bool cycle_graph = true;         // batched engines: a restart cycle as one graph, steps gated on the device
    int gpu_setup_rows = 1 << 20;    // batches: systems from this size on build their Ruge-Stueben chain
                                     // on the GPU (0: none); smaller ones share the host threads
    long long launches = 0;          // kernels launched by this context (for reporting)
    // device copies of a call's host arguments, kept between calls (grow-only;
    // calls on a context do not overlap): allocating and freeing them per call
    // cost more than the copies
    void *stage[2] = {nullptr, nullptr};
    size_t stage_cap[2] = {0, 0};
    int stage_used = 0;
    std::string err;
};

// While alive, kernels launched on the context report into the preconditioner's
// status word.  FGMRES is flexible: a wrapped value inside the V-cycle gives a
// different (poorer) direction Z_j but leaves the Arnoldi relation A Z = V H
// exact, so the solvers report such overflow (SA_FLAG_PRECOND_OVERFLOW) and
// keep going, while overflow in A Z_j, the Gram-Schmidt sums or the Givens step
// discards the cycle.
// The Ruge-Stueben chain (host rs_chain) with the strength split, transposes,
// interpolation and Galerkin products on the context's GPU and the C/F
// splitting on the host; bit for bit the host chain (cuda/rs_setup.cu).
struct RsChain;
struct CsrD;
RsChain rs_chain_gpu(Ctx &c, const CsrD &A, double theta, int max_levels, int coarse_size);

struct PrecFlags {
    Ctx &c;
    unsigned *saved;
    explicit PrecFlags(Ctx &ctx) : c(ctx), saved(ctx.d_flags) { c.d_flags = c.d_flags_prec; }
    ~PrecFlags() { c.d_flags = saved; }
};

void *dmalloc(size_t bytes);
void dfree(void *p);
template <typename T>
T *dupload(const std::vector<T> &v) {
    if (v.empty()) return nullptr;
    T *p = (T *)dmalloc(v.size() * sizeof(T));
    SAGB_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

// ------------------------------------------------------------------ matrices
struct DevCsr {
    int n = 0, m = 0;
    int64_t nnz = 0;
    int bit = 0;
    int vt = VT_I32;
    int group = 1;  // lanes per row in the SpMV kernel
    int *rptr = nullptr, *cind = nullptr;
    void *val = nullptr;
    void release();
};

DevCsr upload_csr_i32(const CsrI &A);
template <typename T>
DevCsr upload_csr_fp(const CsrT<T> &A);
DevCsr upload_csr_f64(const CsrD &A);
int pick_group(double avg_nnz_per_row);

// SpMV modes
enum SpmvMode : int {
    SPMV_SET = 0,    // y = A x
    SPMV_RESID = 1,  // y = z - A x
    SPMV_ADD = 2,    // y = A x + y
};
void spmv(Ctx &c, const DevCsr &A, const void *x, void *y, int mode = SPMV_SET, const void *z = nullptr);
// FP64 residual in the reference's row order without contraction (bit-exact with
// the CPU): r = b - A x  (irsolver.hpp:66-67)
void spmv_resid_f64_exact(Ctx &c, const DevCsr &A, const double *x, const double *b, double *r);

// ------------------------------------------------------ triangular sweeps
struct TriSync {
    unsigned ticket, done, epoch, pad;
};

struct DevTri {
    int n = 0, kind = 0, vt = VT_I32;
    int bit = 0, dbit = 0;
    int nchunks = 0, group = 1, grid = 0;
    int nlev = 0, max_level_rows = 0;
    int64_t nnz_off = 0;
    int *perm = nullptr, *prp = nullptr, *pci = nullptr;
    void *pval = nullptr, *dinv = nullptr;
    int *chunk_lv = nullptr, *sub_bound = nullptr;
    unsigned long long *pk = nullptr;  // packed {epoch, value} per row (int32 / f32)
    unsigned *flag = nullptr;          // ready epoch per row (f64)
    TriSync *sync = nullptr;
    // single-CTA mode: the result vector in shared memory, each level's row
    // data in one 16-byte aligned block fetched ahead by bulk copies
    bool one_cta = false;
    unsigned char *blocks = nullptr;
    unsigned *blk_off = nullptr;       // offset of each level's block in 16-byte units (nlev + 1), then
                                       // the rows of each level (nlev)
    int stage_bytes = 0;               // bytes of the single-CTA kernel's bulk-copy ring
    size_t cta_smem = 0;
    void release();
};

// Builds the schedule from a triangular CSR (kind: TRI_LD / TRI_L / TRI_DU) and
// uploads it.  vals points at int32 / double / float values of the source CSR.
// level_hint (optional): the level of each row (colours of a multicolour split).
DevTri upload_tri(const Ctx &c, int n, const int *rptr, const int *cind, const void *vals, int vt, int kind,
                  int bit, int dbit, const int *level_hint = nullptr);
void trsv(Ctx &c, const DevTri &T, const void *in, void *out);
// the same sweep with its scratch in a static device array (no allocation)
void trsv_noalloc(Ctx &c, const DevTri &T, const void *in, void *out);

// Dense coarsest-level LU: strict lower L (unit), strict upper U and D^-1,
// row-major n x n, solved by one block.
struct DevDenseLU {
    int n = 0, vt = VT_I32;
    int bitL = 0, bitU = 0, dbitU = 0;
    void *L = nullptr, *U = nullptr, *dinv = nullptr;
    void *tmp = nullptr;
    void release();
};
DevDenseLU upload_dense_lu(const int *Lrptr, const int *Lcind, const void *Lval, const int *Urptr,
                           const int *Ucind, const void *Uval, int n, int vt, int bitL, int bitU, int dbitU);
void lu_solve(Ctx &c, const DevDenseLU &LU, const void *in, void *out);
void init_kernel_attributes();

// ------------------------------------------------------------------- AMG
struct DevAmg {
    int vt = VT_I32;
    int depth = 0;
    int smooth_iter = 1;
    int nbj = 0;
    DevCsr A0;
    std::vector<DevCsr> CA, P, R, U;
    std::vector<DevTri> LD;
    DevDenseLU LU;
    void *r = nullptr;                   // fine-level residual / prolongation buffer
    std::vector<void *> rr, ee, xx, tmp; // per coarse level (tmp: per smoother level)
    // host copies kept for export and inspection
    std::shared_ptr<IntHierarchy> hi;
    std::shared_ptr<FpHierarchy<double>> hd;
    std::shared_ptr<FpHierarchy<float>> hf;
    void release();
};

std::unique_ptr<DevAmg> upload_amg_int(Ctx &c, std::shared_ptr<IntHierarchy> h);
std::unique_ptr<DevAmg> upload_amg_f64(Ctx &c, std::shared_ptr<FpHierarchy<double>> h);
std::unique_ptr<DevAmg> upload_amg_f32(Ctx &c, std::shared_ptr<FpHierarchy<float>> h);
void smooth(Ctx &c, DevAmg &M, int level, const void *in, void *out, bool inited);
void vcycle(Ctx &c, DevAmg &M, const void *in, void *out);

// --------------------------------------------------------------- elementwise
void vec_sub(Ctx &c, int vt, int n, const void *x, void *y);  // y = x - y
void vec_add(Ctx &c, int vt, int n, const void *x, void *y);  // y = x + y

// ----------------------------------------------------------------- Krylov
struct SolveStats {
    int iters = 0;
    int converged = 0;
    int restarts = 0;
    int fallbacks = 0;
    int final_bit = 0;
    double explicit_res = 0;
    unsigned flags = 0;
    double seconds = 0;
    std::vector<double> history;  // per inner iteration relative residual estimate
};

struct KrylovParams {
    int m = 30;
    double eps = 1e-10;
    int max_outer = 33;
    int bit = 29;
    int verbose = 0;
    int fallback = 1;  // int: on overflow, discard the cycle and redo it with bit - 1
    int explicit_check = 0;  // stop on the explicit FP64 residual instead of the inner estimate
    int cycle_bits = 0;      // batched int: end a cycle once |e_{j+1}| <= 2^(F - cycle_bits) (0: full cycles)
};

class Solver;
std::unique_ptr<Solver> make_solver(Ctx &c, int vt, const DevCsr *dA, const DevCsr *A, DevAmg *M,
                                    const KrylovParams &p);
class Solver {
  public:
    virtual ~Solver() {}
    // Restarted::Solve (irsolver.hpp:61-77); b, x device pointers
    virtual int solve(const double *b, double nrm_b, double *x, SolveStats &st) = 0;
    // one inner cycle (FGMRES*::Solve) on a device residual r; e0: optional
    // injected norm; dumps: optional host buffers for V,Z,H,c,s,e,y
    virtual int cycle(const double *r, double nrm_b, double *x, const double *e0, int *converged,
                      void *const *dumps) = 0;
    virtual void set_bit(int bit) = 0;
};

// FP64 norm of a device vector (deterministic reduction order)
double nrm2_f64(Ctx &c, const double *x, int n);
void nrm2_f64_dev(Ctx &c, const double *x, int n, double *d_out);

// ------------------------------------------------------------ batched solver
struct BatchStats {
    std::vector<int> iters, converged, fallbacks, final_bit;  // per pair (system * nrhs + rhs)
    std::vector<double> explicit_res;
    int restarts = 0;
    unsigned flags = 0;
    int cycle_graphs = 0;  // restart cycles that ran as one graph (no host round trip per step)
};

// The FP64 / FP32-mixed sibling of an integer batch (cuda/batch_fp.cu): the
// same systems, coarsening, level order and colour caps; vectors of T.
class BatchFpEngine {
  public:
    BatchFpEngine(Ctx &c, std::shared_ptr<BatchHierarchy> h, int vt, int nrhs, int threads = 0);
    ~BatchFpEngine();
    int precision() const { return vt_; }
    size_t rows() const;
    int depth() const;
    void precondition(const void *in, void *out);  // device pointers of the engine's type
    // b, x: device (double); nrm_b: per pair (host or device)
    void solve(const KrylovParams &kp, const double *b, const double *nrm_b, double *x, BatchStats &st);
    void autotune(int reps);
    float time_vcycle(int reps);
    // sweeps of one-colour levels fused into the neighbouring SpMVs: set 1 /
    // 0 / -1 (read); returns the levels fused
    int fused_sweeps(int set);
    int last_cycle_graphs() const { return last_cycle_graphs_; }
    class Base;

  private:
    int vt_;
    int last_cycle_graphs_ = 0;
    std::unique_ptr<Base> impl_;
};

// Many systems, nrhs right-hand sides each, solved together (cuda/batch.cu).
// Vectors are level-0 rows with the right-hand sides interleaved.
class BatchEngine {
  public:
    BatchEngine(Ctx &c, std::shared_ptr<BatchHierarchy> h, int nrhs);
    ~BatchEngine();
    int nrhs() const;
    size_t rows() const;
    int depth() const;
    void precondition(const int *in, int *out);  // device pointers
    void pair_norms(const double *v, double *out);
    // b, x: device; nrm_b: per pair (host or device); bits_sys: host, per system
    void solve(const KrylovParams &kp, const int *bits_sys, const double *b, const double *nrm_b, double *x,
               BatchStats &st);
    int last_cycle_graphs() const { return last_cycle_graphs_; }  // of the last solve
    void autotune(int reps);
    void set_groups(int level, int op, int group);  // op: 0 A, 1 LD, 2 U, 3 P, 4 R
    int group(int level, int op) const;
    // the colour sweep's form at one level (0: a launch per colour, 1: cluster
    // launch, 2: packed cluster launch, 3: a launch per colour over LD packed
    // in colour order); set >= 0 chooses it, -1 only reads
    int sweep_form(int level, int set);
    // 16-bit column offsets for A (op 0) or U (op 2) of one level: set 1 / 0
    // chooses them (1 needs offsets that fit), -1 only reads
    int compressed(int level, int op, int set);
    // the ELL copy of a level's A (op 0) or U (op 2), where it has one: set 1 /
    // 0 chooses it (for the level-0 A also in the Arnoldi SpMV), -1 reads
    int ell(int level, int op, int set);
    // sweeps of one-colour levels fused into the neighbouring SpMVs: set 1 / 0
    // turns it on / off, -1 reads; returns the levels whose sweeps are fused
    int fused_sweeps(int set);
    // the V-cycle's persistent coarse tail: set t >= 1 runs levels t .. Dmax-1
    // and the coarsest LU in one cooperative launch, 0 turns it off, -1 reads;
    // returns the first level of the tail (0: none); grid > 0: that many CTAs
    int tail(int set, int grid = 0);
    // failure detection of the tail's bounded grid barrier: one tail launch
    // from `level` whose first barrier can never complete; returns the status
    // bits it raised (ST_TIMEOUT when the wait ran out after timeout_ms and
    // every CTA returned).  The engine's status words and tail are restored.
    unsigned tail_selftest(int level, double timeout_ms);
    // one operator of one level on caller vectors (op 1: the colour sweep LD^-1 in)
    void level_op(int level, int op, const int *in, int *out);
    void coarse_solve();  // the batched LU on the engine's own level vectors
    // milliseconds per call as the solver runs it (inside a CUDA graph when
    // graphs are on): op 0..4 as level_op, 5 the coarsest LU, 6 the V-cycle
    // cold: the L2 flushed before every call (the flush's own time subtracted)
    float time_op(int level, int op, const int *in, int *out, int reps, bool cold = false);
    void level_info(int level, int op, int *n, int *m, int64_t *nnz, int *ncolours) const;

  private:
    struct Impl;
    Impl *impl_;
    int last_cycle_graphs_ = 0;
};

// ------------------------------------------------------ learned bit selector
// 3-layer FP32 MLP (nin -> hid -> hid -> nout, ReLU on the hidden layers),
// trained with a masked MSE loss and Adam.  Inputs are standardised on the
// device with (x - mu) / sd.  Host pointers or device pointers are accepted.
struct Mlp {
    int nin, hid, nout;
    float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // params, grads, Adam moments
    float *norm = nullptr;                                            // mu[nin], sd[nin]
    float *ws = nullptr;                                              // per-batch activations
    int ws_batch = 0;
    float *data = nullptr;  // loaded X, T, M
    int data_n = 0, loaded_n = 0;
    int *perm_d = nullptr;
    long long t = 0;  // Adam step
    Mlp(int in, int hidden, int out, uint64_t seed);
    ~Mlp();
    size_t off_w1() const { return 0; }
    size_t off_b1() const { return off_w1() + (size_t)hid * nin; }
    size_t off_w2() const { return off_b1() + hid; }
    size_t off_b2() const { return off_w2() + (size_t)hid * hid; }
    size_t off_w3() const { return off_b2() + hid; }
    size_t off_b3() const { return off_w3() + (size_t)nout * hid; }
    size_t nparams() const { return off_b3() + nout; }
    void set_norm(const float *mu, const float *sd);
    void predict(Ctx &c, const float *X, int n, float *Y);
    // loss and flat gradient of the whole set as one batch (no update)
    float gradient(Ctx &c, const float *X, const float *T, const float *M, int n, float *grad);
    // mini-batch Adam; loss_hist[epoch] = mean batch loss of that epoch
    void train(Ctx &c, const float *X, const float *T, const float *M, int n, int epochs, int batch, float lr,
               uint64_t seed, float *loss_hist);
    void get_params(float *out) const;
    void set_params(const float *in);

  private:
    void reserve(int B);
    void load(Ctx &c, const float *X, const float *T, const float *M, int n);
    void gather(Ctx &c, const int *perm, int off, int B, bool targets);
    void forward_batch(Ctx &c, int B);
    void backward_batch(Ctx &c, int B);
    float *loss_slot();
};

}  // namespace sagb
