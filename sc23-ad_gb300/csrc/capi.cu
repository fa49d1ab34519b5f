// C ABI (include/sagb.h) over the host setup and the CUDA kernels.
#include <cuda_profiler_api.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>

#include "../../include/sagb.h"
#include "cuda/common.cuh"
#include "host/features.hpp"
#include "host/generators.hpp"
#include "sagb_internal.hpp"

using namespace sagb;

static thread_local std::string g_err;

static int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

#define SA_GUARD_BEGIN try {
#define SA_GUARD_END                                                      \
    }                                                                     \
    catch (const CudaError &e) {                                          \
        return fail(SA_ERR_CUDA, e.msg);                                  \
    }                                                                     \
    catch (const SetupError &e) {                                         \
        return fail(SA_ERR_SETUP, e.msg);                                 \
    }                                                                     \
    catch (const std::bad_alloc &) {                                      \
        return fail(SA_ERR_SETUP, "host allocation failed");              \
    }                                                                     \
    catch (const std::exception &e) {                                     \
        return fail(SA_ERR_ARG, e.what());                                \
    }

struct sa_context {
    Ctx c;
};
struct sa_matrix {
    sa_context *ctx;
    DevCsr d;
    int precision;
};
struct sa_hierarchy {
    int precision = SA_INT;
    sa_amg_params p{};
    std::vector<int> level_caps;     // multicolour caps per level (a batch's tuned caps), overriding p's
    std::shared_ptr<CsrD> A;         // the scaled fine matrix
    std::shared_ptr<RsChain> chain;  // coarsening shared by all precisions
    std::shared_ptr<IntHierarchy> hi;
    std::shared_ptr<FpHierarchy<double>> hd;
    std::shared_ptr<FpHierarchy<float>> hf;
};
struct sa_multigrid {
    sa_context *ctx;
    std::unique_ptr<DevAmg> M;
    int precision;
};
struct sa_krylov {
    sa_context *ctx;
    int precision;
    sa_solver_params p;
    std::unique_ptr<Solver> S;
    DevCsr *dA;
    int N;
    double *db = nullptr, *dx = nullptr;  // staging for host b / x
    SolveStats last;
};
struct sa_host_csr {
    CsrD A;
};
struct sa_timer {
    cudaEvent_t e;
};
struct sa_mlp_net {
    std::unique_ptr<Mlp> net;
};
struct sa_batch_set {
    sa_context *ctx;
    sa_amg_params p;
    std::shared_ptr<BatchHierarchy> h;
    std::unique_ptr<BatchEngine> eng;
};
struct sa_batch_fp_set {
    std::shared_ptr<BatchHierarchy> h;
    int nrhs = 1;
    std::unique_ptr<BatchFpEngine> eng;
};

// ------------------------------------------------------------------ helpers

static bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// A device view of a caller buffer: device pointers pass through, host
// buffers are copied in (and, for outputs, back out at the end).
class Staged {
  public:
    Staged(Ctx &c, const void *p, size_t bytes, bool in, bool out) : c_(c), user_(const_cast<void *>(p)),
                                                                       bytes_(bytes), out_(out) {
        if (is_device_ptr(p)) {
            dev_ = user_;
        } else {
            const int slot = c.stage_used;
            void *buf = nullptr;
            if (slot < 2) {  // the context's kept buffer for this argument
                if (c.stage_cap[slot] < bytes) {
                    cudaStreamSynchronize(c.stream);
                    dfree(c.stage[slot]);
                    c.stage[slot] = nullptr;
                    c.stage_cap[slot] = 0;
                    c.stage[slot] = dmalloc(bytes);
                    c.stage_cap[slot] = bytes;
                }
                buf = c.stage[slot];
            } else {
                buf = dmalloc(bytes);
                own_ = buf;
            }
            if (in) {
                const cudaError_t e = cudaMemcpyAsync(buf, p, bytes, cudaMemcpyHostToDevice, c.stream);
                if (e != cudaSuccess) {
                    dfree(own_);
                    own_ = nullptr;
                    SAGB_CUDA(e);
                }
            }
            dev_ = buf;
            if (slot < 2) {  // in use until this object goes
                slot_ = slot;
                c.stage_used++;
            }
        }
    }
    ~Staged() {
        if (dev_ && dev_ != user_) {
            cudaStreamSynchronize(c_.stream);
            if (slot_ >= 0) c_.stage_used--;
            else dfree(own_);
        }
    }
    // Host outputs are copied back and the stream is synchronised; with device
    // buffers only, the call stays asynchronous on the context's stream.
    void finish() {
        if (!dev_ || dev_ == user_) return;
        if (out_) SAGB_CUDA(cudaMemcpyAsync(user_, dev_, bytes_, cudaMemcpyDeviceToHost, c_.stream));
        SAGB_CUDA(cudaStreamSynchronize(c_.stream));
    }
    void *get() const { return dev_; }

  private:
    Ctx &c_;
    void *user_, *dev_ = nullptr, *own_ = nullptr;
    size_t bytes_;
    bool out_;
    int slot_ = -1;  // the context's kept buffer in use, or -1 (an allocation of this call)
};

// ---------------------------------------------------------------- library

extern "C" const char *sa_version(void) { return "sagb 0.1 (sm_103a)"; }
extern "C" const char *sa_last_error(void) { return g_err.c_str(); }

extern "C" int sa_ctx_create(int device, sa_ctx *out) {
    if (!out) return fail(SA_ERR_ARG, "null output");
    SA_GUARD_BEGIN
    int ndev = 0;
    SAGB_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(SA_ERR_ARG, "no such device");
    SAGB_CUDA(cudaSetDevice(device));
    auto *h = new sa_context();
    h->c.device = device;
    SAGB_CUDA(cudaDeviceGetAttribute(&h->c.num_sms, cudaDevAttrMultiProcessorCount, device));
    SAGB_CUDA(cudaStreamCreateWithFlags(&h->c.stream, cudaStreamNonBlocking));
    h->c.d_flags = (unsigned *)dmalloc(sizeof(unsigned) * 4);
    SAGB_CUDA(cudaMemset(h->c.d_flags, 0, sizeof(unsigned) * 4));
    h->c.d_flags_main = h->c.d_flags;
    h->c.d_flags_prec = h->c.d_flags + 1;
    SAGB_CUDA(cudaMallocHost(&h->c.h_flags, sizeof(unsigned) * 4));
    init_kernel_attributes();
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_ctx_destroy(sa_ctx ctx) {
    if (!ctx) return SA_OK;
    cudaStreamSynchronize(ctx->c.stream);
    dfree(ctx->c.stage[0]);
    dfree(ctx->c.stage[1]);
    dfree(ctx->c.d_flags_main);
    cudaFreeHost(ctx->c.h_flags);
    cudaStreamDestroy(ctx->c.stream);
    delete ctx;
    return SA_OK;
}

extern "C" int sa_ctx_set_option(sa_ctx ctx, int option, int value) {
    if (!ctx) return fail(SA_ERR_ARG, "null context");
    if (option == SA_OPT_FP_EXACT) ctx->c.fp_exact = value != 0;
    else if (option == SA_OPT_GRAPHS) ctx->c.use_graphs = value != 0;
    else if (option == SA_OPT_PDL) ctx->c.use_pdl = value != 0;
    else if (option == SA_OPT_CYCLE_GRAPH) ctx->c.cycle_graph = value != 0;
    else if (option == SA_OPT_GPU_SETUP) ctx->c.gpu_setup_rows = value == 1 ? 1 << 20 : value < 0 ? 0 : value;
    else return fail(SA_ERR_ARG, "unknown option");
    return SA_OK;
}

extern "C" int sa_ctx_flags(sa_ctx ctx, unsigned *flags, int clear) {
    if (!ctx) return fail(SA_ERR_ARG, "null context");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaMemcpyAsync(ctx->c.h_flags, ctx->c.d_flags_main, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost,
                              ctx->c.stream));
    SAGB_CUDA(cudaStreamSynchronize(ctx->c.stream));
    // word 1 (the V-cycle's kernels): an int32 wrap there is SA_FLAG_PRECOND_OVERFLOW
    const unsigned w1 = ctx->c.h_flags[1];
    if (flags) *flags = ctx->c.h_flags[0] | (w1 & ~ST_OVERFLOW) | ((w1 & ST_OVERFLOW) ? ST_PREC_OVF : 0u);
    if (clear) {
        SAGB_CUDA(cudaMemsetAsync(ctx->c.d_flags_main, 0, 2 * sizeof(unsigned), ctx->c.stream));
        SAGB_CUDA(cudaStreamSynchronize(ctx->c.stream));
    }
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_ctx_launches(sa_ctx ctx, long long *count) {
    if (!ctx || !count) return fail(SA_ERR_ARG, "null argument");
    *count = ctx->c.launches;
    return SA_OK;
}

extern "C" int sa_ctx_sync(sa_ctx ctx) {
    if (!ctx) return fail(SA_ERR_ARG, "null context");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaStreamSynchronize(ctx->c.stream));
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_ctx_stream(sa_ctx ctx, void **stream) {
    if (!ctx || !stream) return fail(SA_ERR_ARG, "null argument");
    *stream = (void *)ctx->c.stream;
    return SA_OK;
}

extern "C" int sa_device_alloc(sa_ctx ctx, uint64_t bytes, void **ptr) {
    if (!ctx || !ptr) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    *ptr = dmalloc(bytes);
    return SA_OK;
    SA_GUARD_END
}
extern "C" int sa_device_free(sa_ctx ctx, void *ptr) {
    (void)ctx;
    dfree(ptr);
    return SA_OK;
}
extern "C" int sa_memcpy(sa_ctx ctx, void *dst, const void *src, uint64_t bytes) {
    if (!ctx) return fail(SA_ERR_ARG, "null context");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->c.stream));
    SAGB_CUDA(cudaStreamSynchronize(ctx->c.stream));
    return SA_OK;
    SA_GUARD_END
}
extern "C" int sa_host_alloc(uint64_t bytes, void **ptr) {
    if (!ptr) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaMallocHost(ptr, bytes ? bytes : 16));
    return SA_OK;
    SA_GUARD_END
}
extern "C" int sa_host_free(void *ptr) {
    if (ptr) cudaFreeHost(ptr);
    return SA_OK;
}
extern "C" int sa_event_create(sa_event *out) {
    if (!out) return fail(SA_ERR_ARG, "null output");
    SA_GUARD_BEGIN
    auto *t = new sa_timer();
    SAGB_CUDA(cudaEventCreate(&t->e));
    *out = t;
    return SA_OK;
    SA_GUARD_END
}
extern "C" int sa_event_record(sa_ctx ctx, sa_event ev) {
    if (!ctx || !ev) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaEventRecord(ev->e, ctx->c.stream));
    return SA_OK;
    SA_GUARD_END
}
extern "C" int sa_event_elapsed_ms(sa_event a, sa_event b, float *ms) {
    if (!a || !b || !ms) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaEventSynchronize(b->e));
    SAGB_CUDA(cudaEventElapsedTime(ms, a->e, b->e));
    return SA_OK;
    SA_GUARD_END
}
extern "C" int sa_event_destroy(sa_event ev) {
    if (ev) {
        cudaEventDestroy(ev->e);
        delete ev;
    }
    return SA_OK;
}

// ------------------------------------------------------------ host CSR

extern "C" int sa_hcsr_read_mm(const char *path, sa_hcsr *out) {
    if (!path || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    auto *h = new sa_host_csr();
    h->A = read_matrix_market(path);
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_hcsr_read_mm_cached(const char *mm_path, const char *cache_path, sa_hcsr *out) {
    if (!mm_path || !cache_path || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    auto *h = new sa_host_csr();
    try {
        h->A = read_matrix_market_cached(mm_path, cache_path);
    } catch (...) {
        delete h;
        throw;
    }
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_hcsr_save(sa_hcsr A, const char *path) {
    if (!A || !path) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    write_csr_binary(A->A, path);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_hcsr_load(const char *path, sa_hcsr *out) {
    if (!path || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    auto *h = new sa_host_csr();
    if (!read_csr_binary(path, h->A, nullptr, nullptr)) {
        delete h;
        return fail(SA_ERR_ARG, std::string("not a valid CSR file: ") + path);
    }
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

static int check_csr(int n, int m, const int32_t *rptr, const int32_t *cind) {
    if (n < 0 || m < 0 || !rptr || (!cind && n > 0 && rptr[n] > 0)) return fail(SA_ERR_ARG, "invalid CSR");
    if (rptr[0] != 0) return fail(SA_ERR_ARG, "rptr[0] must be 0");
    for (int i = 0; i < n; i++) {
        if (rptr[i + 1] < rptr[i]) return fail(SA_ERR_ARG, "rptr not monotone");
        for (int j = rptr[i]; j < rptr[i + 1]; j++)
            if (cind[j] < 0 || cind[j] >= m) return fail(SA_ERR_ARG, "column index out of range");
    }
    return SA_OK;
}

extern "C" int sa_hcsr_create(int n, int m, const int32_t *rptr, const int32_t *cind, const double *val,
                              sa_hcsr *out) {
    if (!out) return fail(SA_ERR_ARG, "null output");
    if (int e = check_csr(n, m, rptr, cind)) return e;
    SA_GUARD_BEGIN
    auto *h = new sa_host_csr();
    h->A.n = n;
    h->A.m = m;
    h->A.rptr.assign(rptr, rptr + n + 1);
    h->A.cind.assign(cind, cind + rptr[n]);
    h->A.val.assign(val, val + rptr[n]);
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_hcsr_view(sa_hcsr A, sa_csr_view *out) {
    if (!A || !out) return fail(SA_ERR_ARG, "null argument");
    out->n = A->A.n;
    out->m = A->A.m;
    out->nnz = A->A.nnz();
    out->rptr = A->A.rptr.data();
    out->cind = A->A.cind.data();
    out->val = A->A.val.data();
    out->bit = out->dbit = 0;
    return SA_OK;
}

extern "C" int sa_hcsr_lmax1_scaling(sa_hcsr A, double *b) {
    if (!A) return fail(SA_ERR_ARG, "null matrix");
    lmax1_scaling(A->A, b);
    return SA_OK;
}

extern "C" int sa_hcsr_rhs(sa_hcsr A, uint64_t seed, double *xstar, double *b) {
    if (!A || !xstar || !b) return fail(SA_ERR_ARG, "null argument");
    gen_rhs(A->A, seed, xstar, b);
    return SA_OK;
}

extern "C" int sa_hcsr_destroy(sa_hcsr A) {
    delete A;
    return SA_OK;
}

extern "C" int sa_gen(int kind, int nx, double param, uint64_t seed, sa_hcsr *out) {
    if (!out || nx <= 0) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    auto *h = new sa_host_csr();
    switch (kind) {
        case SA_GEN_POISSON2D: h->A = gen_poisson2d(nx); break;
        case SA_GEN_POISSON3D: h->A = gen_poisson3d(nx); break;
        case SA_GEN_ANISO2D: h->A = gen_aniso2d(nx, param); break;
        case SA_GEN_STENCIL27: h->A = gen_stencil27(nx, seed); break;
        case SA_GEN_CONVDIFF3D: h->A = gen_convdiff3d(nx, param); break;
        case SA_GEN_VARCOEF3D: h->A = gen_varcoef3d(nx, param, seed); break;
        default: delete h; return fail(SA_ERR_ARG, "unknown generator");
    }
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

// -------------------------------------------------------------- matrices

extern "C" int sa_mat_create(sa_ctx ctx, int kind, int bit, int n, int m, const int32_t *rptr,
                             const int32_t *cind, const double *val, sa_mat *out) {
    if (!ctx || !out) return fail(SA_ERR_ARG, "null argument");
    if (int e = check_csr(n, m, rptr, cind)) return e;
    if (kind == SA_MAT_FIXED && (bit < 0 || bit > 30)) return fail(SA_ERR_ARG, "bit must be in [0, 30]");
    SA_GUARD_BEGIN
    CsrD A;
    A.n = n;
    A.m = m;
    A.rptr.assign(rptr, rptr + n + 1);
    A.cind.assign(cind, cind + rptr[n]);
    A.val.assign(val, val + rptr[n]);
    auto *h = new sa_matrix();
    h->ctx = ctx;
    if (kind == SA_MAT_FIXED || kind == SA_MAT_FLEX) {
        h->d = upload_csr_i32(kind == SA_MAT_FIXED ? to_fixed(A, bit) : to_flex(A));
        h->precision = SA_INT;
    } else if (kind == SA_MAT_F64) {
        h->d = upload_csr_f64(A);
        h->precision = SA_F64;
    } else if (kind == SA_MAT_F32) {
        CsrT<float> F;
        F.n = n;
        F.m = m;
        F.rptr = A.rptr;
        F.cind = A.cind;
        F.val.resize(A.val.size());
        for (size_t j = 0; j < A.val.size(); j++) F.val[j] = (float)A.val[j];
        h->d = upload_csr_fp<float>(F);
        h->precision = SA_F32;
    } else {
        delete h;
        return fail(SA_ERR_ARG, "unknown matrix kind");
    }
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mat_create_i32(sa_ctx ctx, int n, int m, const int32_t *rptr, const int32_t *cind,
                                 const int32_t *val, int bit, sa_mat *out) {
    if (!ctx || !out) return fail(SA_ERR_ARG, "null argument");
    if (int e = check_csr(n, m, rptr, cind)) return e;
    if (bit < 0 || bit > 62) return fail(SA_ERR_ARG, "bit out of range");
    SA_GUARD_BEGIN
    CsrI A;
    A.n = n;
    A.m = m;
    A.bit = bit;
    A.rptr.assign(rptr, rptr + n + 1);
    A.cind.assign(cind, cind + rptr[n]);
    A.val.assign(val, val + rptr[n]);
    auto *h = new sa_matrix();
    h->ctx = ctx;
    h->d = upload_csr_i32(A);
    h->precision = SA_INT;
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mat_destroy(sa_mat A) {
    if (!A) return SA_OK;
    A->d.release();
    delete A;
    return SA_OK;
}

extern "C" int sa_mat_info(sa_mat A, int *n, int *m, int64_t *nnz, int *bit, int *precision) {
    if (!A) return fail(SA_ERR_ARG, "null matrix");
    if (n) *n = A->d.n;
    if (m) *m = A->d.m;
    if (nnz) *nnz = A->d.nnz;
    if (bit) *bit = A->d.bit;
    if (precision) *precision = A->precision;
    return SA_OK;
}

static size_t esize(int precision) { return precision == SA_F64 ? 8 : 4; }

extern "C" int sa_spmv(sa_ctx ctx, sa_mat A, const void *x, void *y) {
    if (!ctx || !A || !x || !y) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t es = esize(A->precision);
    Staged sx(c, x, es * A->d.m, true, false);
    Staged sy(c, y, es * A->d.n, false, true);
    spmv(c, A->d, sx.get(), sy.get());
    sy.finish();
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

// ------------------------------------------------------------ host setup

extern "C" void sa_amg_params_default(sa_amg_params *p) {
    if (!p) return;
    p->max_levels = 20;
    p->theta = 0.8;
    p->smoother_blocks = 0;
    p->omega = 1.0;
    p->smooth_iter = 1;
    p->multicolor = 0;
    p->max_colours = 0;
    p->coarse_colours = 0;
    p->coarse_size = 0;
}

static void build_setup(sa_hierarchy &s, const CsrD &A, Ctx *gpu = nullptr) {
    if (s.p.theta <= 0 || s.p.theta > 1) throw SetupError{"Theta must be in 0 < theta <= 1"};
    const int cs = s.p.coarse_size > 0 ? s.p.coarse_size : 2000;
    if (!s.chain)
        s.chain = std::make_shared<RsChain>(gpu ? rs_chain_gpu(*gpu, A, s.p.theta, s.p.max_levels, cs)
                                                : rs_chain(A, s.p.theta, s.p.max_levels, cs));
    const RsChain &chain = *s.chain;
    SmootherSpec sm;
    sm.block = s.p.smoother_blocks;
    sm.omega = s.p.omega;
    sm.iter = s.p.smooth_iter;
    sm.multicolor = s.p.multicolor;
    sm.max_colours = s.p.max_colours;
    sm.coarse_colours = s.p.coarse_colours;
    sm.level_caps = s.level_caps;
    if (s.precision == SA_INT) s.hi = std::make_shared<IntHierarchy>(build_int_hierarchy(A, chain, sm));
    else if (s.precision == SA_F64) s.hd = std::make_shared<FpHierarchy<double>>(build_f64_hierarchy(A, chain, sm));
    else s.hf = std::make_shared<FpHierarchy<float>>(build_f32_hierarchy(A, chain, sm));
}

static int setup_create(Ctx *gpu, int precision, const sa_amg_params *p, int n, const int32_t *rptr,
                        const int32_t *cind, const double *val, sa_setup *out) {
    if (!out || precision < SA_INT || precision > SA_F32) return fail(SA_ERR_ARG, "invalid argument");
    if (int e = check_csr(n, n, rptr, cind)) return e;
    SA_GUARD_BEGIN
    auto *s = new sa_hierarchy();
    s->precision = precision;
    if (p) s->p = *p;
    else sa_amg_params_default(&s->p);
    if (s->p.smooth_iter < 1 || s->p.max_levels < 1 || s->p.smoother_blocks < 0 ||
        s->p.multicolor < 0 || s->p.multicolor > 2 || (s->p.multicolor && s->p.smoother_blocks) ||
        s->p.max_colours < 0 || s->p.coarse_size < 0 || s->p.coarse_colours < 0) {
        delete s;
        return fail(SA_ERR_ARG, "invalid AMG parameters");
    }
    auto A = std::make_shared<CsrD>();
    A->n = A->m = n;
    A->rptr.assign(rptr, rptr + n + 1);
    A->cind.assign(cind, cind + rptr[n]);
    A->val.assign(val, val + rptr[n]);
    s->A = A;
    try {
        build_setup(*s, *A, gpu);
    } catch (...) {
        delete s;
        throw;
    }
    *out = s;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_setup_create(int precision, const sa_amg_params *p, int n, const int32_t *rptr,
                               const int32_t *cind, const double *val, sa_setup *out) {
    return setup_create(nullptr, precision, p, n, rptr, cind, val, out);
}

extern "C" int sa_setup_create_gpu(sa_ctx ctx, int precision, const sa_amg_params *p, int n, const int32_t *rptr,
                                   const int32_t *cind, const double *val, sa_setup *out) {
    if (!ctx) return fail(SA_ERR_ARG, "null context");
    return setup_create(&ctx->c, precision, p, n, rptr, cind, val, out);
}

extern "C" int sa_setup_derive(sa_setup s, int precision, sa_setup *out) {
    if (!s || !out || precision < SA_INT || precision > SA_F32) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    auto *d = new sa_hierarchy();
    d->precision = precision;
    d->p = s->p;
    d->level_caps = s->level_caps;
    d->A = s->A;
    d->chain = s->chain;
    try {
        build_setup(*d, *d->A);
    } catch (...) {
        delete d;
        throw;
    }
    *out = d;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_setup_destroy(sa_setup s) {
    delete s;
    return SA_OK;
}

extern "C" int sa_setup_depth(sa_setup s) {
    if (!s) return -1;
    if (s->hi) return s->hi->depth;
    if (s->hd) return s->hd->depth;
    if (s->hf) return s->hf->depth;
    return -1;
}

template <typename M>
static void view_of(const M &a, sa_csr_view *o, int bit, int dbit) {
    o->n = a.n;
    o->m = a.m;
    o->nnz = a.nnz();
    o->rptr = a.rptr.data();
    o->cind = a.cind.data();
    o->val = a.val.data();
    o->bit = bit;
    o->dbit = dbit;
}

template <typename H, typename B>
static int view_hier(const H &h, int op, int level, sa_csr_view *o, B bits) {
    const int D = h.depth;
    auto bad = [&] { return fail(SA_ERR_ARG, "no such operator/level"); };
    switch (op) {
        case SA_OP_A0: view_of(h.A0, o, bits(h.A0).first, 0); return SA_OK;
        case SA_OP_CA: if (level < 0 || level >= D - 1) return bad(); view_of(h.CA[level], o, bits(h.CA[level]).first, 0); return SA_OK;
        case SA_OP_P: if (level < 0 || level >= D) return bad(); view_of(h.P[level], o, bits(h.P[level]).first, 0); return SA_OK;
        case SA_OP_R: if (level < 0 || level >= D) return bad(); view_of(h.R[level], o, bits(h.R[level]).first, 0); return SA_OK;
        case SA_OP_LD: if (level < 0 || level >= D) return bad(); view_of(h.LD[level], o, bits(h.LD[level]).first, bits(h.LD[level]).second); return SA_OK;
        case SA_OP_U: if (level < 0 || level >= D) return bad(); view_of(h.U[level], o, bits(h.U[level]).first, 0); return SA_OK;
        case SA_OP_LUL: view_of(h.LUL, o, bits(h.LUL).first, 0); return SA_OK;
        case SA_OP_LUU: view_of(h.LUU, o, bits(h.LUU).first, bits(h.LUU).second); return SA_OK;
        case SA_OP_BJ:
            if (level < 0 || level >= D || h.bj[level].empty()) return bad();
            o->n = (int)h.bj[level].size() - 1;
            o->m = 0;
            o->nnz = 0;
            o->rptr = h.bj[level].data();
            o->cind = nullptr;
            o->val = nullptr;
            o->bit = o->dbit = 0;
            return SA_OK;
        case SA_OP_COLOR:
            if (level < 0 || level >= D || h.colour[level].empty()) return bad();
            o->n = (int)h.colour[level].size();
            o->m = 0;
            o->nnz = 0;
            o->rptr = h.colour[level].data();
            o->cind = nullptr;
            o->val = nullptr;
            o->bit = o->dbit = 0;
            return SA_OK;
    }
    return bad();
}

extern "C" int sa_setup_view(sa_setup s, int op, int level, sa_csr_view *out) {
    if (!s || !out) return fail(SA_ERR_ARG, "null argument");
    if (s->hi) return view_hier(*s->hi, op, level, out, [](const CsrI &m) { return std::make_pair(m.bit, m.dbit); });
    auto nob = [](const auto &) { return std::make_pair(0, 0); };
    if (s->hd) return view_hier(*s->hd, op, level, out, nob);
    if (s->hf) return view_hier(*s->hf, op, level, out, nob);
    return fail(SA_ERR_ARG, "empty setup");
}

// ------------------------------------------------------------------- AMG

extern "C" int sa_amg_create_from_setup(sa_ctx ctx, sa_setup s, sa_amg *out) {
    if (!ctx || !s || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    auto *h = new sa_multigrid();
    h->ctx = ctx;
    h->precision = s->precision;
    if (s->hi) h->M = upload_amg_int(ctx->c, s->hi);
    else if (s->hd) h->M = upload_amg_f64(ctx->c, s->hd);
    else h->M = upload_amg_f32(ctx->c, s->hf);
    SAGB_CUDA(cudaDeviceSynchronize());
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_amg_create(sa_ctx ctx, int precision, const sa_amg_params *p, int n, const int32_t *rptr,
                             const int32_t *cind, const double *val, sa_amg *out) {
    if (!ctx) return fail(SA_ERR_ARG, "null context");
    sa_setup s = nullptr;
    int e = sa_setup_create(precision, p, n, rptr, cind, val, &s);
    if (e) return e;
    e = sa_amg_create_from_setup(ctx, s, out);
    sa_setup_destroy(s);
    return e;
}

extern "C" int sa_amg_destroy(sa_amg M) {
    if (!M) return SA_OK;
    cudaStreamSynchronize(M->ctx->c.stream);
    M->M->release();
    delete M;
    return SA_OK;
}

extern "C" int sa_amg_depth(sa_amg M) { return M ? M->M->depth : -1; }
extern "C" int sa_amg_precision(sa_amg M) { return M ? M->precision : -1; }

extern "C" int sa_amg_precondition(sa_ctx ctx, sa_amg M, const void *in, void *out) {
    if (!ctx || !M || !in || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t bytes = esize(M->precision) * M->M->A0.n;
    Staged si(c, in, bytes, true, false);
    Staged so(c, out, bytes, false, true);
    vcycle(c, *M->M, si.get(), so.get());
    so.finish();
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

static int level_n(sa_amg M, int level) { return M->M->LD[level].n; }

extern "C" int sa_amg_smooth(sa_ctx ctx, sa_amg M, int level, const void *in, void *out, int inited) {
    if (!ctx || !M || !in || !out) return fail(SA_ERR_ARG, "null argument");
    if (level < 0 || level >= M->M->depth) return fail(SA_ERR_ARG, "no such level");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t bytes = esize(M->precision) * level_n(M, level);
    Staged si(c, in, bytes, true, false);
    Staged so(c, out, bytes, inited != 0, true);
    smooth(c, *M->M, level, si.get(), so.get(), inited != 0);
    so.finish();
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_amg_sweep(sa_ctx ctx, sa_amg M, int level, const void *in, void *out) {
    if (!ctx || !M || !in || !out) return fail(SA_ERR_ARG, "null argument");
    if (level < 0 || level >= M->M->depth) return fail(SA_ERR_ARG, "no such level");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t bytes = esize(M->precision) * level_n(M, level);
    Staged si(c, in, bytes, true, false);
    Staged so(c, out, bytes, false, true);
    trsv(c, M->M->LD[level], si.get(), so.get());
    so.finish();
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

// The sweep of sa_amg_sweep without any device allocation (see the header):
// device buffers only, scratch from the sweep kernels' static array.
extern "C" int sa_amg_sweep_noalloc(sa_ctx ctx, sa_amg M, int level, const void *in, void *out) {
    if (!ctx || !M || !in || !out) return fail(SA_ERR_ARG, "null argument");
    if (level < 0 || level >= M->M->depth) return fail(SA_ERR_ARG, "no such level");
    if (!is_device_ptr(in) || !is_device_ptr(out))
        return fail(SA_ERR_ARG, "sa_amg_sweep_noalloc needs device buffers (host buffers would need staging)");
    SA_GUARD_BEGIN
    trsv_noalloc(ctx->c, M->M->LD[level], in, out);
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_amg_coarse_solve(sa_ctx ctx, sa_amg M, const void *in, void *out) {
    if (!ctx || !M || !in || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t bytes = esize(M->precision) * M->M->LU.n;
    Staged si(c, in, bytes, true, false);
    Staged so(c, out, bytes, false, true);
    lu_solve(c, M->M->LU, si.get(), so.get());
    so.finish();
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

static const DevCsr *level_op(sa_amg M, int op, int level) {
    DevAmg &A = *M->M;
    const int D = A.depth;
    switch (op) {
        case SA_OP_A0: return &A.A0;
        case SA_OP_CA: return level >= 0 && level < D - 1 ? &A.CA[level] : nullptr;
        case SA_OP_P: return level >= 0 && level < D ? &A.P[level] : nullptr;
        case SA_OP_R: return level >= 0 && level < D ? &A.R[level] : nullptr;
        case SA_OP_U: return level >= 0 && level < D ? &A.U[level] : nullptr;
    }
    return nullptr;
}

extern "C" int sa_amg_level_spmv(sa_ctx ctx, sa_amg M, int op, int level, const void *in, void *out) {
    if (!ctx || !M || !in || !out) return fail(SA_ERR_ARG, "null argument");
    const DevCsr *A = level_op(M, op, level);
    if (!A) return fail(SA_ERR_ARG, "no such operator/level");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t es = esize(M->precision);
    Staged si(c, in, es * A->m, true, false);
    Staged so(c, out, es * A->n, false, true);
    spmv(c, *A, si.get(), so.get());
    so.finish();
    SAGB_CUDA(cudaGetLastError());
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_amg_level_info(sa_amg M, int op, int level, int *n, int *m, int64_t *nnz, int *bit, int *nlev) {
    if (!M) return fail(SA_ERR_ARG, "null multigrid");
    DevAmg &A = *M->M;
    if (op == SA_OP_LD) {
        if (level < 0 || level >= A.depth) return fail(SA_ERR_ARG, "no such level");
        const DevTri &T = A.LD[level];
        if (n) *n = T.n;
        if (m) *m = T.n;
        if (nnz) *nnz = T.nnz_off + T.n;
        if (bit) *bit = T.bit;
        if (nlev) *nlev = T.nlev;
        return SA_OK;
    }
    if (op == SA_OP_LUL || op == SA_OP_LUU) {
        if (n) *n = A.LU.n;
        if (m) *m = A.LU.n;
        if (nnz) *nnz = (int64_t)A.LU.n * A.LU.n;
        if (bit) *bit = op == SA_OP_LUL ? A.LU.bitL : A.LU.bitU;
        if (nlev) *nlev = A.LU.n;
        return SA_OK;
    }
    const DevCsr *D = level_op(M, op, level);
    if (!D) return fail(SA_ERR_ARG, "no such operator/level");
    if (n) *n = D->n;
    if (m) *m = D->m;
    if (nnz) *nnz = D->nnz;
    if (bit) *bit = D->bit;
    if (nlev) *nlev = 0;
    return SA_OK;
}

// ----------------------------------------------------------------- solvers

extern "C" void sa_solver_params_default(sa_solver_params *p) {
    if (!p) return;
    p->m = 30;
    p->eps = 1.0e-10;
    p->max_outer = 1000 / 30;
    p->frac_bits = 29;
    p->verbose = 0;
    p->overflow_fallback = 1;
    p->explicit_stop = 0;
    p->cycle_bits = 0;
}

extern "C" int sa_solver_create(sa_ctx ctx, int precision, sa_mat dA, sa_mat A, sa_amg M, const sa_solver_params *p,
                                sa_solver *out) {
    if (!ctx || !dA || !A || !M || !out) return fail(SA_ERR_ARG, "null argument");
    if (dA->precision != SA_F64) return fail(SA_ERR_ARG, "the refinement operator must be FP64");
    if (A->precision != precision || M->precision != precision)
        return fail(SA_ERR_ARG, "operator / preconditioner precision mismatch");
    if (dA->d.n != A->d.n || A->d.n != M->M->A0.n) return fail(SA_ERR_ARG, "size mismatch");
    sa_solver_params q;
    if (p) q = *p;
    else sa_solver_params_default(&q);
    if (q.m < 1 || q.m > 64 || q.max_outer < 1 || q.eps <= 0) return fail(SA_ERR_ARG, "invalid solver parameters");
    if (precision == SA_INT && (q.frac_bits < 1 || q.frac_bits > 30)) return fail(SA_ERR_ARG, "frac_bits must be in [1, 30]");
    SA_GUARD_BEGIN
    auto *h = new sa_krylov();
    h->ctx = ctx;
    h->precision = precision;
    h->p = q;
    h->dA = &dA->d;
    h->N = dA->d.n;
    KrylovParams kp;
    kp.m = q.m;
    kp.eps = q.eps;
    kp.max_outer = q.max_outer;
    kp.bit = q.frac_bits;
    kp.verbose = q.verbose;
    kp.fallback = precision == SA_INT ? q.overflow_fallback : 0;
    kp.explicit_check = q.explicit_stop;
    h->S = make_solver(ctx->c, precision == SA_INT ? VT_I32 : (precision == SA_F64 ? VT_F64 : VT_F32), &dA->d, &A->d,
                       M->M.get(), kp);
    *out = h;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_solver_destroy(sa_solver S) {
    if (!S) return SA_OK;
    cudaStreamSynchronize(S->ctx->c.stream);
    S->S.reset();
    dfree(S->db);
    dfree(S->dx);
    delete S;
    return SA_OK;
}

extern "C" int sa_solver_solve(sa_solver S, const double *b, double nrm_b, double *x, int *iters, int *converged) {
    if (!S || !b || !x) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = S->ctx->c;
    const size_t bytes = sizeof(double) * (size_t)S->N;
    const double *db = b;
    double *dx = x;
    const bool hb = !is_device_ptr(b), hx = !is_device_ptr(x);
    if (hb) {
        if (!S->db) S->db = (double *)dmalloc(bytes);
        SAGB_CUDA(cudaMemcpyAsync(S->db, b, bytes, cudaMemcpyHostToDevice, c.stream));
        db = S->db;
    }
    if (hx) {
        if (!S->dx) S->dx = (double *)dmalloc(bytes);
        SAGB_CUDA(cudaMemcpyAsync(S->dx, x, bytes, cudaMemcpyHostToDevice, c.stream));
        dx = S->dx;
    }
    SAGB_CUDA(cudaMemsetAsync(c.d_flags_main, 0, 2 * sizeof(unsigned), c.stream));
    int it = S->S->solve(db, nrm_b, dx, S->last);
    if (hx) SAGB_CUDA(cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    SAGB_CUDA(cudaGetLastError());
    if (iters) *iters = it;
    if (converged) *converged = S->last.converged;
    if (S->precision == SA_INT && S->last.final_bit > 0) S->p.frac_bits = S->last.final_bit;
    if (S->last.flags & ST_TIMEOUT) return fail(SA_ERR_NUMERIC, "device wait timed out");
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_solver_cycle(sa_solver S, const double *r, double nrm_b, double *x, const double *e0, int *iters,
                               int *converged, void *const *dumps) {
    if (!S || !r || !x) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = S->ctx->c;
    const size_t bytes = sizeof(double) * (size_t)S->N;
    Staged sr(c, r, bytes, true, false);
    Staged sx(c, x, bytes, true, true);
    int conv = 0;
    SAGB_CUDA(cudaMemsetAsync(c.d_flags_main, 0, 2 * sizeof(unsigned), c.stream));
    int it = S->S->cycle((const double *)sr.get(), nrm_b, (double *)sx.get(), e0, &conv, dumps);
    if (it < 0) {
        sx.finish();
        if (iters) *iters = 0;
        if (converged) *converged = 0;
        return fail(SA_ERR_NUMERIC, "integer overflow in the cycle (lower frac_bits)");
    }
    sx.finish();
    SAGB_CUDA(cudaGetLastError());
    if (iters) *iters = it;
    if (converged) *converged = conv;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_solver_set_bits(sa_solver S, int bits) {
    if (!S) return fail(SA_ERR_ARG, "null solver");
    if (S->precision != SA_INT) return fail(SA_ERR_ARG, "only the integer solver has fractional bits");
    if (bits < 1 || bits > 30) return fail(SA_ERR_ARG, "frac_bits must be in [1, 30]");
    S->p.frac_bits = bits;
    S->S->set_bit(bits);
    return SA_OK;
}

extern "C" int sa_solver_bits(sa_solver S, int *bits) {
    if (!S || !bits) return fail(SA_ERR_ARG, "null argument");
    *bits = S->p.frac_bits;
    return SA_OK;
}

extern "C" int sa_solver_history(sa_solver S, double *hist, int cap, int *n, unsigned *flags) {
    if (!S) return fail(SA_ERR_ARG, "null solver");
    const int k = (int)S->last.history.size();
    if (n) *n = k;
    if (flags) *flags = S->last.flags;
    if (hist)
        for (int i = 0; i < k && i < cap; i++) hist[i] = S->last.history[i];
    return SA_OK;
}

extern "C" int sa_rule_ratio(sa_ctx ctx, sa_amg M, const double *b, double nrm_b, double *ratio) {
    if (!ctx || !M || !b || !ratio) return fail(SA_ERR_ARG, "null argument");
    if (M->precision != SA_F64) return fail(SA_ERR_ARG, "the bit rule uses the FP64 preconditioner");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const int N = M->M->A0.n;
    std::vector<double> ch(N);
    Staged sb(c, b, sizeof(double) * N, true, false);
    double *dc = (double *)dmalloc(sizeof(double) * N);
    vcycle(c, *M->M, sb.get(), dc);
    SAGB_CUDA(cudaMemcpyAsync(ch.data(), dc, sizeof(double) * N, cudaMemcpyDeviceToHost, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    dfree(dc);
    double cmax = 0;
    for (int i = 0; i < N; i++)
        if (std::fabs(ch[i]) > cmax) cmax = std::fabs(ch[i]);
    *ratio = cmax / nrm_b;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_rule_bits(sa_ctx ctx, sa_amg M, const double *b, double nrm_b, int *bits) {
    if (!ctx || !M || !b || !bits) return fail(SA_ERR_ARG, "null argument");
    if (M->precision != SA_F64) return fail(SA_ERR_ARG, "the bit rule uses the FP64 preconditioner");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const int N = M->M->A0.n;
    std::vector<double> ch(N);
    Staged sb(c, b, sizeof(double) * N, true, false);
    double *dc = (double *)dmalloc(sizeof(double) * N);
    vcycle(c, *M->M, sb.get(), dc);
    SAGB_CUDA(cudaMemcpyAsync(ch.data(), dc, sizeof(double) * N, cudaMemcpyDeviceToHost, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    dfree(dc);
    double cmax = 0;
    for (int i = 0; i < N; i++)
        if (std::fabs(ch[i]) > cmax) cmax = std::fabs(ch[i]);
    *bits = rule_frac_bits(cmax, nrm_b);
    return SA_OK;
    SA_GUARD_END
}

// ------------------------------------------------------ learned bit selector

extern "C" int sa_setup_features(sa_setup s, double ratio, float *feat) {
    if (!s || !feat) return fail(SA_ERR_ARG, "null argument");
    if (!s->hi || !s->A) return fail(SA_ERR_ARG, "features need an integer setup");
    SA_GUARD_BEGIN
    bit_features(*s->A, *s->hi, ratio, feat);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_create(sa_ctx ctx, int n_in, int hidden, int n_out, uint64_t seed, sa_mlp *out) {
    if (!ctx || !out) return fail(SA_ERR_ARG, "null argument");
    if (n_in < 1 || hidden < 1 || n_out < 1 || n_in > 4096 || hidden > 4096 || n_out > 4096)
        return fail(SA_ERR_ARG, "invalid MLP shape");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaSetDevice(ctx->c.device));
    auto *m = new sa_mlp_net();
    m->net = std::make_unique<Mlp>(n_in, hidden, n_out, seed);
    *out = m;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_destroy(sa_mlp m) {
    delete m;
    return SA_OK;
}

extern "C" int sa_mlp_nparams(sa_mlp m, int64_t *n) {
    if (!m || !n) return fail(SA_ERR_ARG, "null argument");
    *n = (int64_t)m->net->nparams();
    return SA_OK;
}

extern "C" int sa_mlp_get_params(sa_mlp m, float *out) {
    if (!m || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    m->net->get_params(out);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_set_params(sa_mlp m, const float *in) {
    if (!m || !in) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    m->net->set_params(in);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_set_norm(sa_mlp m, const float *mu, const float *sd) {
    if (!m || !mu || !sd) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    m->net->set_norm(mu, sd);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_predict(sa_ctx ctx, sa_mlp m, const float *X, int n, float *Y) {
    if (!ctx || !m || !X || !Y || n < 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    m->net->predict(ctx->c, X, n, Y);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_gradient(sa_ctx ctx, sa_mlp m, const float *X, const float *T, const float *M, int n,
                               float *grad, float *loss) {
    if (!ctx || !m || !X || !T || !M || n < 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    const float l = m->net->gradient(ctx->c, X, T, M, n, grad);
    if (loss) *loss = l;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_train(sa_ctx ctx, sa_mlp m, const float *X, const float *T, const float *M, int n,
                            int epochs, int batch, float lr, uint64_t seed, float *loss_hist) {
    if (!ctx || !m || !X || !T || !M || n < 1 || epochs < 1 || batch < 1 || !(lr > 0))
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    m->net->train(ctx->c, X, T, M, n, epochs, batch, lr, seed, loss_hist);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_mlp_select_bits(sa_ctx ctx, sa_mlp m, const float *feat, int f_lo, int *bits) {
    if (!ctx || !m || !feat || !bits) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    std::vector<float> y(m->net->nout);
    m->net->predict(ctx->c, feat, 1, y.data());
    int k = 0;
    for (int i = 1; i < (int)y.size(); i++)
        if (y[i] < y[k]) k = i;
    *bits = f_lo + k;
    return SA_OK;
    SA_GUARD_END
}

// ------------------------------------------------------------ batched solver

extern "C" int sa_batch_create(sa_ctx ctx, int nsys, const int *n, const int32_t *const *rptr,
                               const int32_t *const *cind, const double *const *val, int nrhs,
                               const sa_amg_params *p, int threads, sa_batch *out) {
    if (!ctx || !n || !rptr || !cind || !val || !out || nsys < 1) return fail(SA_ERR_ARG, "invalid argument");
    if (nrhs != 1 && nrhs != 2 && nrhs != 4) return fail(SA_ERR_ARG, "nrhs must be 1, 2 or 4");
    for (int s = 0; s < nsys; s++)
        if (int e = check_csr(n[s], n[s], rptr[s], cind[s])) return e;
    sa_amg_params q;
    if (p) q = *p;
    else sa_amg_params_default(&q);
    if (q.smooth_iter < 1 || q.max_levels < 1 || q.smoother_blocks != 0 || q.theta <= 0 || q.theta > 1 ||
        q.max_colours < 0 || q.coarse_size < 0 || q.coarse_colours < 0)
        return fail(SA_ERR_ARG, "invalid AMG parameters (the batch uses the multicolour SOR smoother)");
    q.multicolor = 1;
    SA_GUARD_BEGIN
    // systems passed with the same arrays share one setup
    std::vector<CsrD> sys(nsys);
    std::vector<int> src(nsys);
    for (int s = 0; s < nsys; s++) {
        src[s] = s;
        for (int t = 0; t < s; t++)
            if (src[t] == t && n[t] == n[s] && rptr[t] == rptr[s] && cind[t] == cind[s] && val[t] == val[s]) {
                src[s] = t;
                break;
            }
        if (src[s] != s) {
            sys[s].n = sys[s].m = n[s];
            continue;
        }
        sys[s].n = sys[s].m = n[s];
        sys[s].rptr.assign(rptr[s], rptr[s] + n[s] + 1);
        sys[s].cind.assign(cind[s], cind[s] + rptr[s][n[s]]);
        sys[s].val.assign(val[s], val[s] + rptr[s][n[s]]);
    }
    if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    auto *B = new sa_batch_set();
    B->ctx = ctx;
    B->p = q;
    try {
        const int cs = q.coarse_size > 0 ? q.coarse_size : 2000;
        std::function<RsChain(const CsrD &)> gpu_chain;
        if (ctx->c.gpu_setup_rows > 0)
            gpu_chain = [&](const CsrD &A) { return rs_chain_gpu(ctx->c, A, q.theta, q.max_levels, cs); };
        B->h = std::make_shared<BatchHierarchy>(build_batch(sys, q.theta, q.max_levels, q.omega, q.smooth_iter,
                                                            threads, src, q.max_colours, q.coarse_colours, cs,
                                                            gpu_chain,
                                                            ctx->c.gpu_setup_rows));
        SAGB_CUDA(cudaSetDevice(ctx->c.device));
        B->eng = std::make_unique<BatchEngine>(ctx->c, B->h, nrhs);
        SAGB_CUDA(cudaDeviceSynchronize());
    } catch (...) {
        delete B;
        throw;
    }
    *out = B;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_set_colour_caps(sa_ctx ctx, sa_batch B, int ncaps, const int *caps, int threads) {
    if (!ctx || !B || ncaps < 0 || (ncaps > 0 && !caps)) return fail(SA_ERR_ARG, "invalid argument");
    for (int k = 0; k < ncaps; k++)
        if (caps[k] < 0) return fail(SA_ERR_ARG, "colour caps must be >= 0");
    SA_GUARD_BEGIN
    SmootherSpec sm = B->h->sm;
    sm.level_caps.assign(caps, caps + ncaps);
    if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    auto h = std::make_shared<BatchHierarchy>(rebuild_batch_smoothers(*B->h, sm, threads));
    const int nrhs = B->eng->nrhs();
    SAGB_CUDA(cudaSetDevice(ctx->c.device));
    B->eng.reset();  // the old engine's device arrays go before the new ones come
    B->h = h;
    B->eng = std::make_unique<BatchEngine>(ctx->c, B->h, nrhs);
    SAGB_CUDA(cudaDeviceSynchronize());
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_colour_caps(sa_batch B, int cap, int *ncaps, int *caps) {
    if (!B || !ncaps) return fail(SA_ERR_ARG, "null argument");
    const SmootherSpec &sm = B->h->sm;
    const int D = B->h->Dmax;
    *ncaps = D;
    for (int l = 0; l < D && l < cap && caps; l++) caps[l] = sm.cap(l);
    return SA_OK;
}

extern "C" int sa_batch_destroy(sa_batch B) {
    delete B;
    return SA_OK;
}

extern "C" int sa_batch_info(sa_batch B, int *nsys, int *nrhs, int *depth_max, int64_t *rows) {
    if (!B) return fail(SA_ERR_ARG, "null argument");
    if (nsys) *nsys = B->h->S;
    if (nrhs) *nrhs = B->eng->nrhs();
    if (depth_max) *depth_max = B->h->Dmax;
    if (rows) *rows = (int64_t)B->eng->rows();
    return SA_OK;
}

extern "C" int sa_batch_offsets(sa_batch B, int64_t *offsets) {
    if (!B || !offsets) return fail(SA_ERR_ARG, "null argument");
    for (int s = 0; s < B->h->S; s++) offsets[s] = B->h->offset[0][s];
    offsets[B->h->S] = B->h->n_level[0];
    return SA_OK;
}

extern "C" int sa_batch_system_setup(sa_batch B, int sys, sa_setup *out) {
    if (!B || !out || sys < 0 || sys >= B->h->S) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    auto *s = new sa_hierarchy();
    s->precision = SA_INT;
    s->p = B->p;
    s->level_caps = B->h->sm.level_caps;
    s->A = B->h->A_sys[sys];
    s->chain = B->h->chain[sys];
    s->hi = B->h->hi[sys];
    *out = s;
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_precondition(sa_ctx ctx, sa_batch B, const int32_t *in, int32_t *out) {
    if (!ctx || !B || !in || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t bytes = sizeof(int32_t) * B->eng->rows() * B->eng->nrhs();
    Staged si(c, in, bytes, true, false);
    Staged so(c, out, bytes, false, true);
    B->eng->precondition((const int *)si.get(), (int *)so.get());
    so.finish();
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_autotune(sa_ctx ctx, sa_batch B, int reps) {
    if (!ctx || !B || reps < 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    B->eng->autotune(reps);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_set_group(sa_batch B, int level, int op, int group) {
    if (!B || level < 0 || level >= B->h->Dmax || op < 0 || op > 4 ||
        !(group == 1 || group == 2 || group == 4 || group == 8 || group == 16 || group == 32 || (group == 0 && op != 1)))
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    B->eng->set_groups(level, op, group);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_compressed(sa_batch B, int level, int op, int set, int *on) {
    if (!B || !on || level < 0 || level >= B->h->Dmax || (op != 0 && op != 2) || set < -1 || set > 1)
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *on = B->eng->compressed(level, op, set);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_ell(sa_batch B, int level, int op, int set, int *on) {
    if (!B || !on || level < 0 || level >= B->h->Dmax || (op != 0 && op != 2) || set < -1 || set > 1)
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *on = B->eng->ell(level, op, set);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_fused_sweeps(sa_batch B, int set, int *levels) {
    if (!B || !levels || set < -1 || set > 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *levels = B->eng->fused_sweeps(set);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_fp_fused_sweeps(sa_batch_fp F, int set, int *levels) {
    if (!F || !levels || set < -1 || set > 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *levels = F->eng->fused_sweeps(set);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_tail(sa_batch B, int set, int *from) {
    if (!B || !from || set < -1 || set >= B->h->Dmax) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *from = B->eng->tail(set);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_tail_selftest(sa_ctx ctx, sa_batch B, int level, double timeout_ms, unsigned *status) {
    if (!ctx || !B || !status || level < 1 || level >= B->h->Dmax || !(timeout_ms > 0) || timeout_ms > 2000)
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *status = B->eng->tail_selftest(level, timeout_ms);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_sweep_form(sa_batch B, int level, int set, int *form) {
    if (!B || !form || level < 0 || level >= B->h->Dmax || set < -1 || set > 3)
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *form = B->eng->sweep_form(level, set);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_group(sa_batch B, int level, int op, int *group) {
    if (!B || !group || level < 0 || level >= B->h->Dmax || op < 0 || op > 4) return fail(SA_ERR_ARG, "invalid argument");
    *group = B->eng->group(level, op);
    return SA_OK;
}

extern "C" int sa_batch_rule_ratios(sa_ctx ctx, sa_batch B, const double *b, const double *nrm_b, double *ratio) {
    if (!ctx || !B || !b || !nrm_b || !ratio) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const int S = B->h->S, R = B->eng->nrhs();
    const size_t N0 = B->eng->rows();
    std::vector<double> hb(N0 * R), hn((size_t)S * R);
    SAGB_CUDA(cudaMemcpy(hb.data(), b, sizeof(double) * hb.size(), cudaMemcpyDefault));
    SAGB_CUDA(cudaMemcpy(hn.data(), nrm_b, sizeof(double) * hn.size(), cudaMemcpyDefault));
    const SmootherSpec sm = B->h->sm;
    // FP64 hierarchies of all systems on host threads (copies of one matrix share one)
    std::vector<std::shared_ptr<FpHierarchy<double>>> hds(S);
    {
        std::atomic<int> next{0};
        auto work = [&]() {
            for (;;) {
                const int s = next.fetch_add(1);
                if (s >= S) return;
                bool copy = false;
                for (int t = 0; t < s && !copy; t++) copy = B->h->hi[t] == B->h->hi[s];
                if (!copy)
                    hds[s] = std::make_shared<FpHierarchy<double>>(
                        build_f64_hierarchy(*B->h->A_sys[s], *B->h->chain[s], sm));
            }
        };
        const int T = std::max(1, std::min(S, (int)std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int t = 1; t < T; t++) pool.emplace_back(work);
        work();
        for (auto &t : pool) t.join();
        for (int s = 0; s < S; s++)
            if (!hds[s])
                for (int t = 0; t < s; t++)
                    if (B->h->hi[t] == B->h->hi[s] && hds[t]) {
                        hds[s] = hds[t];
                        break;
                    }
    }
    for (int s = 0; s < S; s++) {
        // Work/main.cpp:153-161 per system: one FP64 V-cycle of its own hierarchy
        auto M = upload_amg_f64(c, hds[s]);
        const int n = B->h->n_sys[s];
        const size_t off = (size_t)B->h->offset[0][s];
        std::vector<double> col(n), out(n);
        double *db = (double *)dmalloc(sizeof(double) * n), *dc = (double *)dmalloc(sizeof(double) * n);
        for (int r = 0; r < R; r++) {
            for (int i = 0; i < n; i++) col[i] = hb[(off + i) * R + r];
            SAGB_CUDA(cudaMemcpyAsync(db, col.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
            vcycle(c, *M, db, dc);
            SAGB_CUDA(cudaMemcpyAsync(out.data(), dc, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
            SAGB_CUDA(cudaStreamSynchronize(c.stream));
            double cmax = 0;
            for (int i = 0; i < n; i++) cmax = std::max(cmax, std::fabs(out[i]));
            ratio[(size_t)s * R + r] = cmax / hn[(size_t)s * R + r];
        }
        dfree(db);
        dfree(dc);
        M->release();
        if (s + 1 < S && hds[s + 1] != hds[s]) hds[s].reset();
    }
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_solve(sa_ctx ctx, sa_batch B, const sa_solver_params *p, const int *bits, const double *b,
                              const double *nrm_b, double *x, int *iters, int *converged, int *final_bits) {
    if (!ctx || !B || !p || !bits || !b || !nrm_b || !x) return fail(SA_ERR_ARG, "null argument");
    if (p->m < 1 || p->m > 64 || p->max_outer < 1 || !(p->eps > 0)) return fail(SA_ERR_ARG, "invalid solver parameters");
    const int S = B->h->S, R = B->eng->nrhs();
    for (int s = 0; s < S; s++)
        if (bits[s] < 1 || bits[s] > 30) return fail(SA_ERR_ARG, "fractional bits out of range");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    KrylovParams kp;
    kp.m = p->m;
    kp.eps = p->eps;
    kp.max_outer = p->max_outer;
    kp.fallback = p->overflow_fallback;
    kp.explicit_check = p->explicit_stop;
    kp.cycle_bits = p->cycle_bits;
    if (p->cycle_bits < 0 || p->cycle_bits > 30) return fail(SA_ERR_ARG, "cycle_bits out of range (0..30)");
    const size_t bytes = sizeof(double) * B->eng->rows() * R;
    Staged sb(c, b, bytes, true, false);
    Staged sx(c, x, bytes, true, true);
    BatchStats st;
    B->eng->solve(kp, bits, (const double *)sb.get(), nrm_b, (double *)sx.get(), st);
    sx.finish();
    for (int q = 0; q < S * R; q++) {
        if (iters) iters[q] = st.iters[q];
        if (converged) converged[q] = st.converged[q];
        if (final_bits) final_bits[q] = st.final_bit[q];
    }
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_level_op(sa_ctx ctx, sa_batch B, int level, int op, const int32_t *in, int32_t *out) {
    if (!ctx || !B || !in || !out) return fail(SA_ERR_ARG, "null argument");
    if (level < 0 || level >= B->h->Dmax || op < 0 || op > 4) return fail(SA_ERR_ARG, "no such operator/level");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    int n = 0, m = 0;
    B->eng->level_info(level, op, &n, &m, nullptr, nullptr);
    const int R = B->eng->nrhs();
    const size_t rows_in = (size_t)(op == 1 ? n : m), rows_out = (size_t)n;
    Staged si(c, in, sizeof(int32_t) * std::max<size_t>(rows_in, 1) * R, true, false);
    Staged so(c, out, sizeof(int32_t) * std::max<size_t>(rows_out, 1) * R, op == 1, true);
    B->eng->level_op(level, op, (const int *)si.get(), (int *)so.get());
    so.finish();
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_time_op(sa_ctx ctx, sa_batch B, int level, int op, const int32_t *in, int32_t *out, int reps,
                                float *ms) {
    if (!ctx || !B || !ms || reps < 1 || op < 0 || op > 6 || (op <= 4 && (level < 0 || level >= B->h->Dmax)) ||
        (op != 5 && (!in || !out)))
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *ms = B->eng->time_op(level, op, in, out, reps);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_time_op_cold(sa_ctx ctx, sa_batch B, int level, int op, const int32_t *in, int32_t *out,
                                     int reps, float *ms) {
    if (!ctx || !B || !ms || reps < 1 || op < 0 || op > 6 || (op <= 4 && (level < 0 || level >= B->h->Dmax)) ||
        (op != 5 && (!in || !out)))
        return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *ms = B->eng->time_op(level, op, in, out, reps, true);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_coarse_solve(sa_ctx ctx, sa_batch B) {
    if (!ctx || !B) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    B->eng->coarse_solve();
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_level_info(sa_batch B, int level, int op, int *n, int *m, int64_t *nnz, int *ncolours) {
    if (!B || level < 0 || level >= B->h->Dmax || op < 0 || op > 4) return fail(SA_ERR_ARG, "no such operator/level");
    SA_GUARD_BEGIN
    B->eng->level_info(level, op, n, m, nnz, ncolours);
    return SA_OK;
    SA_GUARD_END
}

// ------------------------------------------------------------- profiling

extern "C" int sa_profiler_range(int on) {
    SA_GUARD_BEGIN
    SAGB_CUDA(on ? cudaProfilerStart() : cudaProfilerStop());
    return SA_OK;
    SA_GUARD_END
}

// --------------------------------------- floating-point siblings of a batch

extern "C" int sa_batch_fp_create(sa_ctx ctx, sa_batch B, int precision, int threads, sa_batch_fp *out) {
    if (!ctx || !B || !out) return fail(SA_ERR_ARG, "null argument");
    if (precision != SA_F64 && precision != SA_F32) return fail(SA_ERR_ARG, "precision must be SA_F64 or SA_F32");
    SA_GUARD_BEGIN
    SAGB_CUDA(cudaSetDevice(ctx->c.device));
    auto F = std::make_unique<sa_batch_fp_set>();
    F->h = B->h;
    F->nrhs = B->eng->nrhs();
    F->eng = std::make_unique<BatchFpEngine>(ctx->c, B->h, precision == SA_F64 ? VT_F64 : VT_F32, F->nrhs,
                                             threads);
    SAGB_CUDA(cudaDeviceSynchronize());
    *out = F.release();
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_fp_destroy(sa_batch_fp F) {
    delete F;
    return SA_OK;
}

extern "C" int sa_batch_fp_precondition(sa_ctx ctx, sa_batch_fp F, const void *in, void *out) {
    if (!ctx || !F || !in || !out) return fail(SA_ERR_ARG, "null argument");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    const size_t bytes = vt_size(F->eng->precision()) * F->eng->rows() * F->nrhs;
    Staged si(c, in, bytes, true, false);
    Staged so(c, out, bytes, false, true);
    F->eng->precondition(si.get(), so.get());
    so.finish();
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_fp_autotune(sa_ctx ctx, sa_batch_fp F, int reps) {
    if (!ctx || !F || reps < 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    F->eng->autotune(reps);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_fp_time_vcycle(sa_ctx ctx, sa_batch_fp F, int reps, float *ms) {
    if (!ctx || !F || !ms || reps < 1) return fail(SA_ERR_ARG, "invalid argument");
    SA_GUARD_BEGIN
    *ms = F->eng->time_vcycle(reps);
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_fp_solve(sa_ctx ctx, sa_batch_fp F, const sa_solver_params *p, const double *b,
                                 const double *nrm_b, double *x, int *iters, int *converged) {
    if (!ctx || !F || !p || !b || !nrm_b || !x) return fail(SA_ERR_ARG, "null argument");
    if (p->m < 1 || p->m > 64 || p->max_outer < 1 || !(p->eps > 0)) return fail(SA_ERR_ARG, "invalid solver parameters");
    SA_GUARD_BEGIN
    Ctx &c = ctx->c;
    KrylovParams kp;
    kp.m = p->m;
    kp.eps = p->eps;
    kp.max_outer = p->max_outer;
    kp.explicit_check = p->explicit_stop;
    const size_t bytes = sizeof(double) * F->eng->rows() * F->nrhs;
    Staged sb(c, b, bytes, true, false);
    Staged sx(c, x, bytes, true, true);
    BatchStats st;
    F->eng->solve(kp, (const double *)sb.get(), nrm_b, (double *)sx.get(), st);
    sx.finish();
    const int P = F->h->S * F->nrhs;
    for (int q = 0; q < P; q++) {
        if (iters) iters[q] = st.iters[q];
        if (converged) converged[q] = st.converged[q];
    }
    return SA_OK;
    SA_GUARD_END
}

extern "C" int sa_batch_cycle_graphs(sa_batch B, sa_batch_fp F, int *cycles) {
    if ((!B) == (!F) || !cycles) return fail(SA_ERR_ARG, "pass one of the two batches and an output");
    *cycles = B ? B->eng->last_cycle_graphs() : F->eng->last_cycle_graphs();
    return SA_OK;
}
