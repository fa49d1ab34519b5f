// FGMRES(m) with FP64 iterative refinement on the GPU.
//
//   Restarted::Solve            solver/irsolver.hpp:61-77
//   FGMRESflex::Solve (int)     solver/gmres.hpp:307-353
//   FGMRES<double>::Solve       solver/gmres.hpp:130-170
//   FGMRES<float>::Solve        solver/gmres.hpp:212-252
//
// Arnoldi uses modified Gram-Schmidt exactly as the reference: H_kj is the dot
// of V_k with the current w, then w is updated, for k = 0..j in order.  Each
// update pass is fused with the next dot (w -= h_k V_k; dot(V_{k+1}, w)), so
// step j costs j+2 passes over w.  Integer dots are exact int64 sums (wrapping
// atomics); FP dots use a fixed-order two-level reduction (reproducible).
// Givens rotations, the convergence test and the Hessenberg back solve run on
// one device thread, so the inner loop needs no host round trip except one
// small status read per step.  Each Arnoldi step is captured once into a CUDA
// graph and replayed.
#include <cmath>
#include <cstdio>
#include <type_traits>

#include "../sagb_internal.hpp"
#include "common.cuh"
#include "stream.cuh"

namespace sagb {

constexpr int kRedThreads = 256;

template <typename T>
__device__ __forceinline__ T block_sum(T v, T *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        if constexpr (std::is_same<T, long long>::value) v = wadd(v, shfl_xor(v, o));
        else v += shfl_xor(v, o);
    }
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    T r = 0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            if constexpr (std::is_same<T, long long>::value) r = wadd(r, sh[w]);
            else r += sh[w];
        }
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// Fixed-order finish of a two-level FP reduction: called by every block after
// it stored its partial; the last block sums the partials (fixed tree) and
// returns true in thread 0 with *res set.
template <typename T>
__device__ bool finish_reduce(T bsum, T *partials, unsigned *counter, T &res) {
    __shared__ bool s_last;
    __shared__ T s_part[kRedThreads];
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bsum;
        __threadfence();
        s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
    T v = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) v += *(volatile T *)(partials + b);
    s_part[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) s_part[threadIdx.x] += s_part[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        res = s_part[0];
        *counter = 0;
    }
    return threadIdx.x == 0;
}

// ------------------------------------------------------------- FP64 norm

__global__ void __launch_bounds__(kRedThreads)
k_nrm2_f64(int n, const double *__restrict__ x, double *partials, unsigned *counter, double *out) {
    __shared__ double sh[32];
    double v = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += x[i] * x[i];
    v = block_sum(v, sh);
    double r;
    if (finish_reduce(v, partials, counter, r)) *out = sqrt(r);
}

struct RedBuf {
    double *partials = nullptr;
    unsigned *counter = nullptr;
    double *val = nullptr;
    int grid = 0;
};

static RedBuf &red_buf(Ctx &c) {
    static thread_local RedBuf rb;  // one per thread; sized for the largest grid
    if (!rb.partials) {
        rb.grid = c.num_sms * 4;
        rb.partials = (double *)dmalloc(sizeof(double) * rb.grid);
        rb.counter = (unsigned *)dmalloc(sizeof(unsigned) * 4);
        rb.val = (double *)dmalloc(sizeof(double) * 4);
        SAGB_CUDA(cudaMemset(rb.counter, 0, sizeof(unsigned) * 4));
    }
    return rb;
}

// ------------------------------------------- sequential-order reductions
//
// The sequential-order mode (SA_OPT_FP_EXACT) follows the reference's FP loops
// operation for operation: every product and sum rounded on its own (no fused
// multiply-add, which the compiler would otherwise form from a * b + c), each
// dot product and norm summed by one thread in index order as the reference's
// single-threaded build does (blas1.hpp:74-88).  It is a parity mode: one
// thread per reduction is slow at large sizes.

template <typename T>
__device__ __forceinline__ T rn_mul(T a, T b) {
    if constexpr (sizeof(T) == 8) return __dmul_rn(a, b);
    else return __fmul_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T rn_add(T a, T b) {
    if constexpr (sizeof(T) == 8) return __dadd_rn(a, b);
    else return __fadd_rn(a, b);
}
template <typename T>
__device__ __forceinline__ T rn_sub(T a, T b) {
    if constexpr (sizeof(T) == 8) return __dsub_rn(a, b);
    else return __fsub_rn(a, b);
}

// blas1::Dot / Nrm2 (blas1.hpp:74-88) in index order
template <typename T, bool NRM>
__global__ void k_dot_seq(int n, const T *__restrict__ x, const T *__restrict__ y, T *out) {
    if (threadIdx.x || blockIdx.x) return;
    T acc = 0;
    for (int i = 0; i < n; i++) acc = rn_add(acc, rn_mul(x[i], NRM ? x[i] : y[i]));
    *out = NRM ? (T)sqrt(acc) : acc;
}

void nrm2_f64_dev(Ctx &c, const double *x, int n, double *d_out) {
    if (c.fp_exact) {
        k_dot_seq<double, true><<<1, 32, 0, c.stream>>>(n, x, x, d_out);
    } else {
        RedBuf &rb = red_buf(c);
        k_nrm2_f64<<<rb.grid, kRedThreads, 0, c.stream>>>(n, x, rb.partials, rb.counter, d_out);
    }
    c.launches++;
}

double nrm2_f64(Ctx &c, const double *x, int n) {
    RedBuf &rb = red_buf(c);
    nrm2_f64_dev(c, x, n, rb.val);
    double h;
    SAGB_CUDA(cudaMemcpyAsync(&h, rb.val, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    return h;
}

// ================================================================= integer

struct IScal {
    double e0, e_inv, relres, nrm_b;
    long long criteria, hinv;
    int conv, pad;
};

struct StepInfo {  // read back by the host after every Arnoldi step
    int conv;
    unsigned flags;
    double relres;
};

__global__ void k_begin_i32(const double *e0p, double nrm_b, double eps, int bit, IScal *sc, long long *e,
                            unsigned long long *acc, int m) {
    const double e0 = *e0p;
    const double fact = (double)(1LL << bit);
    sc->e0 = e0;
    sc->e_inv = 1.0 / e0;
    sc->nrm_b = nrm_b;
    sc->criteria = d2l_x86(__dmul_rn(__dmul_rn(__dmul_rn(nrm_b, eps), sc->e_inv), fact));
    e[0] = 1LL << bit;
    for (int k = 0; k <= m + 1; k++) acc[k] = 0;
}

__global__ void k_v0_i32(int n, const double *__restrict__ r, const IScal *__restrict__ sc, int bit,
                         int *__restrict__ V0) {
    const double e_inv = sc->e_inv, fact = (double)(1LL << bit);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        V0[i] = d2i_x86(__dmul_rn(__dmul_rn(r[i], e_inv), fact));
}

// w = A z (CSR<Fixed<bit>> rows), and acc[0] += sum_i V0_i * w_i
template <int G>
__global__ void __launch_bounds__(kRedThreads)
k_spmv_dot_i32(int n, const int *__restrict__ rptr, const int *__restrict__ cind, const int *__restrict__ val,
               const int *__restrict__ z, int *__restrict__ w, const int *__restrict__ v0, int bit,
               unsigned long long *acc, unsigned *flags) {
    __shared__ long long sh[32];
    const long long tid = (long long)blockIdx.x * kRedThreads + threadIdx.x;
    const int row = (int)(tid / G), lane = (int)(tid % G);
    long long a = 0;
    if (row < n) {
        const int b0 = __ldg(rptr + row), b1 = __ldg(rptr + row + 1);
        for (int j = b0 + lane; j < b1; j += G) a = wadd(a, (long long)__ldg(val + j) * __ldg(z + __ldg(cind + j)));
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) a = wadd(a, shfl_xor(a, o));
    long long d = 0;
    if (lane == 0 && row < n) {
        const long long s = a >> bit;
        const int y = lo32(s);
        if (!fits32(s)) atomicOr(flags, ST_OVERFLOW);
        w[row] = y;
        d = (long long)__ldg(v0 + row) * y;
    }
    d = block_sum(d, sh);
    if (threadIdx.x == 0) atomicAdd(acc, (unsigned long long)d);
}

// the same through the tile-staged stream (short rows)
__global__ void __launch_bounds__(kStreamThreads)
k_spmv_dot_stream_i32(int n, const int *__restrict__ rptr, const int *__restrict__ cind, const int *__restrict__ val,
                      const int *__restrict__ z, int *__restrict__ w, const int *__restrict__ v0, int bit,
                      unsigned long long *acc, unsigned *flags) {
    __shared__ long long sh[32];
    long long a[1] = {0};
    const int r0 = blockIdx.x * kStreamThreads;
    stream_rows<1>(r0, min(n, r0 + kStreamThreads), rptr, cind, val, z, a);
    const int row = r0 + threadIdx.x;
    long long d = 0;
    if (row < n) {
        const long long s = a[0] >> bit;
        const int y = lo32(s);
        if (!fits32(s)) atomicOr(flags, ST_OVERFLOW);
        w[row] = y;
        d = (long long)__ldg(v0 + row) * y;
    }
    d = block_sum(d, sh);
    if (threadIdx.x == 0) atomicAdd(acc, (unsigned long long)d);
}

// MGS pass k of step j: h = acc[k] >> bit; H[j][k] = h; w += (int)((-h)*V_k >> bit);
// then acc[k+1] += dot(V_{k+1}, w), or acc[m+1] += dot(w, w) when k == j.
template <bool LAST>
__global__ void __launch_bounds__(kRedThreads)
k_mgs_i32(int n, int k, int j, int m, int bit, const int *__restrict__ V, int *__restrict__ w,
          unsigned long long *acc, long long *H) {
    __shared__ long long sh[32];
    const long long h = ((long long)acc[k]) >> bit;
    if (blockIdx.x == 0 && threadIdx.x == 0) H[(size_t)j * (m + 1) + k] = h;
    const long long a = wsub(0, h);
    const int *vk = V + (size_t)k * n;
    const int *vk1 = V + (size_t)(k + 1) * n;
    long long part = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int wi = (int)((unsigned)w[i] + (unsigned)lo32(wmul(a, (long long)__ldg(vk + i)) >> bit));
        w[i] = wi;
        if (LAST) part = wadd(part, (long long)wi * wi);
        else part = wadd(part, (long long)__ldg(vk1 + i) * wi);
    }
    part = block_sum(part, sh);
    if (threadIdx.x == 0) atomicAdd(acc + (LAST ? m + 1 : k + 1), (unsigned long long)part);
}

__device__ long long ggen_i32(long long a, long long b, long long *c, long long *s, int bit, unsigned *flags) {
    long long r = lsqrt_dev(wadd(wmul(a, a), wmul(b, b)));
    long long inv_r = 0;
    if (r == 0) atomicOr(flags, ST_DIVZERO);
    else inv_r = ((1LL << 62) / r) >> (62 - bit - bit);
    *c = wmul(a, inv_r) >> bit;
    *s = wsub(0, wmul(b, inv_r)) >> bit;
    return r;
}

// blas1::int32::Nrm2 / lsqrt, the H reciprocal, Grot/Ggen and the e update
// (gmres.hpp:325-334), then the convergence test (gmres.hpp:339)
// the step's status: the main word, plus the V-cycle's word with its int32
// wraps reported as ST_PREC_OVF (flags[0], flags[1] of the context)
__device__ __forceinline__ unsigned step_flags(const unsigned *flags) {
    const unsigned w0 = *(volatile const unsigned *)flags, w1 = *(volatile const unsigned *)(flags + 1);
    return w0 | (w1 & ~ST_OVERFLOW) | ((w1 & ST_OVERFLOW) ? ST_PREC_OVF : 0u);
}

__global__ void k_givens_i32(int j, int m, int bit, long long *H, long long *c, long long *s, long long *e,
                             IScal *sc, unsigned long long *acc, StepInfo *info, unsigned *flags) {
    long long *Hj = H + (size_t)j * (m + 1);
    const long long nsq = (long long)acc[m + 1];
    if (nsq < 0) atomicOr(flags, ST_NORM_OVF);
    Hj[j + 1] = lsqrt_dev(nsq);
    long long hinv = 0;
    if (Hj[j + 1] == 0) atomicOr(flags, ST_DIVZERO);
    else hinv = ((1LL << 62) / Hj[j + 1]) >> (62 - bit - bit);
    sc->hinv = hinv;
    for (int k = 0; k < j; k++) {
        const long long t = Hj[k];
        Hj[k] = wsub(wmul(c[k], t), wmul(s[k], Hj[k + 1])) >> bit;
        Hj[k + 1] = wadd(wmul(s[k], t), wmul(c[k], Hj[k + 1])) >> bit;
    }
    Hj[j] = ggen_i32(Hj[j], Hj[j + 1], &c[j], &s[j], bit, flags);
    Hj[j + 1] = 0;
    e[j + 1] = wmul(s[j], e[j]) >> bit;
    e[j] = wmul(c[j], e[j]) >> bit;
    const double fact = (double)(1LL << bit);
    const double relres = fabs(__ddiv_rn(__dmul_rn(sc->e0, (double)e[j + 1]), fact)) / sc->nrm_b;
    const long long en = e[j + 1];
    const long long aen = en < 0 ? wsub(0, en) : en;
    const int conv = aen <= sc->criteria;
    sc->conv = conv;
    sc->relres = relres;
    for (int k = 0; k <= m + 1; k++) acc[k] = 0;
    info->conv = conv;
    info->relres = relres;
    info->flags = step_flags(flags);
}

__global__ void k_scal_i32(int n, const IScal *__restrict__ sc, int bit, int *__restrict__ w) {
    const long long a = sc->hinv;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w[i] = lo32(wmul(a, (long long)w[i]) >> bit);
}

// blas2::int32::Trsv (blas2.hpp:366-376) on one thread
__global__ void k_trsv_i32(int jn, int m, int bit, const long long *H, const long long *e, const IScal *sc,
                           double *y) {
    const double fact = (double)(1LL << bit);
    const double e0 = sc->e0;
    for (int i = jn - 1; i >= 0; i--) {
        double t = __ddiv_rn(__dmul_rn(e0, (double)e[i]), fact);
        for (int q = jn - 1; q > i; q--) t = __dsub_rn(t, __dmul_rn(__ddiv_rn((double)H[(size_t)q * (m + 1) + i], fact), y[q]));
        y[i] = __ddiv_rn(t, __ddiv_rn((double)H[(size_t)i * (m + 1) + i], fact));
    }
}

// x += y_k * Z_k * 2^-bit for k = 0..jn-1 in order (Axpy_D, blas1.hpp:252-258)
__global__ void k_xupd_i32(int n, int jn, int bit, const double *__restrict__ y, const int *__restrict__ Z,
                           double *__restrict__ x) {
    __shared__ double sy[64];
    if (threadIdx.x < jn) sy[threadIdx.x] = y[threadIdx.x];
    __syncthreads();
    const double fi = 1.0 / (double)(1LL << bit);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double xi = x[i];
        for (int k = 0; k < jn; k++) xi = __dadd_rn(xi, __dmul_rn(__dmul_rn(sy[k], (double)Z[(size_t)k * n + i]), fi));
        x[i] = xi;
    }
}

// ====================================================================== FP

template <typename T>
struct FScal {
    double e0d;  // FP64 norm of r (the reference computes it in double)
    double e_inv;
    double nrm_b, eps;
    T a_scal;    // 1 / H_{j+1,j}
    T relres_t;
    int conv, pad;
    double relres;
};

template <typename T>
__global__ void k_begin_fp(const double *e0p, double nrm_b, double eps, FScal<T> *sc, T *e, int m) {
    const double e0 = *e0p;
    e[0] = (T)e0;  // FGMRES<float> stores the FP64 norm into a float (gmres.hpp:214)
    sc->e0d = e0;
    sc->e_inv = 1.0 / (double)e[0];
    sc->nrm_b = nrm_b;
    sc->eps = eps;
}

template <typename T>
__global__ void k_v0_fp(int n, const double *__restrict__ r, const FScal<T> *__restrict__ sc, T *__restrict__ V0) {
    const double e_inv = sc->e_inv;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        V0[i] = (T)__dmul_rn(r[i], e_inv);
}

template <typename T, int G>
__global__ void __launch_bounds__(kRedThreads)
k_spmv_dot_fp(int n, const int *__restrict__ rptr, const int *__restrict__ cind, const T *__restrict__ val,
              const T *__restrict__ z, T *__restrict__ w, const T *__restrict__ v0, T *partials,
              unsigned *counter, T *hout) {
    __shared__ T sh[32];
    const long long tid = (long long)blockIdx.x * kRedThreads + threadIdx.x;
    const int row = (int)(tid / G), lane = (int)(tid % G);
    T a = 0;
    if (row < n) {
        const int b0 = __ldg(rptr + row), b1 = __ldg(rptr + row + 1);
        for (int j = b0 + lane; j < b1; j += G) a += __ldg(val + j) * __ldg(z + __ldg(cind + j));
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) a += shfl_xor(a, o);
    T d = 0;
    if (lane == 0 && row < n) {
        w[row] = a;
        d = __ldg(v0 + row) * a;
    }
    d = block_sum(d, sh);
    T res;
    if (finish_reduce(d, partials, counter, res)) *hout = res;
}

// w += (-h) V_k, then H[j][k+1] = dot(V_{k+1}, w) or (k == j) ||w||
template <typename T, bool LAST>
__global__ void __launch_bounds__(kRedThreads)
k_mgs_fp(int n, int k, int j, int m, const T *__restrict__ V, T *__restrict__ w, T *H, T *partials,
         unsigned *counter) {
    __shared__ T sh[32];
    T *Hj = H + (size_t)j * (m + 1);
    const T a = -Hj[k];
    const T *vk = V + (size_t)k * n;
    const T *vk1 = V + (size_t)(k + 1) * n;
    T part = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const T wi = w[i] + a * __ldg(vk + i);
        w[i] = wi;
        part += LAST ? wi * wi : __ldg(vk1 + i) * wi;
    }
    part = block_sum(part, sh);
    T res;
    if (finish_reduce(part, partials, counter, res)) {
        if (LAST) Hj[j + 1] = sqrt(res);
        else Hj[k + 1] = res;
    }
}

template <typename T, bool EXACT = false>
__global__ void k_givens_fp(int j, int m, T *H, T *c, T *s, T *e, FScal<T> *sc, StepInfo *info,
                            unsigned *flags) {
    T *Hj = H + (size_t)j * (m + 1);
    if (Hj[j + 1] == 0) atomicOr(flags, ST_DIVZERO);
    sc->a_scal = (T)1 / Hj[j + 1];
    for (int k = 0; k < j; k++) {  // Grot (blas1.hpp:302-307)
        const T t = Hj[k];
        if constexpr (EXACT) {
            Hj[k] = rn_sub(rn_mul(c[k], t), rn_mul(s[k], Hj[k + 1]));
            Hj[k + 1] = rn_add(rn_mul(s[k], t), rn_mul(c[k], Hj[k + 1]));
        } else {
            Hj[k] = c[k] * t - s[k] * Hj[k + 1];
            Hj[k + 1] = s[k] * t + c[k] * Hj[k + 1];
        }
    }
    const T aa = Hj[j], bb = Hj[j + 1];  // Ggen (blas1.hpp:292-300)
    const T r = EXACT ? (T)sqrt(rn_add(rn_mul(aa, aa), rn_mul(bb, bb))) : (T)sqrt(aa * aa + bb * bb);
    c[j] = aa / r;
    s[j] = -bb / r;
    Hj[j] = r;
    Hj[j + 1] = 0;
    e[j + 1] = s[j] * e[j];
    e[j] = c[j] * e[j];
    const double relres = fabs((double)e[j + 1] / sc->nrm_b);
    const int conv = fabs((double)e[j + 1]) <= sc->nrm_b * sc->eps;
    sc->conv = conv;
    sc->relres = relres;
    info->conv = conv;
    info->relres = relres;
    info->flags = step_flags(flags);
}

template <typename T>
__global__ void k_scal_fp(int n, const FScal<T> *__restrict__ sc, T *__restrict__ w) {
    const T a = sc->a_scal;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) w[i] *= a;
}

// blas2::Trsv (blas2.hpp:25-34)
template <typename T, bool EXACT = false>
__global__ void k_trsv_fp(int jn, int m, const T *H, const T *e, T *y) {
    for (int i = jn - 1; i >= 0; i--) {
        T t = e[i];
        for (int q = jn - 1; q > i; q--) {
            if constexpr (EXACT) t = rn_sub(t, rn_mul(H[(size_t)q * (m + 1) + i], y[q]));
            else t -= H[(size_t)q * (m + 1) + i] * y[q];
        }
        y[i] = t / H[(size_t)i * (m + 1) + i];
    }
}

// x += y_k Z_k (Axpy<double>, or AxpyFD for float: (double)(y_k * z))
template <typename T, bool EXACT = false>
__global__ void k_xupd_fp(int n, int jn, const T *__restrict__ y, const T *__restrict__ Z, double *__restrict__ x) {
    __shared__ T sy[64];
    if (threadIdx.x < jn) sy[threadIdx.x] = y[threadIdx.x];
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double xi = x[i];
        for (int k = 0; k < jn; k++) {
            if constexpr (EXACT) xi = __dadd_rn(xi, (double)rn_mul(sy[k], Z[(size_t)k * n + i]));
            else xi += (double)(sy[k] * Z[(size_t)k * n + i]);
        }
        x[i] = xi;
    }
}

// w += (-h) x with h read on the device (Axpy, blas1.hpp:50-54), each
// product and sum rounded on its own
template <typename T>
__global__ void k_axpy_neg_rn(int n, const T *__restrict__ hp, const T *__restrict__ x, T *__restrict__ w) {
    const T a = -*hp;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        w[i] = rn_add(w[i], rn_mul(a, x[i]));
}

// ================================================================ driver

class GraphCache {
  public:
    ~GraphCache() { clear(); }
    void clear() {
        for (auto &g : execs)
            if (g) cudaGraphExecDestroy(g);
        execs.clear();
        counts.clear();
    }
    // run `body` (which enqueues on c.stream) through graph slot `slot`
    template <typename F>
    void run(Ctx &c, int slot, F &&body) {
        if (!c.use_graphs) {
            body();
            return;
        }
        if ((int)execs.size() <= slot) {
            execs.resize(slot + 1, nullptr);
            counts.resize(slot + 1, 0);
        }
        if (!execs[slot]) {
            cudaGraph_t g;
            const long long before = c.launches;
            SAGB_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            try {
                body();
            } catch (...) {
                cudaStreamEndCapture(c.stream, &g);
                throw;
            }
            SAGB_CUDA(cudaStreamEndCapture(c.stream, &g));
            SAGB_CUDA(cudaGraphInstantiate(&execs[slot], g, 0));
            cudaGraphDestroy(g);
            counts[slot] = c.launches - before;
            c.launches = before;
        }
        SAGB_CUDA(cudaGraphLaunch(execs[slot], c.stream));
        c.launches += counts[slot];
    }

  private:
    std::vector<cudaGraphExec_t> execs;
    std::vector<long long> counts;
};

static int grid_for(const Ctx &c, int n) {
    int b = (n + kRedThreads - 1) / kRedThreads;
    const int cap = c.num_sms * 4;
    return b < 1 ? 1 : (b > cap ? cap : b);
}

template <typename F>
static void by_group(int G, F &&f) {
    switch (G) {
        case 1: f(std::integral_constant<int, 1>()); break;
        case 2: f(std::integral_constant<int, 2>()); break;
        case 4: f(std::integral_constant<int, 4>()); break;
        case 8: f(std::integral_constant<int, 8>()); break;
        case 16: f(std::integral_constant<int, 16>()); break;
        default: f(std::integral_constant<int, 32>()); break;
    }
}

// Common Restarted loop; the inner cycle is precision specific.
class SolverBase : public Solver {
  public:
    SolverBase(Ctx &c, const DevCsr *dA, const KrylovParams &p) : c_(c), dA_(dA), p_(p) {
        N_ = dA->n;
        r_ = (double *)dmalloc(sizeof(double) * (size_t)N_);
        nrm_ = (double *)dmalloc(sizeof(double) * 2);
        SAGB_CUDA(cudaMallocHost(&info_h_, sizeof(StepInfo)));
        info_d_ = (StepInfo *)dmalloc(sizeof(StepInfo));
        SAGB_CUDA(cudaMallocHost(&nrm_h_, sizeof(double)));
    }
    ~SolverBase() override {
        dfree(r_);
        dfree(nrm_);
        dfree(info_d_);
        cudaFreeHost(info_h_);
        cudaFreeHost(nrm_h_);
    }
    void set_bit(int bit) override {
        p_.bit = bit;
        graphs_.clear();
    }

    int solve(const double *b, double nrm_b, double *x, SolveStats &st) override {
        double prev = 0;
        int iter = 0;
        st = SolveStats();
        SAGB_CUDA(cudaMemsetAsync(c_.d_flags_main, 0, 2 * sizeof(unsigned), c_.stream));
        for (int i = 0; i < p_.max_outer; i++) {
            spmv_resid_f64_exact(c_, *dA_, x, b, r_);
            nrm2_f64_dev(c_, r_, N_, nrm_);
            SAGB_CUDA(cudaMemcpyAsync(nrm_h_, nrm_, sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
            SAGB_CUDA(cudaStreamSynchronize(c_.stream));
            const double nrm_r = *nrm_h_;
            st.restarts++;
            st.explicit_res = nrm_r / nrm_b;
            if (p_.explicit_check && i > 0 && nrm_r <= p_.eps * nrm_b) {
                // explicit relative residual reached: stop here rather than on
                // the inner solver's implicit estimate
                st.converged = 1;
                st.iters = iter;
                return iter;
            }
            if (std::fabs(nrm_r - prev) / nrm_r < 1.0e-8) {
                st.converged = 0;
                st.iters = 0;
                return 0;
            }
            prev = nrm_r;
            int conv = 0;
            int it = run_cycle(r_, nrm_, nrm_b, x, &conv, nullptr, st);
            while (it < 0) {
                // the cycle overflowed and was discarded: one fractional bit
                // less, same residual (the reference would continue on
                // wrapped values or stop with a division by zero)
                if (p_.bit <= 1) {
                    st.final_bit = p_.bit;
                    return 0;
                }
                set_bit(p_.bit - 1);
                st.fallbacks++;
                SAGB_CUDA(cudaMemsetAsync(c_.d_flags_main, 0, 2 * sizeof(unsigned), c_.stream));
                it = run_cycle(r_, nrm_, nrm_b, x, &conv, nullptr, st);
            }
            st.final_bit = p_.bit;
            if (st.flags & ST_TIMEOUT) return 0;
            iter += it;
            if (conv && !p_.explicit_check) {
                st.converged = 1;
                st.iters = iter;
                return iter;
            }
        }
        if (p_.explicit_check) {
            // the last cycle's update has not been checked yet
            spmv_resid_f64_exact(c_, *dA_, x, b, r_);
            nrm2_f64_dev(c_, r_, N_, nrm_);
            SAGB_CUDA(cudaMemcpyAsync(nrm_h_, nrm_, sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
            SAGB_CUDA(cudaStreamSynchronize(c_.stream));
            st.explicit_res = *nrm_h_ / nrm_b;
            if (*nrm_h_ <= p_.eps * nrm_b) {
                st.converged = 1;
                st.iters = iter;
                return iter;
            }
        }
        st.converged = 0;
        st.iters = 0;
        return 0;
    }

    int cycle(const double *r, double nrm_b, double *x, const double *e0, int *converged,
              void *const *dumps) override {
        SolveStats st;
        double *e0d = nrm_;
        if (e0) {
            SAGB_CUDA(cudaMemcpyAsync(nrm_, e0, sizeof(double), cudaMemcpyHostToDevice, c_.stream));
        } else {
            nrm2_f64_dev(c_, r, N_, nrm_);
        }
        return run_cycle(r, e0d, nrm_b, x, converged, dumps, st);
    }

  protected:
    virtual int run_cycle(const double *r, const double *e0d, double nrm_b, double *x, int *conv,
                          void *const *dumps, SolveStats &st) = 0;

    // one Arnoldi step through its graph, then read the step status
    template <typename F>
    StepInfo step(int j, F &&body) {
        graphs_.run(c_, j, [&] {
            body();
            SAGB_CUDA(cudaMemcpyAsync(info_h_, info_d_, sizeof(StepInfo), cudaMemcpyDeviceToHost, c_.stream));
        });
        SAGB_CUDA(cudaStreamSynchronize(c_.stream));
        return *info_h_;
    }

    Ctx &c_;
    const DevCsr *dA_;
    KrylovParams p_;
    int N_ = 0;
    double *r_ = nullptr, *nrm_ = nullptr;
    StepInfo *info_h_ = nullptr, *info_d_ = nullptr;
    double *nrm_h_ = nullptr;
    GraphCache graphs_;
};

class IntSolver : public SolverBase {
  public:
    IntSolver(Ctx &c, const DevCsr *dA, const DevCsr *A, DevAmg *M, const KrylovParams &p)
        : SolverBase(c, dA, p), A_(A), M_(M) {
        const int m = p.m;
        V_ = (int *)dmalloc(sizeof(int) * (size_t)N_ * (m + 1));
        Z_ = (int *)dmalloc(sizeof(int) * (size_t)N_ * (m + 1));
        H_ = (long long *)dmalloc(sizeof(long long) * (size_t)(m + 1) * m);
        cs_ = (long long *)dmalloc(sizeof(long long) * (size_t)m);
        sn_ = (long long *)dmalloc(sizeof(long long) * (size_t)m);
        e_ = (long long *)dmalloc(sizeof(long long) * (size_t)(m + 1));
        y_ = (double *)dmalloc(sizeof(double) * (size_t)m);
        acc_ = (unsigned long long *)dmalloc(sizeof(unsigned long long) * (size_t)(m + 2));
        sc_ = (IScal *)dmalloc(sizeof(IScal));
        SAGB_CUDA(cudaMemset(H_, 0, sizeof(long long) * (size_t)(m + 1) * m));
    }
    ~IntSolver() override {
        dfree(V_); dfree(Z_); dfree(H_); dfree(cs_); dfree(sn_); dfree(e_); dfree(y_); dfree(acc_); dfree(sc_);
    }

  protected:
    int run_cycle(const double *r, const double *e0d, double nrm_b, double *x, int *conv, void *const *dumps,
                  SolveStats &st) override {
        const int m = p_.m, bit = p_.bit, N = N_;
        const int gb = grid_for(c_, N);
        k_begin_i32<<<1, 1, 0, c_.stream>>>(e0d, nrm_b, p_.eps, bit, sc_, e_, acc_, m);
        k_v0_i32<<<gb, kRedThreads, 0, c_.stream>>>(N, r, sc_, bit, V_);
        c_.launches += 2;
        int j, flag = 0;
        for (j = 0; j < m; j++) {
            int *vj = V_ + (size_t)j * N, *zj = Z_ + (size_t)j * N, *w = V_ + (size_t)(j + 1) * N;
            StepInfo inf = step(j, [&] {
                vcycle(c_, *M_, vj, zj);
                if (A_->group == 0) {
                    k_spmv_dot_stream_i32<<<(N + kStreamThreads - 1) / kStreamThreads, kStreamThreads, 0,
                                            c_.stream>>>(N, A_->rptr, A_->cind, (const int *)A_->val, zj, w, V_,
                                                         A_->bit, acc_, c_.d_flags);
                } else {
                    by_group(A_->group, [&](auto G) {
                        const long long thr = (long long)N * G.value;
                        const int blocks = (int)((thr + kRedThreads - 1) / kRedThreads);
                        k_spmv_dot_i32<G.value><<<blocks, kRedThreads, 0, c_.stream>>>(
                            N, A_->rptr, A_->cind, (const int *)A_->val, zj, w, V_, A_->bit, acc_, c_.d_flags);
                    });
                }
                for (int k = 0; k < j; k++)
                    k_mgs_i32<false><<<gb, kRedThreads, 0, c_.stream>>>(N, k, j, m, bit, V_, w, acc_, H_);
                k_mgs_i32<true><<<gb, kRedThreads, 0, c_.stream>>>(N, j, j, m, bit, V_, w, acc_, H_);
                k_givens_i32<<<1, 1, 0, c_.stream>>>(j, m, bit, H_, cs_, sn_, e_, sc_, acc_, info_d_, c_.d_flags);
                k_scal_i32<<<gb, kRedThreads, 0, c_.stream>>>(N, sc_, bit, w);
                c_.launches += j + 4;
            });
            st.flags |= inf.flags;
            st.history.push_back(inf.relres);
            if (p_.verbose) printf("# [%d] %e\n", j + 1, inf.relres);
            const unsigned bad = ST_OVERFLOW | ST_DIVZERO | ST_NORM_OVF;
            if (p_.fallback && (inf.flags & bad) && !dumps) {
                st.flags |= inf.flags;
                return -1;  // discard this cycle; the caller lowers the bit
            }
            if (inf.flags & (ST_TIMEOUT | ST_DIVZERO | ST_NORM_OVF)) {
                j++;
                break;
            }
            if (inf.conv) {
                if (p_.verbose) printf("[Res] : %e\n", inf.relres);
                j++;
                flag = 1;
                break;
            }
        }
        k_trsv_i32<<<1, 1, 0, c_.stream>>>(j, m, bit, H_, e_, sc_, y_);
        k_xupd_i32<<<gb, kRedThreads, 0, c_.stream>>>(N, j, bit, y_, Z_, x);
        c_.launches += 2;
        if (dumps) dump(dumps);
        SAGB_CUDA(cudaStreamSynchronize(c_.stream));
        *conv = flag;
        return flag ? j : m;
    }

    void dump(void *const *d) {
        const int m = p_.m;
        const size_t NN = (size_t)N_;
        if (d[0]) SAGB_CUDA(cudaMemcpyAsync(d[0], V_, 4 * NN * (m + 1), cudaMemcpyDeviceToHost, c_.stream));
        if (d[1]) SAGB_CUDA(cudaMemcpyAsync(d[1], Z_, 4 * NN * (m + 1), cudaMemcpyDeviceToHost, c_.stream));
        if (d[2]) SAGB_CUDA(cudaMemcpyAsync(d[2], H_, 8 * (size_t)(m + 1) * m, cudaMemcpyDeviceToHost, c_.stream));
        if (d[3]) SAGB_CUDA(cudaMemcpyAsync(d[3], cs_, 8 * (size_t)m, cudaMemcpyDeviceToHost, c_.stream));
        if (d[4]) SAGB_CUDA(cudaMemcpyAsync(d[4], sn_, 8 * (size_t)m, cudaMemcpyDeviceToHost, c_.stream));
        if (d[5]) SAGB_CUDA(cudaMemcpyAsync(d[5], e_, 8 * (size_t)(m + 1), cudaMemcpyDeviceToHost, c_.stream));
        if (d[6]) SAGB_CUDA(cudaMemcpyAsync(d[6], y_, 8 * (size_t)m, cudaMemcpyDeviceToHost, c_.stream));
    }

  private:
    const DevCsr *A_;
    DevAmg *M_;
    int *V_ = nullptr, *Z_ = nullptr;
    long long *H_ = nullptr, *cs_ = nullptr, *sn_ = nullptr, *e_ = nullptr;
    double *y_ = nullptr;
    unsigned long long *acc_ = nullptr;
    IScal *sc_ = nullptr;
};

template <typename T>
class FpSolver : public SolverBase {
  public:
    FpSolver(Ctx &c, const DevCsr *dA, const DevCsr *A, DevAmg *M, const KrylovParams &p)
        : SolverBase(c, dA, p), A_(A), M_(M) {
        const int m = p.m;
        V_ = (T *)dmalloc(sizeof(T) * (size_t)N_ * (m + 1));
        Z_ = (T *)dmalloc(sizeof(T) * (size_t)N_ * (m + 1));
        H_ = (T *)dmalloc(sizeof(T) * (size_t)(m + 1) * m);
        cs_ = (T *)dmalloc(sizeof(T) * (size_t)m);
        sn_ = (T *)dmalloc(sizeof(T) * (size_t)m);
        e_ = (T *)dmalloc(sizeof(T) * (size_t)(m + 1));
        y_ = (T *)dmalloc(sizeof(T) * (size_t)m);
        sc_ = (FScal<T> *)dmalloc(sizeof(FScal<T>));
        const int gb = grid_for(c, N_);
        partials_ = (T *)dmalloc(sizeof(T) * (size_t)std::max(gb, (int)((N_ * 32LL + kRedThreads - 1) / kRedThreads)));
        counter_ = (unsigned *)dmalloc(sizeof(unsigned) * 2);
        SAGB_CUDA(cudaMemset(counter_, 0, sizeof(unsigned) * 2));
        SAGB_CUDA(cudaMemset(H_, 0, sizeof(T) * (size_t)(m + 1) * m));
    }
    ~FpSolver() override {
        dfree(V_); dfree(Z_); dfree(H_); dfree(cs_); dfree(sn_); dfree(e_); dfree(y_); dfree(sc_);
        dfree(partials_); dfree(counter_);
    }

  protected:
    int run_cycle(const double *r, const double *e0d, double nrm_b, double *x, int *conv, void *const *dumps,
                  SolveStats &st) override {
        const int m = p_.m, N = N_;
        const int gb = grid_for(c_, N);
        const bool exact = c_.fp_exact;
        if (exact != graphs_exact_) {  // the step graphs hold one mode's kernels
            graphs_.clear();
            graphs_exact_ = exact;
        }
        k_begin_fp<T><<<1, 1, 0, c_.stream>>>(e0d, nrm_b, p_.eps, sc_, e_, m);
        k_v0_fp<T><<<gb, kRedThreads, 0, c_.stream>>>(N, r, sc_, V_);
        c_.launches += 2;
        int j, flag = 0;
        for (j = 0; j < m; j++) {
            T *vj = V_ + (size_t)j * N, *zj = Z_ + (size_t)j * N, *w = V_ + (size_t)(j + 1) * N;
            T *Hj = H_ + (size_t)j * (m + 1);
            StepInfo inf = step(j, [&] {
                vcycle(c_, *M_, vj, zj);
                if (exact) {
                    // the reference's order: SpMV, then per k Dot and Axpy, Nrm2
                    spmv(c_, *A_, zj, w);
                    for (int k = 0; k <= j; k++) {
                        k_dot_seq<T, false><<<1, 32, 0, c_.stream>>>(N, V_ + (size_t)k * N, w, Hj + k);
                        k_axpy_neg_rn<T><<<gb, kRedThreads, 0, c_.stream>>>(N, Hj + k, V_ + (size_t)k * N, w);
                    }
                    k_dot_seq<T, true><<<1, 32, 0, c_.stream>>>(N, w, w, Hj + j + 1);
                    k_givens_fp<T, true><<<1, 1, 0, c_.stream>>>(j, m, H_, cs_, sn_, e_, sc_, info_d_, c_.d_flags);
                    c_.launches += 2 * j + 4;
                } else {
                    by_group(A_->group, [&](auto G) {
                        const long long thr = (long long)N * G.value;
                        const int blocks = (int)((thr + kRedThreads - 1) / kRedThreads);
                        k_spmv_dot_fp<T, G.value><<<blocks, kRedThreads, 0, c_.stream>>>(
                            N, A_->rptr, A_->cind, (const T *)A_->val, zj, w, V_, partials_, counter_, Hj);
                    });
                    for (int k = 0; k < j; k++)
                        k_mgs_fp<T, false><<<gb, kRedThreads, 0, c_.stream>>>(N, k, j, m, V_, w, H_, partials_,
                                                                             counter_);
                    k_mgs_fp<T, true><<<gb, kRedThreads, 0, c_.stream>>>(N, j, j, m, V_, w, H_, partials_, counter_);
                    k_givens_fp<T><<<1, 1, 0, c_.stream>>>(j, m, H_, cs_, sn_, e_, sc_, info_d_, c_.d_flags);
                    c_.launches += j + 3;
                }
                k_scal_fp<T><<<gb, kRedThreads, 0, c_.stream>>>(N, sc_, w);
                c_.launches++;
            });
            st.flags |= inf.flags;
            st.history.push_back(inf.relres);
            if (p_.verbose) printf("# [%d] %e\n", j + 1, inf.relres);
            if (inf.flags & (ST_TIMEOUT | ST_DIVZERO)) {
                j++;
                break;
            }
            if (inf.conv) {
                if (p_.verbose) printf("[Res] : %e\n", inf.relres);
                j++;
                flag = 1;
                break;
            }
        }
        if (exact) {
            k_trsv_fp<T, true><<<1, 1, 0, c_.stream>>>(j, m, H_, e_, y_);
            k_xupd_fp<T, true><<<gb, kRedThreads, 0, c_.stream>>>(N, j, y_, Z_, x);
        } else {
            k_trsv_fp<T><<<1, 1, 0, c_.stream>>>(j, m, H_, e_, y_);
            k_xupd_fp<T><<<gb, kRedThreads, 0, c_.stream>>>(N, j, y_, Z_, x);
        }
        c_.launches += 2;
        SAGB_CUDA(cudaStreamSynchronize(c_.stream));
        (void)dumps;
        *conv = flag;
        return flag ? j : m;
    }

  private:
    const DevCsr *A_;
    DevAmg *M_;
    T *V_ = nullptr, *Z_ = nullptr, *H_ = nullptr, *cs_ = nullptr, *sn_ = nullptr, *e_ = nullptr, *y_ = nullptr;
    FScal<T> *sc_ = nullptr;
    T *partials_ = nullptr;
    unsigned *counter_ = nullptr;
    bool graphs_exact_ = false;
};

std::unique_ptr<Solver> make_solver(Ctx &c, int vt, const DevCsr *dA, const DevCsr *A, DevAmg *M,
                                    const KrylovParams &p) {
    if (vt == VT_I32) return std::make_unique<IntSolver>(c, dA, A, M, p);
    if (vt == VT_F64) return std::make_unique<FpSolver<double>>(c, dA, A, M, p);
    return std::make_unique<FpSolver<float>>(c, dA, A, M, p);
}

}  // namespace sagb
