// CSR SpMV kernels (int32 fixed point with int64 accumulation, FP64, FP32)
// and the small elementwise kernels of the V-cycle.
//
// Integer rows follow CSRflex::SpMV / CSR<Fixed<bit>>::SpMV
// (matrix/spmat.hpp:128-137, 77-86): y_i = (int)((sum_j (long)a_ij*(long)x_j) >> bit).
// The int64 sum wraps exactly like the reference's, so the lane split inside a
// row does not change any result.  A result outside int32 is stored wrapped
// (as the reference does) and raises ST_OVERFLOW.
#include <cstdio>
#include <stdexcept>

#include "../sagb_internal.hpp"
#include "common.cuh"
#include "stream.cuh"

namespace sagb {

void cuda_check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw CudaError{std::string(what) + ": " + cudaGetErrorString(e)};
}

void *dmalloc(size_t bytes) {
    void *p = nullptr;
    if (bytes == 0) bytes = 16;
    SAGB_CUDA(cudaMalloc(&p, bytes));
    return p;
}
void dfree(void *p) {
    if (p) cudaFree(p);
}

void DevCsr::release() {
    dfree(rptr);
    dfree(cind);
    dfree(val);
    rptr = cind = nullptr;
    val = nullptr;
}

// integer matrices with at most this many entries per row on average use the
// tile-staged stream kernel (group 0)
constexpr double kStreamMaxAvg = 32.0;

int pick_group(double avg) {
    // lanes per row: about the average row length, within [1, 32]
    int g = 1;
    while (g < 32 && g < avg * 0.75) g <<= 1;
    return g;
}

DevCsr upload_csr_i32(const CsrI &A) {
    DevCsr d;
    d.n = A.n;
    d.m = A.m;
    d.nnz = A.nnz();
    d.bit = A.bit;
    d.vt = VT_I32;
    d.rptr = dupload(A.rptr);
    d.cind = A.cind.empty() ? (int *)dmalloc(16) : dupload(A.cind);
    d.val = A.val.empty() ? dmalloc(16) : (void *)dupload(A.val);
    d.group = pick_group(A.n ? (double)d.nnz / A.n : 1.0);
    if (A.n && (double)d.nnz / A.n <= kStreamMaxAvg) d.group = 0;  // tile-staged stream
    return d;
}

template <typename T>
DevCsr upload_csr_fp(const CsrT<T> &A) {
    DevCsr d;
    d.n = A.n;
    d.m = A.m;
    d.nnz = A.nnz();
    d.vt = sizeof(T) == 8 ? VT_F64 : VT_F32;
    d.rptr = dupload(A.rptr);
    d.cind = A.cind.empty() ? (int *)dmalloc(16) : dupload(A.cind);
    d.val = A.val.empty() ? dmalloc(16) : (void *)dupload(A.val);
    d.group = pick_group(A.n ? (double)d.nnz / A.n : 1.0);
    return d;
}
template DevCsr upload_csr_fp<double>(const CsrT<double> &);
template DevCsr upload_csr_fp<float>(const CsrT<float> &);

DevCsr upload_csr_f64(const CsrD &A) {
    DevCsr d;
    d.n = A.n;
    d.m = A.m;
    d.nnz = A.nnz();
    d.vt = VT_F64;
    d.rptr = dupload(A.rptr);
    d.cind = dupload(A.cind);
    d.val = dupload(A.val);
    d.group = pick_group(A.n ? (double)d.nnz / A.n : 1.0);
    return d;
}

// ------------------------------------------------------------------ kernels

constexpr int kSpmvThreads = 256;

template <int G, int MODE>
__global__ void __launch_bounds__(kSpmvThreads)
k_spmv_i32(int n, const int *__restrict__ rptr, const int *__restrict__ cind, const int *__restrict__ val,
           const int *__restrict__ x, int *__restrict__ y, const int *__restrict__ z, int bit,
           unsigned *__restrict__ flags) {
    const long long tid = (long long)blockIdx.x * kSpmvThreads + threadIdx.x;
    const int row = (int)(tid / G);
    const int lane = (int)(tid % G);
    long long acc = 0;
    if (row < n) {
        const int a = __ldg(rptr + row), b = __ldg(rptr + row + 1);
        int j = a + lane;
        // four entries per lane in flight (integer sums wrap: any order gives the same result)
        for (; j + 3 * G < b; j += 4 * G) {
            const int c0 = __ldg(cind + j), c1 = __ldg(cind + j + G), c2 = __ldg(cind + j + 2 * G),
                      c3 = __ldg(cind + j + 3 * G);
            const long long v0 = __ldg(val + j), v1 = __ldg(val + j + G), v2 = __ldg(val + j + 2 * G),
                            v3 = __ldg(val + j + 3 * G);
            const long long x0 = __ldg(x + c0), x1 = __ldg(x + c1), x2 = __ldg(x + c2), x3 = __ldg(x + c3);
            acc = wadd(acc, wadd(wadd(v0 * x0, v1 * x1), wadd(v2 * x2, v3 * x3)));
        }
        for (; j < b; j += G) acc = wadd(acc, (long long)__ldg(val + j) * (long long)__ldg(x + __ldg(cind + j)));
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc = wadd(acc, shfl_xor(acc, o));
    if (lane == 0 && row < n) {
        const long long s = acc >> bit;
        bool ovf = !fits32(s);
        long long v = (long long)lo32(s);
        if (MODE == SPMV_RESID) v = (long long)z[row] - v;
        if (MODE == SPMV_ADD) v = v + (long long)y[row];
        ovf |= !fits32(v);
        y[row] = lo32(v);
        if (ovf) atomicOr(flags, ST_OVERFLOW);
    }
}

template <typename T, int G, int MODE, bool EXACT>
__global__ void __launch_bounds__(kSpmvThreads)
k_spmv_fp(int n, const int *__restrict__ rptr, const int *__restrict__ cind, const T *__restrict__ val,
          const T *__restrict__ x, T *__restrict__ y, const T *__restrict__ z) {
    const long long tid = (long long)blockIdx.x * kSpmvThreads + threadIdx.x;
    const int row = (int)(tid / G);
    const int lane = (int)(tid % G);
    T acc = 0;
    if (row < n) {
        const int a = __ldg(rptr + row), b = __ldg(rptr + row + 1);
        for (int j = a + lane; j < b; j += G) {
            const T p = __ldg(val + j), q = __ldg(x + __ldg(cind + j));
            if constexpr (EXACT) {
                if constexpr (sizeof(T) == 8) acc = __dadd_rn(acc, __dmul_rn(p, q));
                else acc = __fadd_rn(acc, __fmul_rn(p, q));
            } else {
                acc += p * q;
            }
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += shfl_xor(acc, o);
    if (lane == 0 && row < n) {
        T v = acc;
        if (MODE == SPMV_RESID) v = z[row] - v;
        if (MODE == SPMV_ADD) v = v + y[row];
        y[row] = v;
    }
}

// the same rows through the tile-staged stream (short rows)
template <int MODE>
__global__ void __launch_bounds__(kStreamThreads)
k_spmv_stream_i32(int n, const int *__restrict__ rptr, const int *__restrict__ cind, const int *__restrict__ val,
                  const int *__restrict__ x, int *__restrict__ y, const int *__restrict__ z, int bit,
                  unsigned *__restrict__ flags) {
    long long acc[1] = {0};
    const int r0 = blockIdx.x * kStreamThreads;
    stream_rows<1>(r0, min(n, r0 + kStreamThreads), rptr, cind, val, x, acc);
    const int row = r0 + threadIdx.x;
    if (row < n) {
        const long long s = acc[0] >> bit;
        bool ovf = !fits32(s);
        long long v = (long long)lo32(s);
        if (MODE == SPMV_RESID) v = (long long)z[row] - v;
        if (MODE == SPMV_ADD) v = v + (long long)y[row];
        ovf |= !fits32(v);
        y[row] = lo32(v);
        if (ovf) atomicOr(flags, ST_OVERFLOW);
    }
}

static void launch_stream_i32(Ctx &c, const DevCsr &A, const void *x, void *y, int mode, const void *z) {
    const int blocks = (A.n + kStreamThreads - 1) / kStreamThreads;
    if (blocks == 0) return;
    auto args = [&](auto kern) {
        kern<<<blocks, kStreamThreads, 0, c.stream>>>(A.n, A.rptr, A.cind, (const int *)A.val, (const int *)x,
                                                        (int *)y, (const int *)z, A.bit, c.d_flags);
    };
    if (mode == SPMV_SET) args(k_spmv_stream_i32<SPMV_SET>);
    else if (mode == SPMV_RESID) args(k_spmv_stream_i32<SPMV_RESID>);
    else args(k_spmv_stream_i32<SPMV_ADD>);
    c.launches++;
}

template <int G>
static void launch_i32(Ctx &c, const DevCsr &A, const void *x, void *y, int mode, const void *z) {
    const long long threads = (long long)A.n * G;
    const int blocks = (int)((threads + kSpmvThreads - 1) / kSpmvThreads);
    if (blocks == 0) return;
    auto args = [&](auto kern) {
        kern<<<blocks, kSpmvThreads, 0, c.stream>>>(A.n, A.rptr, A.cind, (const int *)A.val, (const int *)x,
                                                      (int *)y, (const int *)z, A.bit, c.d_flags);
    };
    if (mode == SPMV_SET) args(k_spmv_i32<G, SPMV_SET>);
    else if (mode == SPMV_RESID) args(k_spmv_i32<G, SPMV_RESID>);
    else args(k_spmv_i32<G, SPMV_ADD>);
    c.launches++;
}

template <typename T, int G, bool EXACT>
static void launch_fp(Ctx &c, const DevCsr &A, const void *x, void *y, int mode, const void *z) {
    const long long threads = (long long)A.n * G;
    const int blocks = (int)((threads + kSpmvThreads - 1) / kSpmvThreads);
    if (blocks == 0) return;
    auto args = [&](auto kern) {
        kern<<<blocks, kSpmvThreads, 0, c.stream>>>(A.n, A.rptr, A.cind, (const T *)A.val, (const T *)x, (T *)y,
                                                      (const T *)z);
    };
    if (mode == SPMV_SET) args(k_spmv_fp<T, G, SPMV_SET, EXACT>);
    else if (mode == SPMV_RESID) args(k_spmv_fp<T, G, SPMV_RESID, EXACT>);
    else args(k_spmv_fp<T, G, SPMV_ADD, EXACT>);
    c.launches++;
}

template <typename T>
static void dispatch_fp(Ctx &c, const DevCsr &A, const void *x, void *y, int mode, const void *z) {
    if (c.fp_exact) return launch_fp<T, 1, true>(c, A, x, y, mode, z);
    switch (A.group) {
        case 1: return launch_fp<T, 1, false>(c, A, x, y, mode, z);
        case 2: return launch_fp<T, 2, false>(c, A, x, y, mode, z);
        case 4: return launch_fp<T, 4, false>(c, A, x, y, mode, z);
        case 8: return launch_fp<T, 8, false>(c, A, x, y, mode, z);
        case 16: return launch_fp<T, 16, false>(c, A, x, y, mode, z);
        default: return launch_fp<T, 32, false>(c, A, x, y, mode, z);
    }
}

void spmv(Ctx &c, const DevCsr &A, const void *x, void *y, int mode, const void *z) {
    if (A.vt == VT_I32) {
        switch (A.group) {
            case 0: return launch_stream_i32(c, A, x, y, mode, z);
            case 1: return launch_i32<1>(c, A, x, y, mode, z);
            case 2: return launch_i32<2>(c, A, x, y, mode, z);
            case 4: return launch_i32<4>(c, A, x, y, mode, z);
            case 8: return launch_i32<8>(c, A, x, y, mode, z);
            case 16: return launch_i32<16>(c, A, x, y, mode, z);
            default: return launch_i32<32>(c, A, x, y, mode, z);
        }
    }
    if (A.vt == VT_F64) return dispatch_fp<double>(c, A, x, y, mode, z);
    return dispatch_fp<float>(c, A, x, y, mode, z);
}

void spmv_resid_f64_exact(Ctx &c, const DevCsr &A, const double *x, const double *b, double *r) {
    // r = 1*b + (-1)*(A x): the reference's Axpby<double>(1, b, -1, r) after a
    // row-sequential SpMV; 1*b and -1*t are exact, so this is b - t.
    launch_fp<double, 1, true>(c, A, x, r, SPMV_RESID, b);
}

// ------------------------------------------------------------- elementwise

template <typename T, bool SUB>
__global__ void k_vec_fp(int n, const T *__restrict__ x, T *__restrict__ y) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = SUB ? x[i] - y[i] : x[i] + y[i];
}
template <bool SUB>
__global__ void k_vec_i32(int n, const int *__restrict__ x, int *__restrict__ y, unsigned *flags) {
    bool ovf = false;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        long long v = SUB ? (long long)x[i] - y[i] : (long long)x[i] + y[i];
        ovf |= !fits32(v);
        y[i] = lo32(v);
    }
    if (ovf) atomicOr(flags, ST_OVERFLOW);
}

static int ew_blocks(const Ctx &c, int n) {
    int b = (n + 255) / 256;
    int cap = c.num_sms * 8;
    return b < 1 ? 1 : (b > cap ? cap : b);
}

void vec_sub(Ctx &c, int vt, int n, const void *x, void *y) {
    if (n <= 0) return;
    const int b = ew_blocks(c, n);
    if (vt == VT_I32) k_vec_i32<true><<<b, 256, 0, c.stream>>>(n, (const int *)x, (int *)y, c.d_flags);
    else if (vt == VT_F64) k_vec_fp<double, true><<<b, 256, 0, c.stream>>>(n, (const double *)x, (double *)y);
    else k_vec_fp<float, true><<<b, 256, 0, c.stream>>>(n, (const float *)x, (float *)y);
    c.launches++;
}
void vec_add(Ctx &c, int vt, int n, const void *x, void *y) {
    if (n <= 0) return;
    const int b = ew_blocks(c, n);
    if (vt == VT_I32) k_vec_i32<false><<<b, 256, 0, c.stream>>>(n, (const int *)x, (int *)y, c.d_flags);
    else if (vt == VT_F64) k_vec_fp<double, false><<<b, 256, 0, c.stream>>>(n, (const double *)x, (double *)y);
    else k_vec_fp<float, false><<<b, 256, 0, c.stream>>>(n, (const float *)x, (float *)y);
    c.launches++;
}

}  // namespace sagb
