// Sparse triangular sweeps (Gauss-Seidel / SOR smoothing and the coarse LU
// solve) in the reference's dependency order.
//
// Integer sweeps follow ldtri::CSRflex::SpTRSV (matrix/trimat/ldtri.hpp:172-183),
// its block-Jacobi form BJCSRflex (ldtri.hpp:511-525), ltri::CSRflex
// (ltri.hpp:125-133) and dutri::CSRflex (dutri.hpp:146-156):
//   t = in_i << bit;  t -= sum_j a_ij * out_j;  out_i = (int)((t >> bit) * dinv_i >> dbit)
// (ltri: out_i = (int)(t >> bit)).  FP sweeps follow the CSR<T> classes.
//
// Sync-free schedule: rows are stored in level order and cut into chunks
// (host/schedule.hpp).  A CTA claims chunks with an atomic ticket, and a row
// waits only for the rows it reads.  Integer and FP32 results are published as
// one 64-bit word {epoch, value}, so a dependency costs a single L2 load; FP64
// results use a separate epoch flag with release/acquire ordering.  The epoch
// and the ticket live in device memory and are advanced by the last CTA, so
// the kernel can be replayed from a CUDA graph.  Every wait is bounded in time
// (ST_TIMEOUT), and once any wait has timed out all CTAs stop waiting.
#include <algorithm>
#include <type_traits>

#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {

constexpr int kTriThreads = 256;

struct TriArgs {
    int n, nchunks, bit, dbit;
    const int *perm, *prp, *pci;
    const void *pval, *dinv;
    const int *chunk_lv, *sub_bound;
    unsigned long long *pk;
    unsigned *flag;
    TriSync *sync;
};

__device__ __forceinline__ bool aborted(const unsigned *flags) {
    return (*(volatile const unsigned *)flags & ST_TIMEOUT) != 0;
}

// wait until the packed word of row c carries epoch ep; returns the word
__device__ __forceinline__ unsigned long long wait_packed(unsigned long long *pk, int c, unsigned ep,
                                                          unsigned *flags) {
    unsigned long long w = ld_relaxed_u64(pk + c);
    if ((unsigned)(w >> 32) == ep) return w;
    const unsigned long long t0 = globaltimer_ns();
    unsigned it = 0;
    for (;;) {
        w = ld_relaxed_u64(pk + c);
        if ((unsigned)(w >> 32) == ep) return w;
        if ((++it & 63u) == 0) {
            if (aborted(flags)) return w;
            if (globaltimer_ns() - t0 > kSpinLimitNs) {
                atomicOr(flags, ST_TIMEOUT);
                return w;
            }
        }
    }
}

__device__ __forceinline__ void wait_flag(const unsigned *flag, int c, unsigned ep, unsigned *flags) {
    if (ld_acquire_u32(flag + c) == ep) return;
    const unsigned long long t0 = globaltimer_ns();
    unsigned it = 0;
    for (;;) {
        if (ld_acquire_u32(flag + c) == ep) return;
        if ((++it & 63u) == 0) {
            if (aborted(flags)) return;
            if (globaltimer_ns() - t0 > kSpinLimitNs) {
                atomicOr(flags, ST_TIMEOUT);
                return;
            }
        }
    }
}

__device__ __forceinline__ double ld_relaxed_f64(const double *p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}

// one row of a sweep, G lanes per row.  VT: 0 int32, 1 f64, 2 f32.
template <int VT, int KIND, int G, bool EXACT>
__device__ __forceinline__ void tri_row(const TriArgs &a, int p, bool valid, int g, unsigned ep, const void *in_,
                                        void *out_, unsigned *flags, bool &ovf) {
    if constexpr (VT == VT_I32) {
        const int *in = (const int *)in_;
        int *out = (int *)out_;
        long long t = 0;
        int row = 0;
        if (valid) {
            row = __ldg(a.perm + p);
            if (g == 0) t = wshl((long long)__ldg(in + row), a.bit);
            const int *pv = (const int *)a.pval;
            for (int j = __ldg(a.prp + p) + g; j < __ldg(a.prp + p + 1); j += G) {
                const int c = __ldg(a.pci + j);
                const long long v = __ldg(pv + j);
                const unsigned long long w = wait_packed(a.pk, c, ep, flags);
                t = wsub(t, v * (long long)(int)(unsigned)w);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) t = wadd(t, shfl_xor(t, o));
        if (valid && g == 0) {
            long long s;
            if (KIND == TRI_L) s = t >> a.bit;
            else s = wmul(t >> a.bit, (long long)__ldg((const int *)a.dinv + p)) >> a.dbit;
            const int o = lo32(s);
            ovf |= !fits32(s);
            out[row] = o;
            st_relaxed_u64(a.pk + row, ((unsigned long long)ep << 32) | (unsigned)o);
        }
    } else {
        using T = typename std::conditional<VT == VT_F64, double, float>::type;
        const T *in = (const T *)in_;
        T *out = (T *)out_;
        T t = 0;
        int row = 0;
        if (valid) {
            row = __ldg(a.perm + p);
            if (g == 0) t = __ldg(in + row);
            const T *pv = (const T *)a.pval;
            for (int j = __ldg(a.prp + p) + g; j < __ldg(a.prp + p + 1); j += G) {
                const int c = __ldg(a.pci + j);
                const T v = __ldg(pv + j);
                T o;
                if constexpr (VT == VT_F64) {
                    wait_flag(a.flag, c, ep, flags);
                    o = ld_relaxed_f64((const double *)out + c);
                } else {
                    const unsigned long long w = wait_packed(a.pk, c, ep, flags);
                    o = __uint_as_float((unsigned)w);
                }
                if constexpr (EXACT) {
                    if constexpr (VT == VT_F64) t = __dsub_rn(t, __dmul_rn(v, o));
                    else t = __fsub_rn(t, __fmul_rn(v, o));
                } else {
                    t -= v * o;
                }
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) t += shfl_xor(t, o);
        if (valid && g == 0) {
            T r = t;
            if (KIND != TRI_L) {
                const T d = __ldg((const T *)a.dinv + p);
                if constexpr (VT == VT_F64) r = __dmul_rn(t, d);
                else r = __fmul_rn(t, d);
            }
            out[row] = r;
            if constexpr (VT == VT_F64) {
                st_release_u32(a.flag + row, ep);
            } else {
                st_relaxed_u64(a.pk + row, ((unsigned long long)ep << 32) | __float_as_uint(r));
            }
        }
    }
}

template <int VT, int KIND, int G, bool EXACT>
__global__ void __launch_bounds__(kTriThreads) k_tri(TriArgs a, const void *in, void *out, unsigned *flags) {
    __shared__ int s_chunk;
    __shared__ unsigned s_epoch;
    if (threadIdx.x == 0) s_epoch = ld_acquire_u32(&a.sync->epoch) + 1;
    __syncthreads();
    const unsigned ep = s_epoch;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int RPW = 32 / G;  // rows per warp per pass
    constexpr int NW = kTriThreads / 32;
    const int g = lane % G, sub = lane / G;
    bool ovf = false;
    for (;;) {
        if (threadIdx.x == 0) s_chunk = aborted(flags) ? a.nchunks : (int)atomicAdd(&a.sync->ticket, 1u);
        __syncthreads();
        const int ch = s_chunk;
        if (ch >= a.nchunks) break;
        const int s0 = __ldg(a.chunk_lv + ch), s1 = __ldg(a.chunk_lv + ch + 1);
        for (int s = s0; s < s1; s++) {
            const int p0 = __ldg(a.sub_bound + s), p1 = __ldg(a.sub_bound + s + 1);
            for (int base = p0 + warp * RPW; base < p1; base += NW * RPW) {
                const int p = base + sub;
                tri_row<VT, KIND, G, EXACT>(a, p, p < p1, g, ep, in, out, flags, ovf);
            }
            if (s + 1 < s1) __syncthreads();
        }
        __syncthreads();
    }
    if (ovf) atomicOr(flags, ST_OVERFLOW);
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned d = atomicAdd(&a.sync->done, 1u);
        if (d == gridDim.x - 1) {
            a.sync->ticket = 0;
            a.sync->done = 0;
            __threadfence();
            st_release_u32(&a.sync->epoch, ep);
        }
    }
}

void DevTri::release() {
    dfree(perm);
    dfree(prp);
    dfree(pci);
    dfree(pval);
    dfree(dinv);
    dfree(chunk_lv);
    dfree(sub_bound);
    dfree(pk);
    dfree(flag);
    dfree(sync);
    perm = prp = pci = chunk_lv = sub_bound = nullptr;
    pval = dinv = nullptr;
    pk = nullptr;
    flag = nullptr;
    sync = nullptr;
}

template <typename T>
static void gather_vals(const TriSchedule &s, const T *vals, std::vector<T> &pv, std::vector<T> &dv) {
    pv.resize(s.src_idx.size());
    for (size_t j = 0; j < s.src_idx.size(); j++) pv[j] = vals[s.src_idx[j]];
    dv.assign(s.n, T(0));
    for (int p = 0; p < s.n; p++)
        if (s.diag_src[p] >= 0) dv[p] = vals[s.diag_src[p]];
}

DevTri upload_tri(const Ctx &c, int n, const int *rptr, const int *cind, const void *vals, int vt, int kind,
                  int bit, int dbit) {
    DevTri d;
    d.n = n;
    d.kind = kind;
    d.vt = vt;
    d.bit = bit;
    d.dbit = dbit;
    const int64_t nnz = n ? rptr[n] : 0;
    const int64_t offd = nnz - (kind == TRI_L ? 0 : n);
    const double avg = n ? (double)offd / n : 0.0;
    int G = pick_group(avg * 0.5);
    if (vt != VT_I32 && c.fp_exact) G = 1;
    d.group = G;
    const int rows_per_chunk = 2 * kTriThreads / G;
    TriSchedule s = build_tri_schedule(rptr, cind, n, kind, rows_per_chunk, 1 << 20);
    d.nlev = s.nlev;
    d.max_level_rows = s.max_level_rows;
    d.nnz_off = (int64_t)s.pci.size();
    d.nchunks = s.nchunks();
    d.perm = dupload(s.perm);
    d.prp = dupload(s.prp);
    d.pci = s.pci.empty() ? (int *)dmalloc(16) : dupload(s.pci);
    if (vt == VT_I32) {
        std::vector<int32_t> pv, dv;
        gather_vals(s, (const int32_t *)vals, pv, dv);
        d.pval = pv.empty() ? dmalloc(16) : (void *)dupload(pv);
        d.dinv = dupload(dv);
    } else if (vt == VT_F64) {
        std::vector<double> pv, dv;
        gather_vals(s, (const double *)vals, pv, dv);
        d.pval = pv.empty() ? dmalloc(16) : (void *)dupload(pv);
        d.dinv = dupload(dv);
    } else {
        std::vector<float> pv, dv;
        gather_vals(s, (const float *)vals, pv, dv);
        d.pval = pv.empty() ? dmalloc(16) : (void *)dupload(pv);
        d.dinv = dupload(dv);
    }
    d.chunk_lv = dupload(s.chunk_lv);
    d.sub_bound = dupload(s.sub_bound);
    if (vt == VT_F64) {
        d.flag = (unsigned *)dmalloc(sizeof(unsigned) * std::max(n, 1));
        SAGB_CUDA(cudaMemset(d.flag, 0, sizeof(unsigned) * std::max(n, 1)));
    } else {
        d.pk = (unsigned long long *)dmalloc(sizeof(unsigned long long) * std::max(n, 1));
        SAGB_CUDA(cudaMemset(d.pk, 0, sizeof(unsigned long long) * std::max(n, 1)));
    }
    d.sync = (TriSync *)dmalloc(sizeof(TriSync));
    SAGB_CUDA(cudaMemset(d.sync, 0, sizeof(TriSync)));
    d.grid = std::max(1, std::min(d.nchunks, c.num_sms * 4));
    return d;
}

template <int VT, int KIND, int G, bool EXACT>
static void launch_tri(Ctx &c, const DevTri &T, const void *in, void *out) {
    TriArgs a{T.n, T.nchunks, T.bit, T.dbit, T.perm, T.prp, T.pci, T.pval, T.dinv,
              T.chunk_lv, T.sub_bound, T.pk, T.flag, T.sync};
    k_tri<VT, KIND, G, EXACT><<<T.grid, kTriThreads, 0, c.stream>>>(a, in, out, c.d_flags);
    c.launches++;
}

template <int VT, int KIND, bool EXACT>
static void tri_by_group(Ctx &c, const DevTri &T, const void *in, void *out) {
    switch (T.group) {
        case 1: return launch_tri<VT, KIND, 1, EXACT>(c, T, in, out);
        case 2: return launch_tri<VT, KIND, 2, EXACT>(c, T, in, out);
        case 4: return launch_tri<VT, KIND, 4, EXACT>(c, T, in, out);
        case 8: return launch_tri<VT, KIND, 8, EXACT>(c, T, in, out);
        case 16: return launch_tri<VT, KIND, 16, EXACT>(c, T, in, out);
        default: return launch_tri<VT, KIND, 32, EXACT>(c, T, in, out);
    }
}

template <int VT, bool EXACT>
static void tri_by_kind(Ctx &c, const DevTri &T, const void *in, void *out) {
    if (T.kind == TRI_LD) tri_by_group<VT, TRI_LD, EXACT>(c, T, in, out);
    else if (T.kind == TRI_L) tri_by_group<VT, TRI_L, EXACT>(c, T, in, out);
    else tri_by_group<VT, TRI_DU, EXACT>(c, T, in, out);
}

void trsv(Ctx &c, const DevTri &T, const void *in, void *out) {
    if (T.n == 0) return;
    if (T.vt == VT_I32) return tri_by_kind<VT_I32, false>(c, T, in, out);
    if (T.vt == VT_F64) {
        if (c.fp_exact) return tri_by_kind<VT_F64, true>(c, T, in, out);
        return tri_by_kind<VT_F64, false>(c, T, in, out);
    }
    if (c.fp_exact) return tri_by_kind<VT_F32, true>(c, T, in, out);
    return tri_by_kind<VT_F32, false>(c, T, in, out);
}

// ======================================================== dense coarse LU
//
// LUflex::Solve (solver/lu.hpp:91-94): ltri forward then dutri backward on the
// coarsest operator's exact LU factors (30-45% dense at these sizes).  Both
// factors are stored column-major and dense; one CTA solves 32-row panels with
// one warp (shuffle broadcast of each solved value) and updates the remaining
// rows with all threads, one thread per row in column order (so FP sums keep
// the reference's order: ascending columns forward, descending backward).

constexpr int kLuThreads = 1024;

template <int VT, bool EXACT>
__global__ void __launch_bounds__(kLuThreads)
k_dense_lu(int n, const void *__restrict__ Lc_, const void *__restrict__ Uc_, const void *__restrict__ dinv_,
           int bitL, int bitU, int dbitU, const void *__restrict__ in_, void *__restrict__ out_, unsigned *flags) {
    using T = typename std::conditional<VT == VT_F64, double, typename std::conditional<VT == VT_F32, float,
                                                                                         long long>::type>::type;
    using V = typename std::conditional<VT == VT_I32, int, T>::type;  // value type
    extern __shared__ unsigned char smem_raw[];
    T *t = (T *)smem_raw;                                  // n accumulators
    V *x = (V *)(smem_raw + sizeof(T) * (size_t)n);        // n solved values
    const V *Lc = (const V *)Lc_;
    const V *Uc = (const V *)Uc_;
    const V *dinv = (const V *)dinv_;
    const V *in = (const V *)in_;
    V *out = (V *)out_;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    bool ovf = false;

    auto fsub = [](T a, T b, T c) -> T {  // a - b*c
        if constexpr (VT == VT_I32) return wsub(a, wmul(b, c));
        else if constexpr (EXACT && VT == VT_F64) return __dsub_rn(a, __dmul_rn(b, c));
        else if constexpr (EXACT) return __fsub_rn(a, __fmul_rn(b, c));
        else return a - b * c;
    };

    // ---- forward: unit lower
    for (int i = tid; i < n; i += kLuThreads) {
        if constexpr (VT == VT_I32) t[i] = wshl((long long)in[i], bitL);
        else t[i] = in[i];
    }
    __syncthreads();
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int kb = min(32, n - k0);
        if (warp == 0) {
            T tr = lane < kb ? t[k0 + lane] : T(0);
            for (int c = 0; c < kb; c++) {
                V xc;
                if constexpr (VT == VT_I32) {
                    const long long s = tr >> bitL;
                    if (lane == c) ovf |= !fits32(s);
                    xc = __shfl_sync(0xffffffffu, lo32(s), c);
                } else {
                    xc = __shfl_sync(0xffffffffu, tr, c);
                }
                if (lane > c && lane < kb) tr = fsub(tr, (T)Lc[(size_t)(k0 + c) * n + k0 + lane], (T)xc);
                if (lane == c) x[k0 + c] = xc;
            }
        }
        __syncthreads();
        for (int i = k0 + kb + tid; i < n; i += kLuThreads) {
            T acc = t[i];
            for (int c = 0; c < kb; c++) acc = fsub(acc, (T)Lc[(size_t)(k0 + c) * n + i], (T)x[k0 + c]);
            t[i] = acc;
        }
        __syncthreads();
    }
    // ---- backward: D^-1 U, last panel first, descending columns
    for (int i = tid; i < n; i += kLuThreads) {
        if constexpr (VT == VT_I32) t[i] = wshl((long long)x[i], bitU);
        else t[i] = x[i];
    }
    __syncthreads();
    for (int k1 = n; k1 > 0; k1 -= 32) {
        const int kb = min(32, k1);
        const int k0 = k1 - kb;
        if (warp == 0) {
            T tr = lane < kb ? t[k0 + lane] : T(0);
            for (int c = kb - 1; c >= 0; c--) {
                V xc;
                if (lane == c) {
                    if constexpr (VT == VT_I32) {
                        const long long s = wmul(tr >> bitU, (long long)dinv[k0 + c]) >> dbitU;
                        ovf |= !fits32(s);
                        xc = lo32(s);
                    } else if constexpr (EXACT && VT == VT_F64) {
                        xc = __dmul_rn(tr, dinv[k0 + c]);
                    } else if constexpr (EXACT) {
                        xc = __fmul_rn(tr, dinv[k0 + c]);
                    } else {
                        xc = tr * dinv[k0 + c];
                    }
                }
                xc = __shfl_sync(0xffffffffu, xc, c);
                if (lane < c) tr = fsub(tr, (T)Uc[(size_t)(k0 + c) * n + k0 + lane], (T)xc);
                if (lane == c) x[k0 + c] = xc;
            }
        }
        __syncthreads();
        for (int i = tid; i < k0; i += kLuThreads) {
            T acc = t[i];
            for (int c = kb - 1; c >= 0; c--) acc = fsub(acc, (T)Uc[(size_t)(k0 + c) * n + i], (T)x[k0 + c]);
            t[i] = acc;
        }
        __syncthreads();
    }
    for (int i = tid; i < n; i += kLuThreads) out[i] = x[i];
    if (ovf) atomicOr(flags, ST_OVERFLOW);
}

void DevDenseLU::release() {
    dfree(L);
    dfree(U);
    dfree(dinv);
    dfree(tmp);
    L = U = dinv = tmp = nullptr;
}

template <typename V>
static void densify(int n, const int *Lrptr, const int *Lcind, const V *Lval, const int *Urptr, const int *Ucind,
                    const V *Uval, std::vector<V> &Lc, std::vector<V> &Uc, std::vector<V> &dinv) {
    Lc.assign((size_t)n * n, V(0));
    Uc.assign((size_t)n * n, V(0));
    dinv.assign(n, V(0));
    for (int i = 0; i < n; i++) {
        for (int j = Lrptr[i]; j < Lrptr[i + 1]; j++) Lc[(size_t)Lcind[j] * n + i] = Lval[j];
        // dutri rows: D^-1 first, then the strict upper entries
        if (Urptr[i + 1] > Urptr[i]) dinv[i] = Uval[Urptr[i]];
        for (int j = Urptr[i] + 1; j < Urptr[i + 1]; j++) Uc[(size_t)Ucind[j] * n + i] = Uval[j];
    }
}

DevDenseLU upload_dense_lu(const int *Lrptr, const int *Lcind, const void *Lval, const int *Urptr,
                           const int *Ucind, const void *Uval, int n, int vt, int bitL, int bitU, int dbitU) {
    DevDenseLU d;
    d.n = n;
    d.vt = vt;
    d.bitL = bitL;
    d.bitU = bitU;
    d.dbitU = dbitU;
    if (vt == VT_I32) {
        std::vector<int32_t> Lc, Uc, dv;
        densify(n, Lrptr, Lcind, (const int32_t *)Lval, Urptr, Ucind, (const int32_t *)Uval, Lc, Uc, dv);
        d.L = dupload(Lc); d.U = dupload(Uc); d.dinv = dupload(dv);
    } else if (vt == VT_F64) {
        std::vector<double> Lc, Uc, dv;
        densify(n, Lrptr, Lcind, (const double *)Lval, Urptr, Ucind, (const double *)Uval, Lc, Uc, dv);
        d.L = dupload(Lc); d.U = dupload(Uc); d.dinv = dupload(dv);
    } else {
        std::vector<float> Lc, Uc, dv;
        densify(n, Lrptr, Lcind, (const float *)Lval, Urptr, Ucind, (const float *)Uval, Lc, Uc, dv);
        d.L = dupload(Lc); d.U = dupload(Uc); d.dinv = dupload(dv);
    }
    return d;
}

template <int VT, bool EXACT>
static void launch_lu(Ctx &c, const DevDenseLU &LU, const void *in, void *out) {
    const size_t acc = VT == VT_F32 ? 4 : 8;
    const size_t val = VT == VT_F64 ? 8 : 4;
    const size_t smem = (acc + val) * (size_t)LU.n;
    k_dense_lu<VT, EXACT><<<1, kLuThreads, smem, c.stream>>>(LU.n, LU.L, LU.U, LU.dinv, LU.bitL, LU.bitU,
                                                                LU.dbitU, in, out, c.d_flags);
    c.launches++;
}

void init_kernel_attributes() {
    const int mx = 227 * 1024;
    SAGB_CUDA(cudaFuncSetAttribute(k_dense_lu<VT_I32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_dense_lu<VT_F64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_dense_lu<VT_F64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_dense_lu<VT_F32, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_dense_lu<VT_F32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
}

void lu_solve(Ctx &c, const DevDenseLU &LU, const void *in, void *out) {
    if (LU.n == 0) return;
    if ((size_t)LU.n * 16 > 227 * 1024) throw CudaError{"coarsest level too large for the dense LU kernel"};
    if (LU.vt == VT_I32) return launch_lu<VT_I32, false>(c, LU, in, out);
    if (LU.vt == VT_F64) return c.fp_exact ? launch_lu<VT_F64, true>(c, LU, in, out)
                                           : launch_lu<VT_F64, false>(c, LU, in, out);
    return c.fp_exact ? launch_lu<VT_F32, true>(c, LU, in, out) : launch_lu<VT_F32, false>(c, LU, in, out);
}

}  // namespace sagb
