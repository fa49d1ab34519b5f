// Gauss-Seidel / SOR sweeps and the coarse LU solve in the reference's
// dependency order.
//
// Integer sweeps follow ldtri::CSRflex::SpTRSV (matrix/trimat/ldtri.hpp:172-183)
// and its block-Jacobi form BJCSRflex (ldtri.hpp:511-525):
//   t = in_i << bit;  t -= sum_j a_ij * out_j;  out_i = (int)((t >> bit) * dinv_i >> dbit)
// FP sweeps follow ldtri::CSR<T> / BJCSR<T> (ldtri.hpp:49-58, 398-412).
// Rows are stored in level order (host/schedule.hpp); a row only waits for the
// rows it reads, so the integer results are those of the sequential loop.
//
// Two kernels:
//  * k_tri_cta: the whole sweep in one CTA, the result vector in shared memory.
//    Levels are separated by block barriers; while one level is computed, the
//    row data of the next level is already being loaded (it does not depend on
//    the solve).  Used when the vector fits in shared memory (coarse levels).
//  * k_tri: many CTAs claim chunks of level-ordered rows by ticket and wait
//    only for the rows they read.  Integer and FP32 results are published as
//    one 64-bit word {epoch, value}; FP64 results use an epoch flag with
//    release/acquire.  All reads of one row's dependencies are issued together.
//    Every wait is bounded in time (ST_TIMEOUT); once a wait has timed out, all
//    CTAs stop waiting.  Ticket and epoch are advanced by the last CTA, so the
//    kernel replays from a CUDA graph.
#include <algorithm>
#include <type_traits>

#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {

constexpr int kTriThreads = 256;   // multi-CTA kernel
constexpr int kCtaThreads = 1024;  // single-CTA kernel
constexpr int kBatch = 4;          // dependencies read together per lane (multi-CTA)
constexpr int kCtaBatch = 8;       // entries held in registers per lane (single CTA)
constexpr size_t kCtaSmem = 200 * 1024;

template <int VT>
using vt_t = typename std::conditional<VT == VT_I32, int, typename std::conditional<VT == VT_F64, double, float>::type>::type;

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

__device__ __forceinline__ unsigned long long wait_packed(unsigned long long *pk, int c, unsigned ep,
                                                          unsigned *flags) {
    const unsigned long long t0 = globaltimer_ns();
    unsigned it = 0;
    for (;;) {
        const unsigned long long w = ld_relaxed_u64(pk + c);
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

// t - v*o in the accumulator type of each precision
template <int VT, bool EXACT>
__device__ __forceinline__ auto acc_sub(typename std::conditional<VT == VT_I32, long long, vt_t<VT>>::type t,
                                        vt_t<VT> v, vt_t<VT> o) {
    if constexpr (VT == VT_I32) return wsub(t, (long long)v * (long long)o);
    else if constexpr (EXACT && VT == VT_F64) return __dsub_rn(t, __dmul_rn(v, o));
    else if constexpr (EXACT) return __fsub_rn(t, __fmul_rn(v, o));
    else return t - v * o;
}

// ============================================================== multi-CTA

template <int VT, int G, bool EXACT>
__device__ __forceinline__ void tri_row(const TriArgs &a, int p, bool valid, int g, unsigned ep, const void *in_,
                                        void *out_, unsigned *flags, bool &ovf) {
    using V = vt_t<VT>;
    using A = typename std::conditional<VT == VT_I32, long long, V>::type;
    const V *in = (const V *)in_;
    V *out = (V *)out_;
    const V *pv = (const V *)a.pval;
    A t = 0;
    int row = 0;
    if (valid) {
        row = __ldg(a.perm + p);
        if (g == 0) {
            if constexpr (VT == VT_I32) t = wshl((long long)__ldg(in + row), a.bit);
            else t = __ldg(in + row);
        }
        const int jb = __ldg(a.prp + p), je = __ldg(a.prp + p + 1);
        for (int j0 = jb + g; j0 < je; j0 += G * kBatch) {
            int c[kBatch];
            V v[kBatch];
#pragma unroll
            for (int k = 0; k < kBatch; k++) {
                const int j = j0 + k * G;
                c[k] = j < je ? __ldg(a.pci + j) : -1;
                v[k] = j < je ? __ldg(pv + j) : V(0);
            }
            if constexpr (VT == VT_F64) {
                // relaxed reads of all ready flags, then one acquire fence
                unsigned f[kBatch];
#pragma unroll
                for (int k = 0; k < kBatch; k++) f[k] = c[k] >= 0 ? ld_relaxed_u32(a.flag + c[k]) : ep;
#pragma unroll
                for (int k = 0; k < kBatch; k++)
                    if (f[k] != ep) wait_flag(a.flag, c[k], ep, flags);
                fence_acq_rel_gpu();
#pragma unroll
                for (int k = 0; k < kBatch; k++)
                    if (c[k] >= 0) t = acc_sub<VT, EXACT>(t, v[k], ld_relaxed_f64((const double *)out + c[k]));
            } else {
                unsigned long long w[kBatch];
#pragma unroll
                for (int k = 0; k < kBatch; k++) w[k] = c[k] >= 0 ? ld_relaxed_u64(a.pk + c[k]) : 0ull;
#pragma unroll
                for (int k = 0; k < kBatch; k++) {
                    if (c[k] < 0) continue;
                    if ((unsigned)(w[k] >> 32) != ep) w[k] = wait_packed(a.pk, c[k], ep, flags);
                    V o;
                    if constexpr (VT == VT_I32) o = (int)(unsigned)w[k];
                    else o = __uint_as_float((unsigned)w[k]);
                    t = acc_sub<VT, EXACT>(t, v[k], o);
                }
            }
        }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        if constexpr (VT == VT_I32) t = wadd(t, shfl_xor(t, o));
        else t += shfl_xor(t, o);
    }
    if (valid && g == 0) {
        if constexpr (VT == VT_I32) {
            const long long s = wmul(t >> a.bit, (long long)__ldg((const int *)a.dinv + p)) >> a.dbit;
            const int o = lo32(s);
            ovf |= !fits32(s);
            out[row] = o;
            st_relaxed_u64(a.pk + row, ((unsigned long long)ep << 32) | (unsigned)o);
        } else {
            const V d = __ldg((const V *)a.dinv + p);
            V r;
            if constexpr (VT == VT_F64) r = __dmul_rn(t, d);
            else r = __fmul_rn(t, d);
            out[row] = r;
            if constexpr (VT == VT_F64) st_release_u32(a.flag + row, ep);
            else st_relaxed_u64(a.pk + row, ((unsigned long long)ep << 32) | __float_as_uint(r));
        }
    }
}

template <int VT, int G, bool EXACT>
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
                tri_row<VT, G, EXACT>(a, p, p < p1, g, ep, in, out, flags, ovf);
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

// ============================================================= single CTA

template <int VT>
struct RowPre {
    int row, jb, je;
    vt_t<VT> in, dinv;
    int c[kCtaBatch];
    vt_t<VT> v[kCtaBatch];
};

template <int VT, int G>
__device__ __forceinline__ void cta_load(RowPre<VT> &r, const TriArgs &a, int p, bool valid, int g,
                                         const vt_t<VT> *in) {
    using V = vt_t<VT>;
    r.row = 0;
    r.jb = r.je = 0;
    if (!valid) return;
    r.row = __ldg(a.perm + p);
    r.jb = __ldg(a.prp + p);
    r.je = __ldg(a.prp + p + 1);
    r.in = __ldg(in + r.row);
    r.dinv = __ldg((const V *)a.dinv + p);
#pragma unroll
    for (int k = 0; k < kCtaBatch; k++) {
        const int j = r.jb + g + k * G;
        r.c[k] = j < r.je ? __ldg(a.pci + j) : 0;
        r.v[k] = j < r.je ? __ldg((const V *)a.pval + j) : V(0);
    }
}

template <int VT, int G, bool EXACT>
__device__ __forceinline__ void cta_row(const RowPre<VT> &r, const TriArgs &a, bool valid, int g,
                                        vt_t<VT> *s_out, bool &ovf) {
    using V = vt_t<VT>;
    using A = typename std::conditional<VT == VT_I32, long long, V>::type;
    A t = 0;
    if (valid) {
        if (g == 0) {
            if constexpr (VT == VT_I32) t = wshl((long long)r.in, a.bit);
            else t = r.in;
        }
#pragma unroll
        for (int k = 0; k < kCtaBatch; k++)
            if (r.jb + g + k * G < r.je) t = acc_sub<VT, EXACT>(t, r.v[k], s_out[r.c[k]]);
        for (int j = r.jb + g + kCtaBatch * G; j < r.je; j += G)
            t = acc_sub<VT, EXACT>(t, __ldg((const V *)a.pval + j), s_out[__ldg(a.pci + j)]);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        if constexpr (VT == VT_I32) t = wadd(t, shfl_xor(t, o));
        else t += shfl_xor(t, o);
    }
    if (valid && g == 0) {
        if constexpr (VT == VT_I32) {
            const long long s = wmul(t >> a.bit, (long long)r.dinv) >> a.dbit;
            ovf |= !fits32(s);
            s_out[r.row] = lo32(s);
        } else if constexpr (VT == VT_F64) {
            s_out[r.row] = __dmul_rn(t, r.dinv);
        } else {
            s_out[r.row] = __fmul_rn(t, r.dinv);
        }
    }
}

template <int VT, int G, bool EXACT>
__global__ void __launch_bounds__(kCtaThreads, 1)
k_tri_cta(TriArgs a, const int *__restrict__ lvl_ptr, int nlev, const void *in_, void *out_, unsigned *flags) {
    using V = vt_t<VT>;
    extern __shared__ unsigned char smem_raw[];
    V *s_out = (V *)smem_raw;
    const V *in = (const V *)in_;
    V *out = (V *)out_;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int RPW = 32 / G;
    constexpr int NW = kCtaThreads / 32;
    const int g = lane % G, sub = lane / G;
    const int gid = warp * RPW + sub;
    bool ovf = false;
    RowPre<VT> pre, cur;
    int p0 = nlev > 0 ? __ldg(lvl_ptr) : 0;
    int p1 = nlev > 0 ? __ldg(lvl_ptr + 1) : 0;
    cta_load<VT, G>(pre, a, p0 + gid, p0 + gid < p1, g, in);
    for (int d = 0; d < nlev; d++) {
        cur = pre;
        const int q0 = p1, q1 = d + 2 <= nlev ? __ldg(lvl_ptr + d + 2) : p1;
        // the next level's first row of this group, loaded while this level runs
        cta_load<VT, G>(pre, a, q0 + gid, q0 + gid < q1, g, in);
        bool first = true;
        for (int base = p0 + warp * RPW; base < p1; base += NW * RPW) {
            const int p = base + sub;
            if (!first) cta_load<VT, G>(cur, a, p, p < p1, g, in);
            first = false;
            cta_row<VT, G, EXACT>(cur, a, p < p1, g, s_out, ovf);
        }
        __syncthreads();
        p0 = q0;
        p1 = q1;
    }
    for (int i = threadIdx.x; i < a.n; i += kCtaThreads) out[i] = s_out[i];
    if (ovf) atomicOr(flags, ST_OVERFLOW);
}

// ================================================================ upload

void DevTri::release() {
    dfree(perm);
    dfree(prp);
    dfree(pci);
    dfree(pval);
    dfree(dinv);
    dfree(chunk_lv);
    dfree(sub_bound);
    dfree(lvl_ptr);
    dfree(pk);
    dfree(flag);
    dfree(sync);
    perm = prp = pci = chunk_lv = sub_bound = lvl_ptr = nullptr;
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

static int pow2_at_least(double x) {
    int g = 1;
    while (g < 32 && g < x) g <<= 1;
    return g;
}

DevTri upload_tri(const Ctx &c, int n, const int *rptr, const int *cind, const void *vals, int vt, int kind,
                  int bit, int dbit) {
    if (kind != TRI_LD) throw CudaError{"only LD sweeps are uploaded as sparse triangles"};
    DevTri d;
    d.n = n;
    d.kind = kind;
    d.vt = vt;
    d.bit = bit;
    d.dbit = dbit;
    const int64_t nnz = n ? rptr[n] : 0;
    const double avg = n ? (double)(nnz - n) / n : 0.0;
    d.one_cta = (size_t)n * vt_size(vt) <= kCtaSmem;
    int G;
    if (d.one_cta) G = pow2_at_least(avg / kCtaBatch);        // registers hold G * kCtaBatch entries
    else G = pow2_at_least(avg / kBatch);                    // one batch covers a typical row
    if (vt != VT_I32 && c.fp_exact) G = 1;                   // sequential order inside a row
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
    d.lvl_ptr = dupload(s.lvl_ptr);
    if (!d.one_cta) {
        if (vt == VT_F64) {
            d.flag = (unsigned *)dmalloc(sizeof(unsigned) * std::max(n, 1));
            SAGB_CUDA(cudaMemset(d.flag, 0, sizeof(unsigned) * std::max(n, 1)));
        } else {
            d.pk = (unsigned long long *)dmalloc(sizeof(unsigned long long) * std::max(n, 1));
            SAGB_CUDA(cudaMemset(d.pk, 0, sizeof(unsigned long long) * std::max(n, 1)));
        }
        d.sync = (TriSync *)dmalloc(sizeof(TriSync));
        SAGB_CUDA(cudaMemset(d.sync, 0, sizeof(TriSync)));
    }
    d.grid = std::max(1, std::min(d.nchunks, c.num_sms * 4));
    return d;
}

template <int VT, int G, bool EXACT>
static void launch_tri(Ctx &c, const DevTri &T, const void *in, void *out) {
    TriArgs a{T.n, T.nchunks, T.bit, T.dbit, T.perm, T.prp, T.pci, T.pval, T.dinv,
              T.chunk_lv, T.sub_bound, T.pk, T.flag, T.sync};
    if (T.one_cta) {
        const size_t smem = (size_t)T.n * sizeof(vt_t<VT>);
        k_tri_cta<VT, G, EXACT><<<1, kCtaThreads, smem, c.stream>>>(a, T.lvl_ptr, T.nlev, in, out, c.d_flags);
    } else {
        k_tri<VT, G, EXACT><<<T.grid, kTriThreads, 0, c.stream>>>(a, in, out, c.d_flags);
    }
    c.launches++;
}

template <int VT, bool EXACT>
static void tri_by_group(Ctx &c, const DevTri &T, const void *in, void *out) {
    switch (T.group) {
        case 1: return launch_tri<VT, 1, EXACT>(c, T, in, out);
        case 2: return launch_tri<VT, 2, EXACT>(c, T, in, out);
        case 4: return launch_tri<VT, 4, EXACT>(c, T, in, out);
        case 8: return launch_tri<VT, 8, EXACT>(c, T, in, out);
        case 16: return launch_tri<VT, 16, EXACT>(c, T, in, out);
        default: return launch_tri<VT, 32, EXACT>(c, T, in, out);
    }
}

void trsv(Ctx &c, const DevTri &T, const void *in, void *out) {
    if (T.n == 0) return;
    if (T.vt == VT_I32) return tri_by_group<VT_I32, false>(c, T, in, out);
    if (T.vt == VT_F64) {
        if (c.fp_exact) return tri_by_group<VT_F64, true>(c, T, in, out);
        return tri_by_group<VT_F64, false>(c, T, in, out);
    }
    if (c.fp_exact) return tri_by_group<VT_F32, true>(c, T, in, out);
    return tri_by_group<VT_F32, false>(c, T, in, out);
}

// ======================================================== dense coarse LU
//
// LUflex::Solve / LU<T>::Solve (solver/lu.hpp:91-94, 30-33): ltri forward then
// dutri backward on the coarsest operator's exact LU factors (30-45% dense at
// these sizes), stored dense and row-major.  One CTA, 32-row panels, left
// looking: the 32 warps first reduce each panel row against the solved part
// (one warp per row, lanes over columns), then warp 0 solves the 32x32 diagonal
// block with the block held in registers (shuffle broadcast of each value).
// Integer sums are exact in any order.  In the FP sequential-order mode the
// panel reduction runs one thread per row in column order (ascending forward,
// descending backward), which is the reference's order.

constexpr int kLuThreads = 1024;

template <int VT, bool EXACT>
__global__ void __launch_bounds__(kLuThreads, 1)
k_dense_lu(int n, const void *__restrict__ L_, const void *__restrict__ U_, const void *__restrict__ dinv_,
           int bitL, int bitU, int dbitU, const void *__restrict__ in_, void *__restrict__ out_, unsigned *flags) {
    using V = vt_t<VT>;
    using T = typename std::conditional<VT == VT_I32, long long, V>::type;
    extern __shared__ unsigned char smem_raw[];
    T *t = (T *)smem_raw;                           // n accumulators
    V *x = (V *)(smem_raw + sizeof(T) * (size_t)n); // n solved values
    const V *L = (const V *)L_;
    const V *U = (const V *)U_;
    const V *dinv = (const V *)dinv_;
    const V *in = (const V *)in_;
    V *out = (V *)out_;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    bool ovf = false;

    // ---------------- forward: unit lower, t = in << bit
    for (int i = tid; i < n; i += kLuThreads) {
        if constexpr (VT == VT_I32) t[i] = wshl((long long)in[i], bitL);
        else t[i] = in[i];
    }
    __syncthreads();
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int kb = min(32, n - k0);
        // panel rows against columns [0, k0)
        if (k0 > 0) {
            if constexpr (EXACT && VT != VT_I32) {
                if (tid < kb) {
                    const V *row = L + (size_t)(k0 + tid) * n;
                    T acc = t[k0 + tid];
                    for (int c = 0; c < k0; c++) acc = acc_sub<VT, true>(acc, row[c], x[c]);
                    t[k0 + tid] = acc;
                }
            } else if (warp < kb) {
                const V *row = L + (size_t)(k0 + warp) * n;
                T acc = 0;
                for (int c = lane; c < k0; c += 32) acc = acc_sub<VT, false>(acc, __ldg(row + c), x[c]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    if constexpr (VT == VT_I32) acc = wadd(acc, shfl_xor(acc, o));
                    else acc += shfl_xor(acc, o);
                }
                if (lane == 0) {
                    if constexpr (VT == VT_I32) t[k0 + warp] = wadd(t[k0 + warp], acc);
                    else t[k0 + warp] += acc;
                }
            }
        }
        __syncthreads();
        if (warp == 0) {
            V dblk[32];
            const V *row = L + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) dblk[c] = (lane < kb && c < lane) ? __ldg(row + c) : V(0);
            T tr = lane < kb ? t[k0 + lane] : T(0);
#pragma unroll
            for (int c = 0; c < 32; c++) {
                if (c < kb) {
                    V xc;
                    if constexpr (VT == VT_I32) {
                        const long long s = tr >> bitL;
                        if (lane == c) ovf |= !fits32(s);
                        xc = __shfl_sync(0xffffffffu, lo32(s), c);
                    } else {
                        xc = __shfl_sync(0xffffffffu, tr, c);
                    }
                    if (lane > c) tr = acc_sub<VT, EXACT>(tr, dblk[c], xc);
                    if (lane == c) x[k0 + c] = xc;
                }
            }
        }
        __syncthreads();
    }
    // ---------------- backward: D^-1 U, last panel first
    for (int i = tid; i < n; i += kLuThreads) {
        if constexpr (VT == VT_I32) t[i] = wshl((long long)x[i], bitU);
        else t[i] = x[i];
    }
    __syncthreads();
    for (int k1 = n; k1 > 0; k1 -= 32) {
        const int kb = min(32, k1);
        const int k0 = k1 - kb;
        if (k1 < n) {
            if constexpr (EXACT && VT != VT_I32) {
                if (tid < kb) {
                    const V *row = U + (size_t)(k0 + tid) * n;
                    T acc = t[k0 + tid];
                    for (int c = n - 1; c >= k1; c--) acc = acc_sub<VT, true>(acc, row[c], x[c]);
                    t[k0 + tid] = acc;
                }
            } else if (warp < kb) {
                const V *row = U + (size_t)(k0 + warp) * n;
                T acc = 0;
                for (int c = k1 + lane; c < n; c += 32) acc = acc_sub<VT, false>(acc, __ldg(row + c), x[c]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    if constexpr (VT == VT_I32) acc = wadd(acc, shfl_xor(acc, o));
                    else acc += shfl_xor(acc, o);
                }
                if (lane == 0) {
                    if constexpr (VT == VT_I32) t[k0 + warp] = wadd(t[k0 + warp], acc);
                    else t[k0 + warp] += acc;
                }
            }
        }
        __syncthreads();
        if (warp == 0) {
            V dblk[32];
            const V *row = U + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) dblk[c] = (lane < kb && c > lane && c < kb) ? __ldg(row + c) : V(0);
            T tr = lane < kb ? t[k0 + lane] : T(0);
            const V dv = lane < kb ? dinv[k0 + lane] : V(0);
#pragma unroll
            for (int c = 31; c >= 0; c--) {
                if (c < kb) {
                    V xc = V(0);
                    if (lane == c) {
                        if constexpr (VT == VT_I32) {
                            const long long s = wmul(tr >> bitU, (long long)dv) >> dbitU;
                            ovf |= !fits32(s);
                            xc = lo32(s);
                        } else if constexpr (VT == VT_F64) {
                            xc = __dmul_rn(tr, dv);
                        } else {
                            xc = __fmul_rn(tr, dv);
                        }
                    }
                    xc = __shfl_sync(0xffffffffu, xc, c);
                    if (lane < c) tr = acc_sub<VT, EXACT>(tr, dblk[c], xc);
                    if (lane == c) x[k0 + c] = xc;
                }
            }
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
                    const V *Uval, std::vector<V> &Ld, std::vector<V> &Ud, std::vector<V> &dinv) {
    Ld.assign((size_t)n * n, V(0));
    Ud.assign((size_t)n * n, V(0));
    dinv.assign(n, V(0));
    for (int i = 0; i < n; i++) {
        for (int j = Lrptr[i]; j < Lrptr[i + 1]; j++) Ld[(size_t)i * n + Lcind[j]] = Lval[j];
        // dutri rows: D^-1 first, then the strict upper entries
        if (Urptr[i + 1] > Urptr[i]) dinv[i] = Uval[Urptr[i]];
        for (int j = Urptr[i] + 1; j < Urptr[i + 1]; j++) Ud[(size_t)i * n + Ucind[j]] = Uval[j];
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
        std::vector<int32_t> Ld, Ud, dv;
        densify(n, Lrptr, Lcind, (const int32_t *)Lval, Urptr, Ucind, (const int32_t *)Uval, Ld, Ud, dv);
        d.L = dupload(Ld); d.U = dupload(Ud); d.dinv = dupload(dv);
    } else if (vt == VT_F64) {
        std::vector<double> Ld, Ud, dv;
        densify(n, Lrptr, Lcind, (const double *)Lval, Urptr, Ucind, (const double *)Uval, Ld, Ud, dv);
        d.L = dupload(Ld); d.U = dupload(Ud); d.dinv = dupload(dv);
    } else {
        std::vector<float> Ld, Ud, dv;
        densify(n, Lrptr, Lcind, (const float *)Lval, Urptr, Ucind, (const float *)Uval, Ld, Ud, dv);
        d.L = dupload(Ld); d.U = dupload(Ud); d.dinv = dupload(dv);
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

template <int VT, bool EXACT>
static void cta_attrs() {
    const int mx = 227 * 1024;
    SAGB_CUDA(cudaFuncSetAttribute(k_tri_cta<VT, 1, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_tri_cta<VT, 2, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_tri_cta<VT, 4, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_tri_cta<VT, 8, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_tri_cta<VT, 16, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_tri_cta<VT, 32, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    SAGB_CUDA(cudaFuncSetAttribute(k_dense_lu<VT, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
}

void init_kernel_attributes() {
    cta_attrs<VT_I32, false>();
    cta_attrs<VT_F64, false>();
    cta_attrs<VT_F64, true>();
    cta_attrs<VT_F32, false>();
    cta_attrs<VT_F32, true>();
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
