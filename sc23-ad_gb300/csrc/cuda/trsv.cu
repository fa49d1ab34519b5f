// Gauss-Seidel / SOR sweeps and the coarse LU solve in the reference's
// dependency order.
//
// Integer sweeps follow ldtri::CSRflex::SpTRSV (matrix/trimat/ldtri.hpp:172-183)
// and its block-Jacobi form BJCSRflex (ldtri.hpp:511-525):
//   t = in_i << bit;  t -= sum_j a_ij * out_j;  out_i = (int)((t >> bit) * dinv_i >> dbit)
// FP sweeps follow ldtri::CSR<T> / BJCSR<T> (ldtri.hpp:49-58, 398-412).
// Rows are grouped into dependency levels (host/schedule.hpp); every row of a
// level only reads rows of earlier levels, so computing level after level gives
// the integer results of the sequential loop.
//
// Two kernels:
//  * k_tri_cta (coarse levels, the vector fits in shared memory): one CTA.  The
//    result vector lives in shared memory, seeded with `in` (a row reads its own
//    input once and then overwrites it).  Each level's row data is one 16-byte
//    aligned block that a bulk copy (cp.async.bulk + mbarrier) brings into a
//    byte ring in shared memory (all of it not taken by the vector) up to
//    kSlots levels ahead, so a level costs shared memory traffic and one block
//    barrier.
//  * k_tri (fine levels): one CTA per SM claims chunks of level-ordered rows
//    by ticket; a row waits only for the rows it reads.  Integer and FP32
//    results are published as one 64-bit word {epoch, value}, so a dependency
//    costs one L2 load; FP64 results use an epoch flag with release/acquire.
//    Each lane reads a batch of dependencies at once and spins only on those
//    not yet published.  Chunks are claimed in level order and depend only on
//    earlier chunks, so the waits cannot deadlock.
// All waits are bounded in time (ST_TIMEOUT); ticket and epoch are advanced by
// the last CTA, so both kernels replay from a CUDA graph.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {

constexpr int kTriThreads = 256;   // multi-CTA kernel
constexpr int kCtaThreads = 1024;  // single-CTA kernel
constexpr int kBatch = 4;          // dependencies read together per lane (multi-CTA)
constexpr int kSlots = 8;          // levels in flight in the single CTA's bulk-copy ring
constexpr size_t kSmemMax = 227 * 1024;
constexpr size_t kCtaVecMax = 150 * 1024;  // largest shared result vector

template <int VT>
using vt_t = typename std::conditional<VT == VT_I32, int, typename std::conditional<VT == VT_F64, double, float>::type>::type;
template <int VT>
using acc_t = typename std::conditional<VT == VT_I32, long long, vt_t<VT>>::type;

__device__ __forceinline__ bool aborted(const unsigned *flags) {
    return (*(volatile const unsigned *)flags & ST_TIMEOUT) != 0;
}

// t - v*o in the accumulator type of each precision
template <int VT, bool EXACT>
__device__ __forceinline__ acc_t<VT> acc_sub(acc_t<VT> t, vt_t<VT> v, vt_t<VT> o) {
    if constexpr (VT == VT_I32) return wsub(t, (long long)v * (long long)o);
    else if constexpr (EXACT && VT == VT_F64) return __dsub_rn(t, __dmul_rn(v, o));
    else if constexpr (EXACT) return __fsub_rn(t, __fmul_rn(v, o));
    else return t - v * o;
}
template <int VT>
__device__ __forceinline__ acc_t<VT> acc_init(vt_t<VT> in, int bit) {
    if constexpr (VT == VT_I32) return wshl((long long)in, bit);
    else return in;
}
template <int VT>
__device__ __forceinline__ acc_t<VT> acc_reduce(acc_t<VT> t, int G) {
    for (int o = G / 2; o > 0; o >>= 1) {
        if constexpr (VT == VT_I32) t = wadd(t, shfl_xor(t, o));
        else t += shfl_xor(t, o);
    }
    return t;
}
// out_i from the accumulated row: (t >> bit) * dinv >> dbit, or t * dinv
template <int VT>
__device__ __forceinline__ vt_t<VT> acc_finish(acc_t<VT> t, vt_t<VT> d, int bit, int dbit, bool &ovf) {
    if constexpr (VT == VT_I32) {
        const long long s = wmul(t >> bit, (long long)d) >> dbit;
        ovf |= !fits32(s);
        return lo32(s);
    } else if constexpr (VT == VT_F64) {
        return __dmul_rn(t, d);
    } else {
        return __fmul_rn(t, d);
    }
}

// ============================================================== multi-CTA

struct TriArgs {
    int n, nchunks, bit, dbit;
    const int *perm, *prp, *pci;
    const void *pval, *dinv;
    const int *chunk_lv, *sub_bound;
    unsigned long long *pk;
    unsigned *flag;
    TriSync *sync;
};

// spin on one packed {epoch, value} word until it carries epoch ep (bounded;
// the shared status word is read only on the slow path)
__device__ __forceinline__ unsigned long long wait_packed(unsigned long long *pk, int c, unsigned ep,
                                                          unsigned *flags) {
    const unsigned long long t0 = globaltimer_ns();
    for (unsigned it = 1;; it++) {
        const unsigned long long w = ld_relaxed_u64(pk + c);
        if ((unsigned)(w >> 32) == ep) return w;
        if ((it & 255u) == 0) {
            if (globaltimer_ns() - t0 > kSpinLimitNs) {
                atomicOr(flags, ST_TIMEOUT);
                return w;
            }
            if (aborted(flags)) return w;
        }
    }
}

__device__ __forceinline__ void wait_flag(const unsigned *flag, int c, unsigned ep, unsigned *flags) {
    const unsigned long long t0 = globaltimer_ns();
    for (unsigned it = 1;; it++) {
        if (ld_relaxed_u32(flag + c) == ep) return;
        if ((it & 255u) == 0) {
            if (globaltimer_ns() - t0 > kSpinLimitNs) {
                atomicOr(flags, ST_TIMEOUT);
                return;
            }
            if (aborted(flags)) return;
        }
    }
}

__device__ __forceinline__ double ld_relaxed_f64(const double *p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}

// one row, G lanes; each lane reads kBatch dependencies at a time, all
// together, and spins only on those not yet published
template <int VT, int G, bool EXACT>
__device__ __forceinline__ void tri_row(const TriArgs &a, int p, bool valid, int g, unsigned ep, const void *in_,
                                        void *out_, unsigned *flags, bool &ovf) {
    using V = vt_t<VT>;
    const V *in = (const V *)in_;
    V *out = (V *)out_;
    const V *pv = (const V *)a.pval;
    acc_t<VT> t = 0;
    int row = 0;
    if (valid) {
        row = __ldg(a.perm + p);
        if (g == 0) t = acc_init<VT>(__ldg(in + row), a.bit);
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
                unsigned f[kBatch];
#pragma unroll
                for (int k = 0; k < kBatch; k++) f[k] = c[k] >= 0 ? ld_relaxed_u32(a.flag + c[k]) : ep;
#pragma unroll
                for (int k = 0; k < kBatch; k++)
                    if (f[k] != ep) wait_flag(a.flag, c[k], ep, flags);
                fence_acq_rel_gpu();  // the flags were released after the values
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
    t = acc_reduce<VT>(t, G);
    if (valid && g == 0) {
        const V r = acc_finish<VT>(t, __ldg((const V *)a.dinv + p), a.bit, a.dbit, ovf);
        out[row] = r;
        if constexpr (VT == VT_F64) {
            st_release_u32(a.flag + row, ep);
        } else if constexpr (VT == VT_I32) {
            st_relaxed_u64(a.pk + row, ((unsigned long long)ep << 32) | (unsigned)r);
        } else {
            st_relaxed_u64(a.pk + row, ((unsigned long long)ep << 32) | __float_as_uint(r));
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
//
// Level block (host layout, 16-byte aligned, size a multiple of 16):
//   int32 header[8] = {R, E, off_val, off_dinv, off_perm, off_rp, 0, 0}
//   val[E] (V), dinv[R] (V), perm[R], rp[R+1] (0-based inside the block), pci[E]

template <int VT, int G, bool EXACT>
__device__ __forceinline__ void cta_level(const unsigned char *blk, vt_t<VT> *s_out, int bit, int dbit, int warp,
                                          int sub, int g, bool &ovf) {
    using V = vt_t<VT>;
    constexpr int RPW = 32 / G;
    constexpr int NW = kCtaThreads / 32 - 1;  // the last warp issues the bulk copies
    const int *hdr = (const int *)blk;
    const int R = hdr[0];
    const V *val = (const V *)(blk + hdr[2]);
    const V *dv = (const V *)(blk + hdr[3]);
    const int *perm = (const int *)(blk + hdr[4]);
    const int *rp = (const int *)(blk + hdr[5]);
    const int *pci = rp + R + 1;
    for (int base = warp * RPW; base < R; base += NW * RPW) {
        const int r = base + sub;
        const bool valid = r < R;
        acc_t<VT> t = 0;
        int row = 0;
        if (valid) {
            row = perm[r];
            const int jb = rp[r], je = rp[r + 1];
            if (g == 0) t = acc_init<VT>(s_out[row], bit);
            // four entries of the lane at a time: their loads are issued
            // together, the products are taken in the lane's order
            int j = jb + g;
            for (; j + 3 * G < je; j += 4 * G) {
                const int c0 = pci[j], c1 = pci[j + G], c2 = pci[j + 2 * G], c3 = pci[j + 3 * G];
                const V v0 = val[j], v1 = val[j + G], v2 = val[j + 2 * G], v3 = val[j + 3 * G];
                const V o0 = s_out[c0], o1 = s_out[c1], o2 = s_out[c2], o3 = s_out[c3];
                t = acc_sub<VT, EXACT>(t, v0, o0);
                t = acc_sub<VT, EXACT>(t, v1, o1);
                t = acc_sub<VT, EXACT>(t, v2, o2);
                t = acc_sub<VT, EXACT>(t, v3, o3);
            }
            for (; j < je; j += G) t = acc_sub<VT, EXACT>(t, val[j], s_out[pci[j]]);
        }
        t = acc_reduce<VT>(t, G);
        if (valid && g == 0) s_out[row] = acc_finish<VT>(t, dv[r], bit, dbit, ovf);
    }
}

// Shared memory of the single-CTA kernel: the result vector, a byte ring for
// the level blocks, kSlots mbarriers, the ring position of each level in
// flight, the block offsets and the rows of each level.  The first lane of
// the last warp (the producer; that warp computes no rows, so issuing copies
// never delays a level) places every block contiguously in the ring, in level
// order (at the write position, or at the ring's start when the end has no
// room), as soon as the ring has room and fewer than kSlots levels are in
// flight; a block larger than the whole ring is read from global memory
// instead.  Level d is always placed by the time the CTA reaches it: the
// producer places it right after the barrier of level d-1 at the latest, when
// every earlier level has been consumed and the ring is empty.
//
// (A variant without the barrier per level, each row waiting on done bits of
// the rows it reads, ran about twice as slow on the coarse levels of Poisson
// 128^3: the waiting rows' shared-memory polling slowed the rows being
// computed more than the barrier costs.)
template <int VT, int G, bool EXACT>
__global__ void __launch_bounds__(kCtaThreads, 1)
k_tri_cta(const unsigned char *__restrict__ blocks, const unsigned *__restrict__ blk_off, int nlev, int n,
          int bit, int dbit, int ring_bytes, const void *in_, void *out_, unsigned *flags) {
    using V = vt_t<VT>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V *s_out = (V *)smem_raw;
    const size_t vec_bytes = ((size_t)n * sizeof(V) + 15) & ~(size_t)15;
    unsigned char *ring = smem_raw + vec_bytes;
    unsigned long long *bar = (unsigned long long *)(ring + ring_bytes);
    unsigned *s_pos = (unsigned *)(bar + kSlots);  // ring offset of each level in flight
    unsigned *s_off = s_pos + kSlots;              // block offsets in 16-byte units
    const unsigned *s_rows = s_off + nlev + 1;     // rows of each level
    const V *in = (const V *)in_;
    V *out = (V *)out_;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane % G, sub = lane / G;
    constexpr int kProducerWarp = kCtaThreads / 32 - 1;
    const bool compute = warp != kProducerWarp;
    const bool producer = warp == kProducerWarp && lane == 0;
    bool ovf = false;

    if (producer) {
        for (int s = 0; s < kSlots; s++) mbar_init(bar + s, 1);
        fence_mbar_init();
    }
    for (int i = threadIdx.x; i < n; i += kCtaThreads) s_out[i] = in[i];
    for (int i = threadIdx.x; i <= 2 * nlev; i += kCtaThreads) s_off[i] = __ldg(blk_off + i);
    __syncthreads();
    auto bytes_of = [&](int d) { return (s_off[d + 1] - s_off[d]) * 16u; };
    auto staged = [&](int d) { return bytes_of(d) <= (unsigned)ring_bytes; };
    // the producer's ring state: levels [consumed, issued) are in flight; the
    // nst staged ones among them occupy [lo, head), wrapped once when head <= lo
    int issued = 0, nst = 0;
    unsigned lo = 0, head = 0;
    auto issue_more = [&](int consumed) {  // producer only
        while (issued < nlev && issued - consumed < kSlots) {
            const int d = issued;
            if (staged(d)) {
                const unsigned b = bytes_of(d);
                unsigned pos;
                if (nst == 0) {
                    pos = 0;
                    lo = 0;
                } else if (head > lo) {  // [lo, head): room at the end, else at the start
                    if (b <= (unsigned)ring_bytes - head) pos = head;
                    else if (b <= lo) pos = 0;
                    else break;
                } else {  // [lo, ring) and [0, head): room between head and lo
                    if (b <= lo - head) pos = head;
                    else break;
                }
                head = pos + b;
                nst++;
                const int s = d % kSlots;
                // the region's previous readers passed the level barrier
                // before this copy is issued (no proxy fence is needed for a
                // bulk copy into memory that generic loads only read)
                s_pos[s] = pos;  // published to the waiting threads by the arrive below
                mbar_expect_tx(bar + s, b);
                bulk_g2s(ring + pos, blocks + (size_t)s_off[d] * 16, b, bar + s);
            }
            issued++;
        }
    };
    if (producer) issue_more(0);
    unsigned phase = 0;  // bit s: parity of slot s's next completion
    int stuck = -1;      // level whose copy did not arrive in time
    for (int d = 0; d < nlev; d++) {
        const bool st = staged(d);
        const int s = d % kSlots;
        const unsigned char *blk = blocks + (size_t)s_off[d] * 16;
        bool timed_out = false;
        // a warp with no row in this level neither waits for its block nor
        // reads it (it only keeps the slot parities)
        constexpr int kRowsPerWarp = 32 / G;
        const bool mine = compute && warp * kRowsPerWarp < (int)s_rows[d];
        if (st && !mine) {
            phase ^= 1u << s;
        } else if (st) {
            // bounded wait for the bulk copy of this level
            const unsigned par = (phase >> s) & 1u;
            if (!mbar_try_wait(bar + s, par)) {
                const unsigned long long t0 = globaltimer_ns();
                while (!mbar_try_wait(bar + s, par)) {
                    if (globaltimer_ns() - t0 > kSpinLimitNs) {
                        timed_out = true;
                        break;
                    }
                }
            }
            phase ^= 1u << s;
            blk = ring + s_pos[s];
        }
        if (mine && !timed_out) cta_level<VT, G, EXACT>(blk, s_out, bit, dbit, warp, sub, g, ovf);
        // one barrier per level: results visible, the level's ring space free
        if (__syncthreads_or(timed_out)) {
            stuck = d;
            break;
        }
        if (producer) {
            if (st && --nst > 0) {
                for (int e = d + 1; e < issued; e++)
                    if (staged(e)) {
                        lo = s_pos[e % kSlots];
                        break;
                    }
            }
            issue_more(d + 1);
        }
    }
    if (stuck >= 0) {
        // report, then wait (bounded) for the copies this CTA still has in
        // flight before its shared memory goes away
        if (producer) {
            atomicOr(flags, ST_TIMEOUT);
            const unsigned long long t0 = globaltimer_ns();
            for (int dd = stuck; dd < issued; dd++) {
                if (!staged(dd)) continue;
                const int s = dd % kSlots;
                // the stuck level's wait already flipped its parity bit
                const unsigned par = ((phase >> s) & 1u) ^ (dd == stuck ? 1u : 0u);
                while (!mbar_try_wait(bar + s, par) && globaltimer_ns() - t0 < kSpinLimitNs) {
                }
            }
        }
        __syncthreads();
        return;
    }
    for (int i = threadIdx.x; i < n; i += kCtaThreads) out[i] = s_out[i];
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
    dfree(pk);
    dfree(flag);
    dfree(sync);
    dfree(blocks);
    dfree(blk_off);
    perm = prp = pci = chunk_lv = sub_bound = nullptr;
    pval = dinv = nullptr;
    pk = nullptr;
    flag = nullptr;
    sync = nullptr;
    blocks = nullptr;
    blk_off = nullptr;
}

template <typename T>
static void gather_vals(const TriSchedule &s, const T *vals, std::vector<T> &pv, std::vector<T> &dv) {
    pv.resize(s.src_idx.size());
    for (size_t j = 0; j < s.src_idx.size(); j++) pv[j] = vals[s.src_idx[j]];
    dv.assign(s.n, T(0));
    for (int p = 0; p < s.n; p++)
        if (s.diag_src[p] >= 0) dv[p] = vals[s.diag_src[p]];
}

static size_t up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// one block per level (see the layout above k_tri_cta)
template <typename T>
static void build_blocks(const TriSchedule &s, const std::vector<T> &pv, const std::vector<T> &dv,
                         std::vector<unsigned char> &blob, std::vector<long long> &off) {
    off.assign(s.nlev + 1, 0);
    blob.clear();
    for (int l = 0; l < s.nlev; l++) {
        const int p0 = s.lvl_ptr[l], p1 = s.lvl_ptr[l + 1];
        const int R = p1 - p0;
        const int e0 = s.prp[p0], e1 = s.prp[p1];
        const int E = e1 - e0;
        const size_t o_val = 32;
        const size_t o_dinv = up(o_val + sizeof(T) * E, 8);
        const size_t o_perm = up(o_dinv + sizeof(T) * R, 4);
        const size_t o_rp = o_perm + 4 * (size_t)R;
        const size_t o_pci = o_rp + 4 * (size_t)(R + 1);
        const size_t size = up(o_pci + 4 * (size_t)E, 16);
        const size_t base = blob.size();
        blob.resize(base + size, 0);
        unsigned char *b = blob.data() + base;
        int hdr[8] = {R, E, (int)o_val, (int)o_dinv, (int)o_perm, (int)o_rp, 0, 0};
        memcpy(b, hdr, sizeof hdr);
        memcpy(b + o_val, pv.data() + e0, sizeof(T) * E);
        memcpy(b + o_dinv, dv.data() + p0, sizeof(T) * R);
        memcpy(b + o_perm, s.perm.data() + p0, 4 * (size_t)R);
        int *rp = (int *)(b + o_rp);
        for (int r = 0; r <= R; r++) rp[r] = s.prp[p0 + r] - e0;
        memcpy(b + o_pci, s.pci.data() + e0, 4 * (size_t)E);
        off[l + 1] = (long long)blob.size();
    }
}

static int pow2_at_least(double x) {
    int g = 1;
    while (g < 32 && g < x) g <<= 1;
    return g;
}

DevTri upload_tri(const Ctx &c, int n, const int *rptr, const int *cind, const void *vals, int vt, int kind,
                  int bit, int dbit, const int *level_hint) {
    if (kind != TRI_LD) throw CudaError{"only LD sweeps are uploaded as sparse triangles"};
    DevTri d;
    d.n = n;
    d.kind = kind;
    d.vt = vt;
    d.bit = bit;
    d.dbit = dbit;
    const int64_t nnz = n ? rptr[n] : 0;
    const double avg = n ? (double)(nnz - n) / n : 0.0;
    const size_t es = vt_size(vt);
    const size_t vec_bytes = up((size_t)n * es, 16);
    d.one_cta = vec_bytes <= kCtaVecMax;
    int G = pow2_at_least(avg / (d.one_cta ? 4 : kBatch));
    if (vt != VT_I32 && c.fp_exact) G = 1;  // sequential order inside a row
    d.group = G;
    const int rows_per_chunk = 2 * kTriThreads / G;
    TriSchedule s = build_tri_schedule(rptr, cind, n, kind, rows_per_chunk, 1 << 20, level_hint);
    d.nlev = s.nlev;
    d.max_level_rows = s.max_level_rows;
    d.nnz_off = (int64_t)s.pci.size();
    d.nchunks = s.nchunks();
    std::vector<unsigned char> blob;
    std::vector<long long> off;
    auto put_vals = [&](auto tag) {
        using T = decltype(tag);
        std::vector<T> pv, dv;
        gather_vals(s, (const T *)vals, pv, dv);
        if (d.one_cta) {
            build_blocks(s, pv, dv, blob, off);
        } else {
            d.pval = pv.empty() ? dmalloc(16) : (void *)dupload(pv);
            d.dinv = dupload(dv);
        }
    };
    if (vt == VT_I32) put_vals(int32_t());
    else if (vt == VT_F64) put_vals(double());
    else put_vals(float());
    if (d.one_cta) {
        d.blocks = blob.empty() ? (unsigned char *)dmalloc(16) : dupload(blob);
        // block offsets in 16-byte units (nlev + 1), then the rows of each level (nlev)
        std::vector<unsigned> off16(off.size() + s.nlev);
        for (size_t i = 0; i < off.size(); i++) off16[i] = (unsigned)(off[i] / 16);
        for (int l = 0; l < s.nlev; l++) off16[off.size() + l] = (unsigned)(s.lvl_ptr[l + 1] - s.lvl_ptr[l]);
        d.blk_off = dupload(off16);
        const size_t offs_bytes = up(4 * (2 * (size_t)s.nlev + 1), 16);
        const size_t slot_bytes = 8 * kSlots + 4 * kSlots;  // mbarriers and ring positions
        if (vec_bytes + offs_bytes + slot_bytes + 4096 > kSmemMax)
            throw CudaError{"sweep schedule too large for the single-CTA kernel"};
        d.stage_bytes = (int)((kSmemMax - vec_bytes - offs_bytes - slot_bytes) / 16 * 16);
        d.cta_smem = vec_bytes + (size_t)d.stage_bytes + slot_bytes + offs_bytes;
    } else {
        d.perm = dupload(s.perm);
        d.prp = dupload(s.prp);
        d.pci = s.pci.empty() ? (int *)dmalloc(16) : dupload(s.pci);
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
        d.grid = std::max(1, std::min(d.nchunks, c.num_sms));
    }
    return d;
}

template <int VT, int G, bool EXACT>
static void launch_tri(Ctx &c, const DevTri &T, const void *in, void *out) {
    if (T.one_cta) {
        k_tri_cta<VT, G, EXACT><<<1, kCtaThreads, T.cta_smem, c.stream>>>(
            T.blocks, T.blk_off, T.nlev, T.n, T.bit, T.dbit, T.stage_bytes, in, out, c.d_flags);
    } else {
        TriArgs a{T.n, T.nchunks, T.bit, T.dbit, T.perm, T.prp, T.pci, T.pval, T.dinv,
                  T.chunk_lv, T.sub_bound, T.pk, T.flag, T.sync};
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

// ================================================ sweep without allocation
//
// For callers that cannot allocate device memory while they solve (their GPU
// memory is already claimed by another allocator, or they cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree imply).  The fine-level sweep
// kernel needs per-row scratch (the packed {epoch, value} words and the
// ticket/epoch block); this variant takes it from the file-scope array below
// instead of the schedule's own allocation.  The array is sized for
// kNoAllocRows rows (2 MiB) and every GPU that loads the library holds it
// until the process exits.  All calls share it and it keeps the last call's
// contents, so before each call the words of this level's rows and the
// ticket, done and epoch counters are cleared (a previous call may have left
// words of another precision there): every call starts at epoch 1 against
// zeroed words.  Calls that overlap on the GPU race on this array.
constexpr int kNoAllocRows = 262144;
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocRows + 2];

static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[64];

// The array's device address, looked up once per device with that device
// current (in host code the symbol is only a host-side stand-in).
static unsigned long long *noalloc_scratch(int device) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (device < 0 || device >= 64) throw CudaError{"device index out of range"};
    if (!g_noalloc_addr[device]) {
        int cur = -1;
        SAGB_CUDA(cudaGetDevice(&cur));
        if (cur != device) SAGB_CUDA(cudaSetDevice(device));
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (cur != device) cudaSetDevice(cur);
        if (e != cudaSuccess || !p) throw CudaError{std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)};
        g_noalloc_addr[device] = p;
    }
    return (unsigned long long *)g_noalloc_addr[device];
}

void trsv_noalloc(Ctx &c, const DevTri &T, const void *in, void *out) {
    if (T.n == 0 || T.one_cta) return trsv(c, T, in, out);  // shared memory only: no scratch
    if (T.n > kNoAllocRows)
        throw CudaError{"level has more than 262144 rows, the limit of the no-allocation sweep"};
    unsigned long long *s = noalloc_scratch(c.device);
    DevTri U = T;  // same schedule and operator, scratch from the static array
    U.pk = s;
    U.flag = (unsigned *)s;
    U.sync = (TriSync *)(s + kNoAllocRows);
    SAGB_CUDA(cudaMemsetAsync(s, 0, sizeof(unsigned long long) * (size_t)T.n, c.stream));
    SAGB_CUDA(cudaMemsetAsync(U.sync, 0, sizeof(TriSync), c.stream));  // ticket, done, epoch
    if (U.vt == VT_I32) return tri_by_group<VT_I32, false>(c, U, in, out);
    if (U.vt == VT_F64) {
        if (c.fp_exact) return tri_by_group<VT_F64, true>(c, U, in, out);
        return tri_by_group<VT_F64, false>(c, U, in, out);
    }
    if (c.fp_exact) return tri_by_group<VT_F32, true>(c, U, in, out);
    return tri_by_group<VT_F32, false>(c, U, in, out);
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
    using T = acc_t<VT>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
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
    for (int i = tid; i < n; i += kLuThreads) t[i] = acc_init<VT>(in[i], bitL);
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
                acc = acc_reduce<VT>(acc, 32);
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
    for (int i = tid; i < n; i += kLuThreads) t[i] = acc_init<VT>(x[i], bitU);
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
                acc = acc_reduce<VT>(acc, 32);
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
                    if (lane == c) xc = acc_finish<VT>(tr, dv, bitU, dbitU, ovf);
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
    const size_t smem = (sizeof(acc_t<VT>) + sizeof(vt_t<VT>)) * (size_t)LU.n;
    k_dense_lu<VT, EXACT><<<1, kLuThreads, smem, c.stream>>>(LU.n, LU.L, LU.U, LU.dinv, LU.bitL, LU.bitU,
                                                                LU.dbitU, in, out, c.d_flags);
    c.launches++;
}

template <int VT, bool EXACT>
static void cta_attrs() {
    const int mx = (int)kSmemMax;
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
    if ((size_t)LU.n * 16 > kSmemMax) throw CudaError{"coarsest level too large for the dense LU kernel"};
    if (LU.vt == VT_I32) return launch_lu<VT_I32, false>(c, LU, in, out);
    if (LU.vt == VT_F64) return c.fp_exact ? launch_lu<VT_F64, true>(c, LU, in, out)
                                           : launch_lu<VT_F64, false>(c, LU, in, out);
    return c.fp_exact ? launch_lu<VT_F32, true>(c, LU, in, out) : launch_lu<VT_F32, false>(c, LU, in, out);
}

}  // namespace sagb
