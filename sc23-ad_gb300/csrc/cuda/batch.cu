// Batched int-AMG-FGMRES: many independent systems of uneven size, each with
// R right-hand sides, advanced together so that every operation is one launch
// over the whole batch.
//
// Layout.  The systems' level operators are block-diagonal batch matrices
// (host/batch_setup.hpp) with one shift per row.  Vectors interleave the R
// right-hand sides of a row (x[row * R + r]), so a row's R values are one
// 4/8/16-byte load and every matrix entry is read once for all R of them.
//
// Per system and right-hand side ("pair"), the arithmetic is exactly that of
// the single-system solver with the multicolour smoother:
//   * V-cycle: intAMGflex::Precondition (INTAMG.hpp:269-293); the down pass of
//     all systems runs level by level, the coarsest LU of every system is one
//     launch (one CTA per system), then the up pass.
//   * sweeps: ldtri::MCCSR order (matrix/trispmat.hpp:597-640): one launch per
//     colour; the rows of a colour read only earlier colours.
//   * FGMRESflex::Solve (gmres.hpp:225-271) per pair: dots and norms are exact
//     int64 sums per pair (segmented by system), the Givens/e update and the
//     convergence test run one thread per pair, pairs that converge stop while
//     the others continue.
//   * Restarted::Solve (irsolver.hpp:27-43) per pair on the host, with the FP64
//     residual of every pair from one launch.
// Each Arnoldi step of the whole batch is captured once into a CUDA graph and
// replayed; the per-pair state lives in device memory, so the graph does not
// change when pairs stop or change fractional bits.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>

#include <cooperative_groups.h>

#include "../sagb_internal.hpp"
#include "common.cuh"
#include "cycle_graph.cuh"
#include "stream.cuh"

namespace sagb {

constexpr int kBThreads = 256;
constexpr int kTileRows = 2048;
constexpr int kBLuThreads = 512;  // 16 warps: room for 128 registers a thread


struct DBCsr {
    int n;
    const int *rptr, *cind, *val;
    const signed char *bit, *dbit;
    const short *cd;  // compressed columns: cind[j] = row + cd[j] (square operators whose offsets fit 16 bits)
};

template <int R>
__device__ __forceinline__ void load_r(const int *__restrict__ x, int row, int (&v)[R]) {
    if constexpr (R == 4) {
        const int4 q = __ldg(reinterpret_cast<const int4 *>(x) + row);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else if constexpr (R == 2) {
        const int2 q = __ldg(reinterpret_cast<const int2 *>(x) + row);
        v[0] = q.x; v[1] = q.y;
    } else {
        v[0] = __ldg(x + row);
    }
}
// plain (coherent) load: for vectors written earlier in the same sweep
template <int R>
__device__ __forceinline__ void load_rw(const int *x, int row, int (&v)[R]) {
    if constexpr (R == 4) {
        const int4 q = reinterpret_cast<const int4 *>(x)[row];
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else if constexpr (R == 2) {
        const int2 q = reinterpret_cast<const int2 *>(x)[row];
        v[0] = q.x; v[1] = q.y;
    } else {
        v[0] = x[row];
    }
}
template <int R>
__device__ __forceinline__ void load_cg_r(const int *x, int row, int (&v)[R]) {
    if constexpr (R == 4) {
        const int4 q = __ldcg(reinterpret_cast<const int4 *>(x) + row);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else if constexpr (R == 2) {
        const int2 q = __ldcg(reinterpret_cast<const int2 *>(x) + row);
        v[0] = q.x; v[1] = q.y;
    } else {
        v[0] = __ldcg(x + row);
    }
}
template <int R>
__device__ __forceinline__ void store_r(int *x, int row, const int (&v)[R]) {
    if constexpr (R == 4) reinterpret_cast<int4 *>(x)[row] = make_int4(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 2) reinterpret_cast<int2 *>(x)[row] = make_int2(v[0], v[1]);
    else x[row] = v[0];
}

// Row sums with four entries per lane in flight: the column indices and
// values of four entries are loaded together, then their four vector values,
// so a long row costs about a quarter of the dependent round trips.  Integer
// sums wrap, so the grouping does not change any result.
//   SUB = false: acc += a_ij x_j (x through the read-only cache)
//   SUB = true:  acc -= a_ij x_j (x written by earlier launches or colours:
//                plain loads)
//   CG:          x through L2 (written earlier in the same launch)
//   D16:         columns from the 16-bit offsets cd (column = row + cd[j])
template <int R, int G, bool SUB, bool CG, bool D16 = false, int U = 4>
__device__ __forceinline__ void row_accumulate(const int *__restrict__ cind, const short *__restrict__ cd,
                                               const int *__restrict__ val, int e0, int e1, int lane, int row,
                                               const int *x, long long (&acc)[R]) {
    int j = e0 + lane;
    for (; j + (U - 1) * G < e1; j += U * G) {
        int cc[U];
        long long vv[U];
#pragma unroll
        for (int q = 0; q < U; q++) {
            cc[q] = D16 ? row + (int)__ldg(cd + j + q * G) : __ldg(cind + j + q * G);
            vv[q] = __ldg(val + j + q * G);
        }
        int xv[U][R];
#pragma unroll
        for (int q = 0; q < U; q++) {
            if constexpr (CG) load_cg_r<R>(x, cc[q], xv[q]);
            else if constexpr (!SUB) load_r<R>(x, cc[q], xv[q]);
            else load_rw<R>(x, cc[q], xv[q]);
        }
#pragma unroll
        for (int q = 0; q < U; q++)
#pragma unroll
            for (int r = 0; r < R; r++) {
                if constexpr (SUB) acc[r] = wsub(acc[r], vv[q] * (long long)xv[q][r]);
                else acc[r] = wadd(acc[r], vv[q] * (long long)xv[q][r]);
            }
    }
    if (j < e1) {  // the last 1 .. U-1 entries of this lane: one predicated round, not one round trip each
        int cc[U - 1];
        long long vv[U - 1];
#pragma unroll
        for (int q = 0; q < U - 1; q++) {
            const int jj = j + q * G;
            const bool ok = jj < e1;
            cc[q] = ok ? (D16 ? row + (int)__ldg(cd + jj) : __ldg(cind + jj)) : -1;
            vv[q] = ok ? __ldg(val + jj) : 0;
        }
        int xv[U - 1][R];
#pragma unroll
        for (int q = 0; q < U - 1; q++) {
            if (cc[q] < 0) {
#pragma unroll
                for (int r = 0; r < R; r++) xv[q][r] = 0;
            } else if constexpr (CG) {
                load_cg_r<R>(x, cc[q], xv[q]);
            } else if constexpr (!SUB) {
                load_r<R>(x, cc[q], xv[q]);
            } else {
                load_rw<R>(x, cc[q], xv[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < U - 1; q++)
#pragma unroll
            for (int r = 0; r < R; r++) {
                if constexpr (SUB) acc[r] = wsub(acc[r], vv[q] * (long long)xv[q][r]);
                else acc[r] = wadd(acc[r], vv[q] * (long long)xv[q][r]);
            }
    }
}

// ------------------------------------------------------------------ SpMV
// The one-colour smoother step fused into a level SpMV's epilogue.  Where the
// multicolour split of a level kept a single colour, its LD is the diagonal
// alone and a sweep is out_i = (int)(((in_i << b) >> b) * dinv_i >> db)
// (ldtri.hpp:172-183 with no off-diagonal term): a function of the row's own
// input, so it is applied where that input is produced.
//   JAC_PRE:  y = R r (the next level's e) and also x2 = step(y) on that
//             level's smoothing rows (its pre-smoothing sweep from zero)
//   JAC_POST: y = step(z - U x) (the post-smoothing sweep; y is not x: the
//             product reads x of other rows)
enum { JAC_NONE = 0, JAC_PRE = 1, JAC_POST = 2 };
struct BJac {
    const int *dinv;                 // the one-colour LD's values (its inverted diagonal), one per row
    const signed char *bit, *dbit;   // its row shifts
    int n;                           // JAC_PRE: rows of y that smooth (a prefix)
    int *x2;                         // JAC_PRE: the step's output
};

// the sweep step of one row and right-hand side, with the colour kernel's overflow report
__device__ __forceinline__ int jac_step(int v, long long dinv, int bit, int dbit, bool &ovf) {
    const long long t = wshl((long long)v, bit);
    const long long s = wmul(t >> bit, dinv) >> dbit;
    ovf |= !fits32(s);
    return lo32(s);
}

// y = A x (SET), y = z - A x (RESID) or y = A x + y (ADD), per row shift;
// the same integer results as k_spmv_i32 for every right-hand side.
template <int R, int MODE, bool CG = false, int JAC = JAC_NONE>
__device__ __forceinline__ void bspmv_finish(const DBCsr &A, int row, const long long (&acc)[R], int *y,
                                             const int *z, const int *row_sys, unsigned *pflag, unsigned *flags,
                                             const BJac &J = BJac{}) {
    const int bit = A.bit[row];
    int out[R], zz[R], yy[R];
    if (MODE == SPMV_RESID) {
        if constexpr (CG) load_cg_r<R>(z, row, zz);
        else load_r<R>(z, row, zz);
    }
    if (MODE == SPMV_ADD) {
        if constexpr (CG) load_cg_r<R>(y, row, yy);
        else load_rw<R>(y, row, yy);
    }
    bool any = false;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const long long s = acc[r] >> bit;
        bool ovf = !fits32(s);
        long long v = (long long)lo32(s);
        if (MODE == SPMV_RESID) v = (long long)zz[r] - v;
        if (MODE == SPMV_ADD) v = v + (long long)yy[r];
        ovf |= !fits32(v);
        out[r] = lo32(v);
        if constexpr (JAC == JAC_POST)
            out[r] = jac_step(out[r], __ldg(J.dinv + row), J.bit[row], J.dbit[row], ovf);
        if (ovf) {
            atomicOr(pflag + (size_t)row_sys[row] * R + r, ST_OVERFLOW);
            any = true;
        }
    }
    store_r<R>(y, row, out);
    if constexpr (JAC == JAC_PRE) {
        if (row < J.n) {
            const long long dinv = __ldg(J.dinv + row);
            const int b = J.bit[row], db = J.dbit[row];
            int x2[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                bool ovf = false;
                x2[r] = jac_step(out[r], dinv, b, db, ovf);
                if (ovf) {
                    atomicOr(pflag + (size_t)row_sys[row] * R + r, ST_OVERFLOW);
                    any = true;
                }
            }
            store_r<R>(J.x2, row, x2);
        }
    }
    if (any) atomicOr(flags, ST_OVERFLOW);
}

// entries per lane fetched before the launch wait (level SpMVs); eight would
// cover a 7-point row in one round trip but take 48 registers a thread, and
// the lost occupancy cost more than the round trip saved (level-0 SpMV of
// Poisson 128^3: 26.9 us with four, 32.1 us with eight)
template <int R>
constexpr int spmv_pre() { return 4; }

template <int R, int G, int MODE, bool D16, int JAC = JAC_NONE>
__global__ void __launch_bounds__(kBThreads)
k_bspmv(DBCsr A, const int *__restrict__ x, int *__restrict__ y, const int *__restrict__ z,
        const int *__restrict__ row_sys, unsigned *__restrict__ pflag, unsigned *__restrict__ flags, BJac J) {
    pdl_trigger();
    constexpr int kSpmvPre = spmv_pre<R>();
    const long long tid = (long long)blockIdx.x * kBThreads + threadIdx.x;
    const int row = (int)(tid / G), lane = (int)(tid % G);
    long long acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    const int e0 = row < A.n ? __ldg(A.rptr + row) : 0, e1 = row < A.n ? __ldg(A.rptr + row + 1) : 0;
    // the first kSpmvPre entries of each lane are static: fetched before the
    // wait, so a row of up to kSpmvPre * G entries costs one round trip for
    // its entries and one for its vector values
    int cc[kSpmvPre], vv[kSpmvPre];
#pragma unroll
    for (int q = 0; q < kSpmvPre; q++) {
        const int j = e0 + lane + q * G;
        cc[q] = j < e1 ? (D16 ? row + (int)__ldg(A.cd + j) : __ldg(A.cind + j)) : -1;
        vv[q] = j < e1 ? __ldg(A.val + j) : 0;
    }
    pdl_wait();
    {
        int xv[kSpmvPre][R];
#pragma unroll
        for (int q = 0; q < kSpmvPre; q++) {
            if (cc[q] >= 0) load_r<R>(x, cc[q], xv[q]);
            else
#pragma unroll
                for (int r = 0; r < R; r++) xv[q][r] = 0;
        }
#pragma unroll
        for (int q = 0; q < kSpmvPre; q++)
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = wadd(acc[r], (long long)vv[q] * (long long)xv[q][r]);
    }
    // rows long enough for G >= 8 lanes: eight entries a lane in flight (a
    // warp then has 256 of a row's entries in flight at once)
    constexpr int kU = G >= 8 && R == 1 ? 8 : 4;
    if (e1 - e0 > kSpmvPre * G)
        row_accumulate<R, G, false, false, D16, kU>(A.cind, A.cd, A.val, e0 + kSpmvPre * G, e1, lane, row, x, acc);
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc[r] = wadd(acc[r], shfl_xor(acc[r], o));
    if (lane == 0 && row < A.n) bspmv_finish<R, MODE, false, JAC>(A, row, acc, y, z, row_sys, pflag, flags, J);
}

// the same rows through the tile-staged stream (short rows, group 0)
template <int R, int MODE, int JAC = JAC_NONE>
__global__ void __launch_bounds__(kStreamThreads)
k_bspmv_stream(DBCsr A, const int *__restrict__ x, int *__restrict__ y, const int *__restrict__ z,
               const int *__restrict__ row_sys, unsigned *__restrict__ pflag, unsigned *__restrict__ flags,
               BJac J) {
    pdl_trigger();
    long long acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    const int r0 = blockIdx.x * kStreamThreads;
    stream_rows<R, true>(r0, min(A.n, r0 + kStreamThreads), A.rptr, A.cind, A.val, x, acc);  // waits inside
    const int row = r0 + threadIdx.x;
    if (row < A.n) bspmv_finish<R, MODE, false, JAC>(A, row, acc, y, z, row_sys, pflag, flags, J);
}

// ------------------------------------------------------------ ELL SpMV
// Square level operators with short, even rows (the finest level of a stencil
// matrix) also keep their entries as ELL: w slots a row, slot-major (slot k
// of row i at k * n + i, coalesced across rows), 16-bit column offsets
// (column = row + offset), empty slots holding offset 0 and value 0.  A row's
// entries then need no row pointers: their loads depend on the row index
// alone and are all issued before the programmatic-launch wait, so after it a
// row costs one round trip for its vector values.  The sums are the CSR
// sums (integer, order-free; an empty slot adds 0).
constexpr int kEllMax = 8;

struct DEll {
    int n, w;
    const short *cd;  // w * n column offsets
    const int *val;   // w * n values
};

template <int R, int MODE, int JAC = JAC_NONE>
__global__ void __launch_bounds__(kBThreads)
k_bspmv_ell(DBCsr A, DEll E, const int *__restrict__ x, int *__restrict__ y, const int *__restrict__ z,
            const int *__restrict__ row_sys, unsigned *__restrict__ pflag, unsigned *__restrict__ flags, BJac J) {
    pdl_trigger();
    const int row = blockIdx.x * kBThreads + threadIdx.x;
    int cc[kEllMax], vv[kEllMax];
#pragma unroll
    for (int k = 0; k < kEllMax; k++) {
        const bool ok = row < E.n && k < E.w;
        vv[k] = ok ? __ldg(E.val + (size_t)k * E.n + row) : 0;
        cc[k] = ok ? row + (int)__ldg(E.cd + (size_t)k * E.n + row) : 0;
    }
    pdl_wait();
    long long acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    int xv[kEllMax][R];
#pragma unroll
    for (int k = 0; k < kEllMax; k++) {
        if (vv[k] != 0) load_r<R>(x, cc[k], xv[k]);
        else
#pragma unroll
            for (int r = 0; r < R; r++) xv[k][r] = 0;
    }
#pragma unroll
    for (int k = 0; k < kEllMax; k++)
#pragma unroll
        for (int r = 0; r < R; r++) acc[r] = wadd(acc[r], (long long)vv[k] * (long long)xv[k][r]);
    if (row < A.n) bspmv_finish<R, MODE, false, JAC>(A, row, acc, y, z, row_sys, pflag, flags, J);
}

// --------------------------------------------------------- colour sweep
// One colour of the multicolour Gauss-Seidel sweep (ldtri::CSRflex row rule,
// ldtri.hpp:172-183): t = in << b; t -= sum l_ij out_j; out = (int)((t >> b) * dinv >> db).
template <int R, int G>
__global__ void __launch_bounds__(kBThreads)
k_bcolour(int cnt, const int *__restrict__ rows, DBCsr LD, const int *__restrict__ in, int *out,
          const int *__restrict__ row_sys, unsigned *__restrict__ pflag, unsigned *__restrict__ flags) {
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * kBThreads + threadIdx.x;
    const int k = (int)(tid / G), lane = (int)(tid % G);
    long long acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    int row = -1, dpos = 0, e0 = 0;
    if (k < cnt) {
        row = __ldg(rows + k);
        e0 = __ldg(LD.rptr + row);
        dpos = __ldg(LD.rptr + row + 1) - 1;
    }
    pdl_wait();
    if (k < cnt) row_accumulate<R, G, true, false>(LD.cind, nullptr, LD.val, e0, dpos, lane, row, out, acc);
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc[r] = wadd(acc[r], shfl_xor(acc[r], o));
    if (lane == 0 && k < cnt) {
        const int bit = LD.bit[row], dbit = LD.dbit[row];
        const long long dinv = __ldg(LD.val + dpos);
        int iv[R], res[R];
        load_rw<R>(in, row, iv);
        bool any = false;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const long long t = wadd(wshl((long long)iv[r], bit), acc[r]);
            const long long s = wmul(t >> bit, dinv) >> dbit;
            res[r] = lo32(s);
            if (!fits32(s)) {
                atomicOr(pflag + (size_t)row_sys[row] * R + r, ST_OVERFLOW);
                any = true;
            }
        }
        store_r<R>(out, row, res);
        if (any) atomicOr(flags, ST_OVERFLOW);
    }
}

// ------------------------------------------------ cluster sweep (many colours)
// The whole sweep of one level in one launch: cluster g (kClusterCtas CTAs on
// as many SMs) owns a group of systems and walks their colours in order; the
// hardware cluster barrier (release / acquire) separates consecutive colours,
// so a level with hundreds of small colours costs one launch instead of one
// per colour.  Dependencies are read through L2 (ld.global.cg): another SM of
// the cluster wrote them in an earlier colour.
constexpr int kClusterCtas = 8;

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}


template <int R, int G>
__global__ void __launch_bounds__(kBThreads)
k_bsweep_cluster(const int *__restrict__ gc_ptr, const int *__restrict__ cbound, const int *__restrict__ grows,
                 DBCsr LD, const int *__restrict__ in, int *out, const int *__restrict__ row_sys,
                 unsigned *__restrict__ pflag, unsigned *__restrict__ flags) {
    pdl_trigger();
    pdl_wait();
    const int g = blockIdx.x / kClusterCtas, rank = blockIdx.x % kClusterCtas;
    const int t = rank * kBThreads + threadIdx.x;  // thread index inside the cluster
    const int lane = t % G, slot = t / G;
    constexpr int kSlots = kClusterCtas * kBThreads / G;  // rows in flight per pass
    const int c0 = gc_ptr[g], c1 = gc_ptr[g + 1];
    for (int k = c0; k + 1 < c1; k++) {
        const int a = cbound[k], b = cbound[k + 1];
        for (int base = a; base < b; base += kSlots) {
            const int idx = base + slot;
            long long acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            int row = -1, dpos = 0;
            if (idx < b) {
                row = __ldg(grows + idx);
                dpos = __ldg(LD.rptr + row + 1) - 1;
                row_accumulate<R, G, true, true>(LD.cind, nullptr, LD.val, __ldg(LD.rptr + row), dpos, lane, row, out,
                                                 acc);
            }
#pragma unroll
            for (int r = 0; r < R; r++)
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) acc[r] = wadd(acc[r], shfl_xor(acc[r], o));
            if (lane == 0 && idx < b) {
                const int bit = LD.bit[row], dbit = LD.dbit[row];
                const long long dinv = __ldg(LD.val + dpos);
                int iv[R], res[R];
                load_rw<R>(in, row, iv);
                bool any = false;
#pragma unroll
                for (int r = 0; r < R; r++) {
                    const long long tt = wadd(wshl((long long)iv[r], bit), acc[r]);
                    const long long sv = wmul(tt >> bit, dinv) >> dbit;
                    res[r] = lo32(sv);
                    if (!fits32(sv)) {
                        atomicOr(pflag + (size_t)row_sys[row] * R + r, ST_OVERFLOW);
                        any = true;
                    }
                }
                store_r<R>(out, row, res);
                if (any) atomicOr(flags, ST_OVERFLOW);
            }
        }
        cluster_barrier();
    }
}

// ------------------------------------ packed cluster sweep (coarse levels)
// The cluster sweep above spends most of a pass waiting on a chain of
// dependent loads (row list -> row pointers -> entries -> vector -> shifts)
// although only the vector values change during the sweep.  This form reads
// a copy of the level's LD packed at setup in the order the cluster consumes
// it: colour k's rows are dealt to the cluster's CTAs in turn (row i of the
// colour to CTA i % kClusterCtas), each (colour, CTA) run of rows is one
// contiguous range of items, and each item carries everything static about
// its row:
//   item = {row, first entry, inverse diagonal, meta}, meta = len | bit << 20 | dbit << 26
//   entry = {column, value} of the strictly lower part (the diagonal is the item's dinv)
// A CTA fetches the items, up to kPkU entries a lane and the input values of
// its next pass before it works on (and waits at the barrier after) the
// current one, so a pass costs one round trip for the vector values it reads
// plus the barrier.  Results are those of k_bcolour / k_bsweep_cluster.
constexpr int kPkU = 4;          // entries per lane fetched ahead; longer rows finish in a loop
// a CTA per SM with many loads in flight (four right-hand sides need the registers of 512)
template <int R>
constexpr int pk_threads() { return R == 4 ? 512 : 1024; }

template <int R>
struct PkPass {
    int4 hd;
    int2 e[kPkU];
    int iv[R];
    bool ok;
};

template <int R, int G, bool IN = true, bool INCG = false>
__device__ __forceinline__ void pk_fetch(const int4 *__restrict__ items, const int2 *__restrict__ ents,
                                         const int *__restrict__ in, int it, int ie, int lane, PkPass<R> &p) {
    p.ok = it < ie;
    p.hd = p.ok ? __ldg(items + it) : make_int4(0, 0, 0, 0);
    const int len = p.hd.w & 0xFFFFF;
#pragma unroll
    for (int u = 0; u < kPkU; u++) {
        const int j = lane + u * G;
        p.e[u] = j < len ? __ldg(ents + p.hd.y + j) : make_int2(0, 0);
    }
    if (IN && p.ok) {
        if constexpr (INCG) load_cg_r<R>(in, p.hd.x, p.iv);
        else load_r<R>(in, p.hd.x, p.iv);
    }
}

// One row of a packed sweep: subtract the lower entries' products (the first
// kPkU a lane already fetched in cur), then the SOR row update and the store
// (the row rule of k_bcolour).  CG: the vector values come from other CTAs of
// the same launch (read through L2).
template <int R, bool CG>
__device__ __forceinline__ void load_dep(const int *x, int row, int (&v)[R]) {
    if constexpr (CG) load_cg_r<R>(x, row, v);
    else load_rw<R>(x, row, v);
}

template <int R, int G, bool CG>
__device__ __forceinline__ void pk_row(const PkPass<R> &cur, const int2 *__restrict__ ents, int *out, int lane,
                                       const int *__restrict__ row_sys, unsigned *__restrict__ pflag,
                                       unsigned *__restrict__ flags) {
    long long acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    const int len = cur.hd.w & 0xFFFFF;
    {
        int xv[kPkU][R];
#pragma unroll
        for (int u = 0; u < kPkU; u++) {
            if (lane + u * G < len) load_dep<R, CG>(out, cur.e[u].x, xv[u]);
            else
#pragma unroll
                for (int r = 0; r < R; r++) xv[u][r] = 0;
        }
#pragma unroll
        for (int u = 0; u < kPkU; u++)
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], (long long)cur.e[u].y * (long long)xv[u][r]);
    }
    // rows longer than kPkU * G entries: four entries a lane in flight
    int j = lane + kPkU * G;
    for (; j + 3 * G < len; j += 4 * G) {
        int2 ev[4];
#pragma unroll
        for (int u = 0; u < 4; u++) ev[u] = __ldg(ents + cur.hd.y + j + u * G);
        int xv[4][R];
#pragma unroll
        for (int u = 0; u < 4; u++) load_dep<R, CG>(out, ev[u].x, xv[u]);
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], (long long)ev[u].y * (long long)xv[u][r]);
    }
    for (; j < len; j += G) {
        const int2 ev = __ldg(ents + cur.hd.y + j);
        int xv[R];
        load_dep<R, CG>(out, ev.x, xv);
#pragma unroll
        for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], (long long)ev.y * (long long)xv[r]);
    }
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc[r] = wadd(acc[r], shfl_xor(acc[r], o));
    if (lane == 0 && cur.ok) {
        const int row = cur.hd.x;
        const int bit = (cur.hd.w >> 20) & 63, dbit = (int)((unsigned)cur.hd.w >> 26);
        const long long dinv = cur.hd.z;
        int res[R];
        bool any = false;
#pragma unroll
        for (int r = 0; r < R; r++) {
            const long long tt = wadd(wshl((long long)cur.iv[r], bit), acc[r]);
            const long long sv = wmul(tt >> bit, dinv) >> dbit;
            res[r] = lo32(sv);
            if (!fits32(sv)) {
                atomicOr(pflag + (size_t)row_sys[row] * R + r, ST_OVERFLOW);
                any = true;
            }
        }
        store_r<R>(out, row, res);
        if (any) atomicOr(flags, ST_OVERFLOW);
    }
}

template <int R, int G>
__global__ void __launch_bounds__(pk_threads<R>())
k_bsweep_packed(const int *__restrict__ gc_ptr, const int *__restrict__ sw_ptr, const int4 *__restrict__ items,
                const int2 *__restrict__ ents, const int *__restrict__ in, int *out, const int *__restrict__ row_sys,
                unsigned *__restrict__ pflag, unsigned *__restrict__ flags) {
    pdl_trigger();
    const int g = blockIdx.x / kClusterCtas, q = blockIdx.x % kClusterCtas;
    const int lane = threadIdx.x % G, ls = threadIdx.x / G;
    constexpr int kS = pk_threads<R>() / G;  // rows of one pass of this CTA
    const int k1 = gc_ptr[g + 1] - 1;  // colours k of the group: gc_ptr[g] <= k < k1
    int k = gc_ptr[g];
    if (k >= k1) {  // a group without colours (no barrier is reached by any CTA of it)
        pdl_wait();
        return;
    }
    int ie = __ldg(sw_ptr + k * kClusterCtas + q + 1);
    int base = __ldg(sw_ptr + k * kClusterCtas + q);
    PkPass<R> cur, nxt;
    pk_fetch<R, G, false>(items, ents, in, base + ls, ie, lane, cur);  // the packed LD does not change
    pdl_wait();
    if (cur.ok) load_r<R>(in, cur.hd.x, cur.iv);
    while (k < k1) {
        // the next pass: more rows of this colour, or the next colour's first
        int nk = k, nbase = base + kS, nie = ie;
        const bool colour_end = nbase >= ie;
        if (colour_end) {
            nk = k + 1;
            if (nk < k1) {
                nbase = __ldg(sw_ptr + nk * kClusterCtas + q);
                nie = __ldg(sw_ptr + nk * kClusterCtas + q + 1);
            }
        }
        if (nk < k1) pk_fetch<R, G>(items, ents, in, nbase + ls, nie, lane, nxt);
        else nxt.ok = false;

        pk_row<R, G, true>(cur, ents, out, lane, row_sys, pflag, flags);
        if (colour_end) cluster_barrier();
        cur = nxt;
        k = nk;
        base = nbase;
        ie = nie;
    }
}

// One colour of the sweep over a packed copy of LD in colour order (the
// items of colour k are ib..ie-1): the item, its first entries and (after the
// wait for the previous kernel) its input value come in one round trip each,
// the vector values of the earlier colours in one more.
template <int R, int G>
__global__ void __launch_bounds__(kBThreads)
k_bcolour_packed(int ib, int ie, const int4 *__restrict__ items, const int2 *__restrict__ ents,
                 const int *__restrict__ in, int *out, const int *__restrict__ row_sys, unsigned *__restrict__ pflag,
                 unsigned *__restrict__ flags) {
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * kBThreads + threadIdx.x;
    const int lane = (int)(tid % G);
    const long long it = ib + tid / G;
    PkPass<R> cur;
    pk_fetch<R, G, false>(items, ents, in, it < ie ? (int)it : ie, ie, lane, cur);
    pdl_wait();
    if (cur.ok) load_r<R>(in, cur.hd.x, cur.iv);
    pk_row<R, G, false>(cur, ents, out, lane, row_sys, pflag, flags);
}

// ------------------------------------------------------------ coarse LU
struct BLuDesc {
    int n, sys;
    int bitL, bitU, dbitU;
    long long mat_off, d_off;  // offsets into the concatenated L/U and dinv arrays
    const int *in;             // the system's rows of its LU level (interleaved)
    int *out;
};

// LUflex::Solve (solver/lu.hpp:91-94) for every system of the batch: one CTA
// per system, R right-hand sides at once.  Same panel algorithm as the
// single-system dense LU kernel: 32-row panels, warps reduce a panel row
// against the solved part, warp 0 solves the diagonal block from registers.
// The LU solves of one system by the NT threads of one CTA (the body of
// k_blu; CG: the input was written earlier in the same launch).
template <int R, int NT, bool CG>
__device__ void blu_body(const BLuDesc &d, const int *__restrict__ Lcat, const int *__restrict__ Ucat,
                         const int *__restrict__ dcat, unsigned *__restrict__ pflag, unsigned *__restrict__ flags,
                         unsigned char *smem_raw) {
    const int n = d.n;
    long long *t = (long long *)smem_raw;              // n * R accumulators
    int *x = (int *)(smem_raw + sizeof(long long) * (size_t)n * R);  // n * R values
    const int *L = Lcat + d.mat_off, *U = Ucat + d.mat_off, *dinv = dcat + d.d_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned ovf = 0;
    for (int i = tid; i < n * R; i += NT) t[i] = wshl((long long)(CG ? __ldcg(d.in + i) : d.in[i]), d.bitL);
    __syncthreads();
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int kb = min(32, n - k0);
        for (int pr = warp; k0 > 0 && pr < kb; pr += NT / 32) {
            const int *row = L + (size_t)(k0 + pr) * n;
            long long acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            for (int c = lane; c < k0; c += 32) {
                const long long v = __ldg(row + c);
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], v * (long long)x[c * R + r]);
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
                for (int o = 16; o > 0; o >>= 1) acc[r] = wadd(acc[r], shfl_xor(acc[r], o));
                if (lane == 0) t[(k0 + pr) * R + r] = wadd(t[(k0 + pr) * R + r], acc[r]);
            }
        }
        __syncthreads();
        if (warp == 0) {
            int dblk[32];
            const int *row = L + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) dblk[c] = (lane < kb && c < lane) ? __ldg(row + c) : 0;
            long long tr[R];
#pragma unroll
            for (int r = 0; r < R; r++) tr[r] = lane < kb ? t[(k0 + lane) * R + r] : 0;
#pragma unroll
            for (int c = 0; c < 32; c++) {
                if (c < kb) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const long long s = tr[r] >> d.bitL;
                        if (lane == c && !fits32(s)) ovf |= 1u << r;
                        const int xc = __shfl_sync(0xffffffffu, lo32(s), c);
                        if (lane > c) tr[r] = wsub(tr[r], (long long)dblk[c] * xc);
                        if (lane == c) x[(k0 + c) * R + r] = xc;
                    }
                }
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < n * R; i += NT) t[i] = wshl((long long)x[i], d.bitU);
    __syncthreads();
    for (int k1 = n; k1 > 0; k1 -= 32) {
        const int kb = min(32, k1);
        const int k0 = k1 - kb;
        for (int pr = warp; k1 < n && pr < kb; pr += NT / 32) {
            const int *row = U + (size_t)(k0 + pr) * n;
            long long acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            for (int c = k1 + lane; c < n; c += 32) {
                const long long v = __ldg(row + c);
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], v * (long long)x[c * R + r]);
            }
#pragma unroll
            for (int r = 0; r < R; r++) {
                for (int o = 16; o > 0; o >>= 1) acc[r] = wadd(acc[r], shfl_xor(acc[r], o));
                if (lane == 0) t[(k0 + pr) * R + r] = wadd(t[(k0 + pr) * R + r], acc[r]);
            }
        }
        __syncthreads();
        if (warp == 0) {
            int dblk[32];
            const int *row = U + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) dblk[c] = (lane < kb && c > lane && c < kb) ? __ldg(row + c) : 0;
            long long tr[R];
#pragma unroll
            for (int r = 0; r < R; r++) tr[r] = lane < kb ? t[(k0 + lane) * R + r] : 0;
            const long long dv = lane < kb ? (long long)__ldg(dinv + k0 + lane) : 0;
#pragma unroll
            for (int c = 31; c >= 0; c--) {
                if (c < kb) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        int xc = 0;
                        if (lane == c) {
                            const long long s = wmul(tr[r] >> d.bitU, dv) >> d.dbitU;
                            if (!fits32(s)) ovf |= 1u << r;
                            xc = lo32(s);
                        }
                        xc = __shfl_sync(0xffffffffu, xc, c);
                        if (lane < c) tr[r] = wsub(tr[r], (long long)dblk[c] * xc);
                        if (lane == c) x[(k0 + c) * R + r] = xc;
                    }
                }
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < n * R; i += NT) d.out[i] = x[i];
    if (ovf) {
        for (int r = 0; r < R; r++)
            if (ovf & (1u << r)) atomicOr(pflag + (size_t)d.sys * R + r, ST_OVERFLOW);
        atomicOr(flags, ST_OVERFLOW);
    }
}

template <int R>
__global__ void __launch_bounds__(kBLuThreads, 1)
k_blu(const BLuDesc *__restrict__ desc, const int *__restrict__ Lcat, const int *__restrict__ Ucat,
      const int *__restrict__ dcat, unsigned *__restrict__ pflag, unsigned *__restrict__ flags) {
    pdl_trigger();
    pdl_wait();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    blu_body<R, kBLuThreads, false>(desc[blockIdx.x], Lcat, Ucat, dcat, pflag, flags, smem_raw);
}

// ------------------------------------------- persistent coarse tail of the V-cycle
// The coarse levels t .. Dmax-1 and the coarsest LU in one cooperative launch:
// every CTA is resident (one per SM), the steps (one colour of a sweep, one
// SpMV, the LU solves) run one after the other over the whole grid with a
// grid barrier between them, instead of one dependent launch each.  Each step
// computes what its launch computes (the same row rules and overflow flags);
// vectors written earlier in the launch are read through L2.  The barrier's
// wait is bounded in time (ST_TIMEOUT in the main status word, then every CTA
// returns).
constexpr int kTailThreads = 512;
constexpr int kTailSmem = 200 * 1024;  // the LU's shared memory; the kernel's own few bytes come on top
enum TailKind : int { TK_COLOUR = 0, TK_RESID = 1, TK_SET = 2, TK_ADD = 3, TK_LU = 4 };
struct TailStep {
    int kind, G, ib, ie;  // colour: items ib..ie-1 of the packed LD; SpMV: all rows of M
    DBCsr M;
    const int4 *items;
    const int2 *ents;
    const int *x;  // SpMV input; colour: unused
    int *y;        // SpMV output; colour: the vector being swept
    const int *z;  // SpMV residual minuend; colour: the sweep's input
    const int *row_sys;
};

template <int R, int G>
__device__ __forceinline__ void tail_colour(const TailStep &st, unsigned *pflag, unsigned *flags) {
    const long long tid = (long long)blockIdx.x * kTailThreads + threadIdx.x;
    const long long slots = (long long)gridDim.x * kTailThreads / G;
    const int lane = (int)(tid % G);
    for (long long base = st.ib; base < st.ie; base += slots) {
        const long long it = base + tid / G;
        PkPass<R> cur;
        pk_fetch<R, G, true, true>(st.items, st.ents, st.z, it < st.ie ? (int)it : st.ie, st.ie, lane, cur);
        pk_row<R, G, true>(cur, st.ents, st.y, lane, st.row_sys, pflag, flags);
    }
}

template <int R, int G, int MODE>
__device__ __forceinline__ void tail_spmv(const TailStep &st, unsigned *pflag, unsigned *flags) {
    const DBCsr &A = st.M;
    const long long tid = (long long)blockIdx.x * kTailThreads + threadIdx.x;
    const long long rows = (long long)gridDim.x * kTailThreads / G;
    const int lane = (int)(tid % G);
    for (long long base = 0; base < A.n; base += rows) {
        const long long r = base + tid / G;
        const int row = r < A.n ? (int)r : -1;
        long long acc[R];
#pragma unroll
        for (int q = 0; q < R; q++) acc[q] = 0;
        if (row >= 0)
            row_accumulate<R, G, false, true>(A.cind, nullptr, A.val, __ldg(A.rptr + row), __ldg(A.rptr + row + 1),
                                              lane, row, st.x, acc);
#pragma unroll
        for (int q = 0; q < R; q++)
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) acc[q] = wadd(acc[q], shfl_xor(acc[q], o));
        if (lane == 0 && row >= 0) bspmv_finish<R, MODE, true>(A, row, acc, st.y, st.z, st.row_sys, pflag, flags);
    }
}

// Grid barrier k of a launch: every CTA adds one to the arrival counter
// bar[0] and waits until it reaches (k + 1) * (gridDim.x + extra) (extra = 0;
// the self-test's 1 makes the wait run out).  The wait is bounded by limit_ns;
// when it runs out the CTA marks bar[1] (both words are zeroed before each
// launch) and the caller's status word, and every CTA that sees bar[1] set
// stops waiting.  Returns false then.
__device__ __forceinline__ bool tail_barrier(unsigned *bar, unsigned k, unsigned *status, unsigned extra,
                                             unsigned long long limit_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        const unsigned target = (k + 1) * (gridDim.x + extra);
        int ok = 1;
        const unsigned long long t0 = globaltimer_ns();
        while (*(volatile unsigned *)bar < target) {
            if (*(volatile unsigned *)(bar + 1) & ST_TIMEOUT) {
                ok = 0;
                break;
            }
            if (globaltimer_ns() - t0 > limit_ns) {
                atomicOr(bar + 1, ST_TIMEOUT);
                atomicOr(status, ST_TIMEOUT);
                ok = 0;
                break;
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <int R>
__global__ void __launch_bounds__(kTailThreads, 1)
k_btail(const TailStep *__restrict__ steps, int nsteps, const BLuDesc *__restrict__ lu, int nlu,
        const int *__restrict__ Lcat, const int *__restrict__ Ucat, const int *__restrict__ dcat, unsigned *bar,
        unsigned *__restrict__ pflag, unsigned *__restrict__ flags, unsigned *__restrict__ status, unsigned extra,
        unsigned long long limit_ns) {
    pdl_trigger();
    pdl_wait();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    for (int k = 0; k < nsteps; k++) {
        const TailStep st = steps[k];
        if (st.kind == TK_LU) {
            for (int sys = blockIdx.x; sys < nlu; sys += gridDim.x)
                blu_body<R, kTailThreads, true>(lu[sys], Lcat, Ucat, dcat, pflag, flags, smem_raw);
        } else {
            switch (st.G) {
#define SAGB_TAIL_G(GV)                                                                      \
    case GV:                                                                                 \
        if (st.kind == TK_COLOUR) tail_colour<R, GV>(st, pflag, flags);                     \
        else if (st.kind == TK_RESID) tail_spmv<R, GV, SPMV_RESID>(st, pflag, flags);       \
        else if (st.kind == TK_SET) tail_spmv<R, GV, SPMV_SET>(st, pflag, flags);           \
        else tail_spmv<R, GV, SPMV_ADD>(st, pflag, flags);                                  \
        break;
                SAGB_TAIL_G(1)
                SAGB_TAIL_G(2)
                SAGB_TAIL_G(4)
                SAGB_TAIL_G(8)
                SAGB_TAIL_G(16)
                default:
                SAGB_TAIL_G(32)
#undef SAGB_TAIL_G
            }
        }
        if (!tail_barrier(bar, (unsigned)k, status, extra, limit_ns)) return;
    }
}


// The same LU solves spread over a thread-block cluster (kLuCtas CTAs, one
// system per cluster).  Panel p of 32 rows belongs to CTA p % kLuCtas, which
// keeps the int64 accumulators of its rows in its own shared memory; every CTA
// keeps a full copy of the solved values.  Per panel: the owner solves the
// 32x32 diagonal block (warp 0, block in registers) and writes the 32 values
// into every CTA's copy (distributed shared memory); one cluster barrier; then
// each CTA subtracts the panel's columns from its own later rows (one thread
// per row).  Each CTA thus reads only its own rows of L and U, so the factors
// stream through kLuCtas SMs instead of one.  Integer sums wrap, so the
// results are those of k_blu.
constexpr int kLuCtas = 8;
constexpr int kLuCThreads = 256;

template <int R>
__global__ void __launch_bounds__(kLuCThreads, 1)
k_blu_cluster(const BLuDesc *__restrict__ desc, const int *__restrict__ Lcat, const int *__restrict__ Ucat,
              const int *__restrict__ dcat, unsigned *__restrict__ pflag, unsigned *__restrict__ flags) {
    pdl_trigger();
    pdl_wait();
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const BLuDesc d = desc[blockIdx.x / kLuCtas];
    const int q = (int)cl.block_rank();
    const int n = d.n, npan = (n + 31) / 32;
    const int nown = q < npan ? (npan - q + kLuCtas - 1) / kLuCtas : 0;  // panels q, q + C, ...
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int *xs = (int *)smem_raw;                                                   // n * R solved values
    long long *t = (long long *)(smem_raw + (((size_t)n * R * sizeof(int) + 15) & ~(size_t)15));  // own rows
    const int *L = Lcat + d.mat_off, *U = Ucat + d.mat_off, *dinv = dcat + d.d_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned ovf = 0;
    // own row lr (local) <-> global row (q + (lr / 32) * C) * 32 + lr % 32
    auto grow = [&](int lr) { return (q + (lr >> 5) * kLuCtas) * 32 + (lr & 31); };
    for (int i = tid; i < nown * 32 * R; i += kLuCThreads) {
        const int lr = i / R, r = i % R, g = grow(lr);
        t[i] = g < n ? wshl((long long)d.in[(size_t)g * R + r], d.bitL) : 0;
    }
    __syncthreads();
    // ---------------- forward: unit lower
    for (int p = 0; p < npan; p++) {
        const int k0 = p * 32, kb = min(32, n - k0);
        if (p % kLuCtas == q && warp == 0) {
            const int lp = p / kLuCtas;
            int dblk[32];
            const int *row = L + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) dblk[c] = (lane < kb && c < lane) ? __ldg(row + c) : 0;
            long long tr[R];
#pragma unroll
            for (int r = 0; r < R; r++) tr[r] = lane < kb ? t[(lp * 32 + lane) * R + r] : 0;
            int xv[R];
#pragma unroll
            for (int r = 0; r < R; r++) xv[r] = 0;
#pragma unroll
            for (int c = 0; c < 32; c++) {
                if (c < kb) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const long long sv = tr[r] >> d.bitL;
                        if (lane == c && !fits32(sv)) ovf |= 1u << r;
                        const int xc = __shfl_sync(0xffffffffu, lo32(sv), c);
                        if (lane > c) tr[r] = wsub(tr[r], (long long)dblk[c] * xc);
                        if (lane == c) xv[r] = xc;
                    }
                }
            }
            if (lane < kb)
                for (int dst = 0; dst < kLuCtas; dst++) {
                    int *rx = cl.map_shared_rank(xs, dst);
#pragma unroll
                    for (int r = 0; r < R; r++) rx[(k0 + lane) * R + r] = xv[r];
                }
        }
        cl.sync();
        // own rows of later panels: t_i -= L[i][k0 .. k0+kb) x
        const int lp_first = p < q ? 0 : (p - q) / kLuCtas + 1;
        for (int lr = lp_first * 32 + tid; lr < nown * 32; lr += kLuCThreads) {
            const int g = grow(lr);
            if (g >= n) continue;
            const int *row = L + (size_t)g * n + k0;
            long long acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            if (kb == 32) {
                int v[32];  // the row's 32 entries in flight together
#pragma unroll
                for (int c = 0; c < 32; c++) v[c] = __ldg(row + c);
#pragma unroll
                for (int c = 0; c < 32; c++)
#pragma unroll
                    for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], (long long)v[c] * xs[(k0 + c) * R + r]);
            } else {
                for (int c = 0; c < kb; c++) {
                    const long long v = __ldg(row + c);
#pragma unroll
                    for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], v * (long long)xs[(k0 + c) * R + r]);
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) t[lr * R + r] = wadd(t[lr * R + r], acc[r]);
        }
        __syncthreads();
    }
    // ---------------- backward: D^-1 U, last panel first
    for (int i = tid; i < nown * 32 * R; i += kLuCThreads) {
        const int lr = i / R, r = i % R, g = grow(lr);
        t[i] = g < n ? wshl((long long)xs[(size_t)g * R + r], d.bitU) : 0;
    }
    cl.sync();  // every CTA has read its x before the backward values overwrite them
    for (int p = npan - 1; p >= 0; p--) {
        const int k0 = p * 32, kb = min(32, n - k0);
        if (p % kLuCtas == q && warp == 0) {
            const int lp = p / kLuCtas;
            int dblk[32];
            const int *row = U + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) dblk[c] = (lane < kb && c > lane && c < kb) ? __ldg(row + c) : 0;
            long long tr[R];
#pragma unroll
            for (int r = 0; r < R; r++) tr[r] = lane < kb ? t[(lp * 32 + lane) * R + r] : 0;
            const long long dv = lane < kb ? (long long)__ldg(dinv + k0 + lane) : 0;
            int xv[R];
#pragma unroll
            for (int r = 0; r < R; r++) xv[r] = 0;
#pragma unroll
            for (int c = 31; c >= 0; c--) {
                if (c < kb) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        int xc = 0;
                        if (lane == c) {
                            const long long sv = wmul(tr[r] >> d.bitU, dv) >> d.dbitU;
                            if (!fits32(sv)) ovf |= 1u << r;
                            xc = lo32(sv);
                        }
                        xc = __shfl_sync(0xffffffffu, xc, c);
                        if (lane < c) tr[r] = wsub(tr[r], (long long)dblk[c] * xc);
                        if (lane == c) xv[r] = xc;
                    }
                }
            }
            if (lane < kb)
                for (int dst = 0; dst < kLuCtas; dst++) {
                    int *rx = cl.map_shared_rank(xs, dst);
#pragma unroll
                    for (int r = 0; r < R; r++) rx[(k0 + lane) * R + r] = xv[r];
                }
        }
        cl.sync();
        // own rows of earlier panels: t_i -= U[i][k0 .. k0+kb) x
        const int lp_last = p > q ? (p - q - 1) / kLuCtas + 1 : 0;  // own panels strictly before p
        for (int lr = tid; lr < lp_last * 32; lr += kLuCThreads) {
            const int g = grow(lr);
            const int *row = U + (size_t)g * n + k0;
            long long acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            if (kb == 32) {
                int v[32];  // the row's 32 entries in flight together
#pragma unroll
                for (int c = 0; c < 32; c++) v[c] = __ldg(row + c);
#pragma unroll
                for (int c = 0; c < 32; c++)
#pragma unroll
                    for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], (long long)v[c] * xs[(k0 + c) * R + r]);
            } else {
                for (int c = 0; c < kb; c++) {
                    const long long v = __ldg(row + c);
#pragma unroll
                    for (int r = 0; r < R; r++) acc[r] = wsub(acc[r], v * (long long)xs[(k0 + c) * R + r]);
                }
            }
#pragma unroll
            for (int r = 0; r < R; r++) t[lr * R + r] = wadd(t[lr * R + r], acc[r]);
        }
        __syncthreads();
    }
    // every CTA holds all values: CTA q writes its own panels
    for (int i = tid; i < nown * 32 * R; i += kLuCThreads) {
        const int lr = i / R, r = i % R, g = grow(lr);
        if (g < n) d.out[(size_t)g * R + r] = xs[(size_t)g * R + r];
    }
    if (ovf) {
        for (int r = 0; r < R; r++)
            if (ovf & (1u << r)) atomicOr(pflag + (size_t)d.sys * R + r, ST_OVERFLOW);
        atomicOr(flags, ST_OVERFLOW);
    }
}

// ============================================================== Krylov

struct BTile {
    int sys, row0, row1, first;  // rows [row0, row1) of one system; first tile of that system
};

struct BPair {
    double e0, e_inv, nrm_b, relres;
    long long criteria, hinv;
    long long cycle_target;  // the cycle ends once |e_{j+1}| <= this (-1: never)
    int bit, active, jn, conv;
    unsigned bad;  // status bits seen while the pair was active (the cycle is discarded)
    int pad;
};

struct BInfo {
    int n_active;
    unsigned flags;
};

// fixed-order block sum of R int64 partials (wrapping); result valid in thread 0
template <int R>
__device__ __forceinline__ void bsum_i64(long long (&v)[R], long long (*sh)[R]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[r] = wadd(v[r], shfl_xor(v[r], o));
    if (lane == 0)
#pragma unroll
        for (int r = 0; r < R; r++) sh[warp][r] = v[r];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            long long s = 0;
            for (int w = 0; w < kBThreads / 32; w++) s = wadd(s, sh[w][r]);
            v[r] = s;
        }
    }
    __syncthreads();
}

template <int R>
__device__ __forceinline__ void bsum_f64(double (&v)[R], double (*sh)[R]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[r] += __shfl_xor_sync(0xffffffffu, v[r], o);
    if (lane == 0)
#pragma unroll
        for (int r = 0; r < R; r++) sh[warp][r] = v[r];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            double s = 0;
            for (int w = 0; w < kBThreads / 32; w++) s += sh[w][r];
            v[r] = s;
        }
    }
    __syncthreads();
}

// FGMRESflex::Solve prologue per pair (gmres.hpp:228-233)
__global__ void k_bbegin(int P, const double *__restrict__ e0, double eps, BPair *pairs, long long *e,
                         unsigned long long *acc, int m, int cycle_bits) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    BPair &q = pairs[p];
    q.jn = 0;
    q.conv = 0;
    q.bad = 0;
    q.cycle_target = cycle_bits <= 0 ? -1 : q.bit > cycle_bits ? 1LL << (q.bit - cycle_bits) : 1;
    for (int k = 0; k <= m + 1; k++) acc[(size_t)p * (m + 2) + k] = 0;
    if (!q.active) return;
    const double fact = (double)(1LL << q.bit);
    q.e0 = e0[p];
    q.e_inv = 1.0 / q.e0;
    q.criteria = d2l_x86(__dmul_rn(__dmul_rn(__dmul_rn(q.nrm_b, eps), q.e_inv), fact));
    e[(size_t)p * (m + 1)] = 1LL << q.bit;
}

// the elementwise Krylov kernels run one row per thread: block b covers rows
// row0 + (b % kTileSub) * kBThreads + [0, kBThreads) of tile b / kTileSub
constexpr int kTileSub = kTileRows / kBThreads;

template <int R>
__global__ void __launch_bounds__(kBThreads)
k_bv0(const BTile *__restrict__ tiles, const double *__restrict__ rv, const BPair *__restrict__ pairs,
      int *__restrict__ V0) {
    const BTile t = tiles[blockIdx.x / kTileSub];
    const int i = t.row0 + (blockIdx.x % kTileSub) * kBThreads + threadIdx.x;
    if (i >= t.row1) return;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const BPair &q = pairs[t.sys * R + r];
        if (!q.active) continue;
        const double fact = (double)(1LL << q.bit);
        V0[(size_t)i * R + r] = d2i_x86(__dmul_rn(__dmul_rn(__ldg(rv + (size_t)i * R + r), q.e_inv), fact));
    }
}

// w = A z on the tile's rows and acc[p][0] += V0 . w
template <int R, int G, bool D16>
__global__ void __launch_bounds__(kBThreads)
k_bspmv_dot(const BTile *__restrict__ tiles, DBCsr A, const int *__restrict__ z, int *__restrict__ w,
            const int *__restrict__ v0, const BPair *__restrict__ pairs, unsigned long long *acc, int m,
            unsigned *__restrict__ pflag, unsigned *__restrict__ flags) {
    pdl_trigger();
    pdl_wait();
    __shared__ long long sh[kBThreads / 32][R];
    const BTile t = tiles[blockIdx.x];
    const int lane = threadIdx.x % G;
    long long dot[R];
#pragma unroll
    for (int r = 0; r < R; r++) dot[r] = 0;
    unsigned ovf = 0;
    for (int row0 = t.row0; row0 < t.row1; row0 += kBThreads / G) {
        const int row = row0 + threadIdx.x / G;
        long long a[R];
#pragma unroll
        for (int r = 0; r < R; r++) a[r] = 0;
        if (row < t.row1)
            row_accumulate<R, G, false, false, D16>(A.cind, A.cd, A.val, __ldg(A.rptr + row), __ldg(A.rptr + row + 1),
                                                    lane, row, z, a);
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) a[r] = wadd(a[r], shfl_xor(a[r], o));
        if (lane == 0 && row < t.row1) {
            const int bit = A.bit[row];
            int y[R], vv[R];
            load_r<R>(v0, row, vv);
#pragma unroll
            for (int r = 0; r < R; r++) {
                const long long s = a[r] >> bit;
                if (!fits32(s)) ovf |= 1u << r;
                y[r] = lo32(s);
                dot[r] = wadd(dot[r], (long long)vv[r] * y[r]);
            }
            store_r<R>(w, row, y);
        }
    }
    bsum_i64<R>(dot, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) atomicAdd(acc + (size_t)(t.sys * R + r) * (m + 2), (unsigned long long)dot[r]);
    if (ovf) {
#pragma unroll
        for (int r = 0; r < R; r++)
            if (ovf & (1u << r)) atomicOr(pflag + (size_t)t.sys * R + r, ST_OVERFLOW);
        atomicOr(flags, ST_OVERFLOW);
    }
}

// w = A z and acc[p][0] += V0 . w through the tile-staged stream; one CTA per
// tile of at most kStreamThreads rows of one system
template <int R>
__global__ void __launch_bounds__(kStreamThreads)
k_bspmv_dot_stream(const BTile *__restrict__ tiles, DBCsr A, const int *__restrict__ z, int *__restrict__ w,
                   const int *__restrict__ v0, unsigned long long *acc, int m, unsigned *__restrict__ pflag,
                   unsigned *__restrict__ flags) {
    pdl_trigger();
    pdl_wait();
    __shared__ long long sh[kStreamThreads / 32][R];
    const BTile t = tiles[blockIdx.x];
    long long a[R], dot[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = dot[r] = 0;
    stream_rows<R>(t.row0, t.row1, A.rptr, A.cind, A.val, z, a);
    const int row = t.row0 + threadIdx.x;
    unsigned ovf = 0;
    if (row < t.row1) {
        const int bit = A.bit[row];
        int y[R], vv[R];
        load_r<R>(v0, row, vv);
#pragma unroll
        for (int r = 0; r < R; r++) {
            const long long s = a[r] >> bit;
            if (!fits32(s)) ovf |= 1u << r;
            y[r] = lo32(s);
            dot[r] = (long long)vv[r] * y[r];
        }
        store_r<R>(w, row, y);
    }
    bsum_i64<R>(dot, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) atomicAdd(acc + (size_t)(t.sys * R + r) * (m + 2), (unsigned long long)dot[r]);
    if (ovf) {
#pragma unroll
        for (int r = 0; r < R; r++)
            if (ovf & (1u << r)) atomicOr(pflag + (size_t)t.sys * R + r, ST_OVERFLOW);
        atomicOr(flags, ST_OVERFLOW);
    }
}

// w = A z and acc[p][0] += V0 . w over the ELL copy of the level-0 A: one row
// per thread (block b: rows row0 + (b % kTileSub) * kBThreads + [0, kBThreads)
// of tile b / kTileSub), the entries fetched before the launch wait
template <int R>
__global__ void __launch_bounds__(kBThreads)
k_bspmv_dot_ell(const BTile *__restrict__ tiles, DBCsr A, DEll E, const int *__restrict__ z, int *__restrict__ w,
                const int *__restrict__ v0, unsigned long long *acc, int m, unsigned *__restrict__ pflag,
                unsigned *__restrict__ flags) {
    pdl_trigger();
    __shared__ long long sh[kBThreads / 32][R];
    const BTile t = tiles[blockIdx.x / kTileSub];
    const int row = t.row0 + (blockIdx.x % kTileSub) * kBThreads + threadIdx.x;
    const bool ok = row < t.row1;
    int cc[kEllMax], vv[kEllMax];
#pragma unroll
    for (int k = 0; k < kEllMax; k++) {
        const bool in = ok && k < E.w;
        vv[k] = in ? __ldg(E.val + (size_t)k * E.n + row) : 0;
        cc[k] = in ? row + (int)__ldg(E.cd + (size_t)k * E.n + row) : 0;
    }
    pdl_wait();
    long long a[R], dot[R];
#pragma unroll
    for (int r = 0; r < R; r++) a[r] = dot[r] = 0;
    int xv[kEllMax][R];
#pragma unroll
    for (int k = 0; k < kEllMax; k++) {
        if (vv[k] != 0) load_r<R>(z, cc[k], xv[k]);
        else
#pragma unroll
            for (int r = 0; r < R; r++) xv[k][r] = 0;
    }
#pragma unroll
    for (int k = 0; k < kEllMax; k++)
#pragma unroll
        for (int r = 0; r < R; r++) a[r] = wadd(a[r], (long long)vv[k] * (long long)xv[k][r]);
    unsigned ovf = 0;
    if (ok) {
        const int bit = A.bit[row];
        int y[R], vq[R];
        load_r<R>(v0, row, vq);
#pragma unroll
        for (int r = 0; r < R; r++) {
            const long long s = a[r] >> bit;
            if (!fits32(s)) ovf |= 1u << r;
            y[r] = lo32(s);
            dot[r] = wadd(dot[r], (long long)vq[r] * y[r]);
        }
        store_r<R>(w, row, y);
    }
    bsum_i64<R>(dot, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) atomicAdd(acc + (size_t)(t.sys * R + r) * (m + 2), (unsigned long long)dot[r]);
    if (ovf) {
#pragma unroll
        for (int r = 0; r < R; r++)
            if (ovf & (1u << r)) atomicOr(pflag + (size_t)t.sys * R + r, ST_OVERFLOW);
        atomicOr(flags, ST_OVERFLOW);
    }
}

// MGS pass k of step j for every active pair: h = acc[k] >> bit, H[j][k] = h,
// w += (int)((-h) V_k >> bit), then acc[k+1] += V_{k+1} . w (or w . w).
template <int R, bool LAST>
__global__ void __launch_bounds__(kBThreads)
k_bmgs(const BTile *__restrict__ tiles, int k, int j, int m, size_t vstride, const int *__restrict__ V,
       int *__restrict__ w, const BPair *__restrict__ pairs, unsigned long long *acc, long long *H) {
    pdl_trigger();
    pdl_wait();
    __shared__ long long sh[kBThreads / 32][R];
    const BTile t = tiles[blockIdx.x];
    long long a[R];
    int bit[R];
    bool act[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = t.sys * R + r;
        act[r] = pairs[p].active != 0;
        bit[r] = pairs[p].bit;
        const long long h = ((long long)acc[(size_t)p * (m + 2) + k]) >> bit[r];
        if (t.first && threadIdx.x == 0 && act[r]) H[(size_t)p * (m + 1) * m + (size_t)j * (m + 1) + k] = h;
        a[r] = wsub(0, h);
    }
    const int *vk = V + (size_t)k * vstride;
    const int *vk1 = V + (size_t)(k + 1) * vstride;
    long long part[R];
#pragma unroll
    for (int r = 0; r < R; r++) part[r] = 0;
    for (int i = t.row0 + threadIdx.x; i < t.row1; i += kBThreads) {
        int wv[R], v[R], v1[R];
        load_rw<R>(w, i, wv);
        load_r<R>(vk, i, v);
        if (!LAST) load_r<R>(vk1, i, v1);
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (!act[r]) continue;
            wv[r] = (int)((unsigned)wv[r] + (unsigned)lo32(wmul(a[r], (long long)v[r]) >> bit[r]));
            part[r] = wadd(part[r], LAST ? (long long)wv[r] * wv[r] : (long long)v1[r] * wv[r]);
        }
        store_r<R>(w, i, wv);
    }
    bsum_i64<R>(part, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++)
            if (act[r])
                atomicAdd(acc + (size_t)(t.sys * R + r) * (m + 2) + (LAST ? m + 1 : k + 1),
                          (unsigned long long)part[r]);
}

__device__ long long bggen(long long a, long long b, long long *c, long long *s, int bit, unsigned *pf) {
    const long long r = lsqrt_dev(wadd(wmul(a, a), wmul(b, b)));
    long long inv_r = 0;
    if (r == 0) *pf |= ST_DIVZERO;
    else inv_r = ((1LL << 62) / r) >> (62 - bit - bit);
    *c = wmul(a, inv_r) >> bit;
    *s = wsub(0, wmul(b, inv_r)) >> bit;
    return r;
}

// per pair: H_{j+1,j} = lsqrt(w.w), its reciprocal, Givens, e update and the
// convergence test (gmres.hpp:240-262); converged pairs leave the cycle
__global__ void k_bgivens(int P, int j, int m, BPair *pairs, long long *Hall, long long *call, long long *sall,
                          long long *eall, unsigned long long *acc, unsigned *pflag, BInfo *info) {
    pdl_trigger();
    pdl_wait();
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P && pairs[p].active) {
        BPair &q = pairs[p];
        const int bit = q.bit;
        long long *Hj = Hall + (size_t)p * (m + 1) * m + (size_t)j * (m + 1);
        long long *c = call + (size_t)p * m, *s = sall + (size_t)p * m, *e = eall + (size_t)p * (m + 1);
        unsigned long long *ac = acc + (size_t)p * (m + 2);
        unsigned pf = 0;
        const long long nsq = (long long)ac[m + 1];
        if (nsq < 0) pf |= ST_NORM_OVF;
        Hj[j + 1] = lsqrt_dev(nsq);
        long long hinv = 0;
        if (Hj[j + 1] == 0) pf |= ST_DIVZERO;
        else hinv = ((1LL << 62) / Hj[j + 1]) >> (62 - bit - bit);
        q.hinv = hinv;
        for (int k = 0; k < j; k++) {
            const long long tt = Hj[k];
            Hj[k] = wsub(wmul(c[k], tt), wmul(s[k], Hj[k + 1])) >> bit;
            Hj[k + 1] = wadd(wmul(s[k], tt), wmul(c[k], Hj[k + 1])) >> bit;
        }
        Hj[j] = bggen(Hj[j], Hj[j + 1], &c[j], &s[j], bit, &pf);
        Hj[j + 1] = 0;
        e[j + 1] = wmul(s[j], e[j]) >> bit;
        e[j] = wmul(c[j], e[j]) >> bit;
        const double fact = (double)(1LL << bit);
        q.relres = fabs(__ddiv_rn(__dmul_rn(q.e0, (double)e[j + 1]), fact)) / q.nrm_b;
        const long long en = e[j + 1];
        const long long aen = en < 0 ? wsub(0, en) : en;
        q.jn = j + 1;
        for (int k = 0; k <= m + 1; k++) ac[k] = 0;
        // status raised while this pair was active: the V-cycle, SpMV and LU
        // of this step (pflag) or the scalars above (pf)
        const unsigned bad = pf | (pflag[p] & (ST_OVERFLOW | ST_DIVZERO | ST_NORM_OVF));
        if (bad) {
            q.bad = bad;
            q.active = 0;
        } else if (aen <= q.criteria) {
            q.conv = 1;
            q.active = 0;
        } else if (aen <= q.cycle_target) {
            // the F-bit basis has stopped gaining: end this pair's cycle; the
            // refinement restarts it from the true residual
            q.active = 0;
        } else if (j + 1 < m) {
            atomicAdd(&info->n_active, 1);
        }
    }
}

// V_{j+1} = (int)(hinv * w >> bit) for the pairs that took step j
template <int R>
__global__ void k_bscal(const BTile *__restrict__ tiles, int j, const BPair *__restrict__ pairs, int *__restrict__ w) {
    pdl_trigger();
    pdl_wait();
    const BTile t = tiles[blockIdx.x];
    long long a[R];
    int bit[R];
    bool act[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const BPair &q = pairs[t.sys * R + r];
        act[r] = q.jn == j + 1;
        a[r] = q.hinv;
        bit[r] = q.bit;
    }
    for (int i = t.row0 + threadIdx.x; i < t.row1; i += blockDim.x) {
        int wv[R];
        load_rw<R>(w, i, wv);
#pragma unroll
        for (int r = 0; r < R; r++)
            if (act[r]) wv[r] = lo32(wmul(a[r], (long long)wv[r]) >> bit[r]);
        store_r<R>(w, i, wv);
    }
}

// reads n 16-byte words through L2 (evicting what a timed operator would
// otherwise find there); the sum is kept only so that the loads stay
__global__ void k_l2_flush(const int4 *__restrict__ buf, size_t n, unsigned *__restrict__ sink) {
    unsigned acc = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int4 v = __ldcg(buf + i);
        acc ^= (unsigned)(v.x ^ v.y ^ v.z ^ v.w);
    }
    if (acc == 0x9E3779B9u) sink[0] = acc;
}

__global__ void k_binfo_reset(BInfo *info) {
    pdl_trigger();
    pdl_wait();
    info->n_active = 0;
}

// blas2::int32::Trsv per pair (blas2.hpp:366-376); skipped for discarded pairs
__global__ void k_btrsv(int P, int m, const BPair *__restrict__ pairs, const long long *Hall, const long long *eall,
                        double *yall) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const BPair &q = pairs[p];
    const int jn = q.jn;
    if (jn == 0 || q.bad) return;
    const long long *H = Hall + (size_t)p * (m + 1) * m;
    const long long *e = eall + (size_t)p * (m + 1);
    double *y = yall + (size_t)p * m;
    const double fact = (double)(1LL << q.bit);
    for (int i = jn - 1; i >= 0; i--) {
        double t = __ddiv_rn(__dmul_rn(q.e0, (double)e[i]), fact);
        for (int k = jn - 1; k > i; k--) t = __dsub_rn(t, __dmul_rn(__ddiv_rn((double)H[(size_t)k * (m + 1) + i], fact), y[k]));
        y[i] = __ddiv_rn(t, __ddiv_rn((double)H[(size_t)i * (m + 1) + i], fact));
    }
}

// x += y_k Z_k 2^-bit, k = 0..jn-1 in order (Axpy_D, blas1.hpp:252-258).  The
// power-of-two scale is applied to y_k first (exact, so (y_k 2^-bit) Z equals
// (y_k Z) 2^-bit) and each term is one fused multiply-add: GB300's FP64 rate
// is low, and separate operations made this kernel FP64-bound
template <int R>
__global__ void __launch_bounds__(kBThreads)
k_bxupd(const BTile *__restrict__ tiles, int m, size_t vstride, const BPair *__restrict__ pairs,
        const double *__restrict__ yall, const int *__restrict__ Z, double *__restrict__ x) {
    const BTile t = tiles[blockIdx.x / kTileSub];
    __shared__ double sy[R][64];
    __shared__ int sjn[R];
    if (threadIdx.x < R) {
        const BPair &q = pairs[t.sys * R + threadIdx.x];
        sjn[threadIdx.x] = q.jn > 0 && !q.bad ? q.jn : 0;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < R * m; idx += blockDim.x) {
        const int r = idx / m, k = idx % m;
        const BPair &q = pairs[t.sys * R + r];
        sy[r][k] = k < sjn[r] ? __dmul_rn(yall[(size_t)(t.sys * R + r) * m + k], 1.0 / (double)(1LL << q.bit)) : 0.0;
    }
    __syncthreads();
    const int i = t.row0 + (blockIdx.x % kTileSub) * kBThreads + threadIdx.x;
    if (i >= t.row1) return;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int jn = sjn[r];
        if (!jn) continue;
        double xi = x[(size_t)i * R + r];
        for (int k = 0; k < jn; k++) xi = fma(sy[r][k], (double)__ldg(Z + (size_t)k * vstride + (size_t)i * R + r), xi);
        x[(size_t)i * R + r] = xi;
    }
}

// r = b - A x per row (irsolver.hpp:32-33), every right-hand side: the row's
// products summed in index order with fused multiply-adds (GB300's FP64 rate
// is low; a separate multiply and add per entry made this kernel FP64-bound)
template <int R>
__global__ void k_bresid_f64(int n, const int *__restrict__ rptr, const int *__restrict__ cind,
                             const double *__restrict__ val, const double *__restrict__ x, const double *__restrict__ b,
                             double *__restrict__ rv) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    double acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0.0;
    const int e1 = rptr[row + 1];
    // the row in index order, eight entries' loads issued together
    for (int j0 = rptr[row]; j0 < e1; j0 += 8) {
        double a[8], xv[8][R];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int j = j0 + q;
            a[q] = j < e1 ? __ldg(val + j) : 0.0;
            const size_t c = j < e1 ? (size_t)__ldg(cind + j) * R : 0;
#pragma unroll
            for (int r = 0; r < R; r++) xv[q][r] = j < e1 ? __ldg(x + c + r) : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 8; q++)
            if (j0 + q < e1)
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] = fma(a[q], xv[q][r], acc[r]);
    }
#pragma unroll
    for (int r = 0; r < R; r++) rv[(size_t)row * R + r] = __dsub_rn(b[(size_t)row * R + r], acc[r]);
}

// per-tile sums of squares (fixed order), then per pair in tile order
template <int R>
__global__ void k_bnorm_part(const BTile *__restrict__ tiles, const double *__restrict__ v, double *__restrict__ part) {
    __shared__ double sh[kBThreads / 32][R];
    const BTile t = tiles[blockIdx.x];
    double s[R];
#pragma unroll
    for (int r = 0; r < R; r++) s[r] = 0;
    for (int i = t.row0 + threadIdx.x; i < t.row1; i += kBThreads)
#pragma unroll
        for (int r = 0; r < R; r++) {
            const double q = v[(size_t)i * R + r];
            s[r] += q * q;
        }
    bsum_f64<R>(s, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) part[(size_t)blockIdx.x * R + r] = s[r];
}

// one warp per pair: lanes take the system's tiles in turn, then a fixed
// shuffle tree (the same order every time)
__global__ void k_bnorm_fin(int S, int R, const int *__restrict__ tile_ptr, const double *__restrict__ part,
                            double *__restrict__ out) {
    const int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (p >= S * R) return;
    const int s = p / R, r = p % R;
    double acc = 0;
    for (int k = tile_ptr[s] + lane; k < tile_ptr[s + 1]; k += 32) acc += part[(size_t)k * R + r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) out[p] = sqrt(acc);
}

// ============================================================== host side

static DBCsr dview(const BatchCsr &M, int *&rp, int *&ci, int *&va, signed char *&bi, signed char *&db) {
    rp = dupload(M.rptr);
    ci = M.cind.empty() ? nullptr : dupload(M.cind);
    va = M.val.empty() ? nullptr : dupload(M.val);
    bi = M.bit.empty() ? nullptr : dupload(M.bit);
    db = M.dbit.empty() ? nullptr : dupload(M.dbit);
    return DBCsr{M.n, rp, ci, va, bi, db};
}

struct DevBMat {
    DBCsr d{};
    int group = 1;
    int *rp = nullptr, *ci = nullptr, *va = nullptr;
    signed char *bi = nullptr, *db = nullptr;
    short *cdv = nullptr;  // 16-bit column offsets (square operators whose offsets all fit)
    bool d16 = false;      // the lane kernels read cdv instead of ci (6 bytes an entry instead of 8)
    // ELL copy (square operators with at most kEllMax entries a row and at
    // most a quarter of the slots empty, 16-bit offsets): the kernels read it
    // instead of the CSR when ell is set
    DEll e{};
    short *ell_cd = nullptr;
    int *ell_va = nullptr;
    bool ell = false;
    void up(const BatchCsr &M, bool square = false) {
        d = dview(M, rp, ci, va, bi, db);
        const double avg = M.n ? (double)M.nnz() / M.n : 1.0;
        group = avg <= 32.0 ? 0 : pick_group(avg);  // 0: tile-staged stream
        if (!square || M.nnz() == 0) return;
        std::vector<short> cd(M.nnz());
        for (int i = 0; i < M.n; i++)
            for (int j = M.rptr[i]; j < M.rptr[i + 1]; j++) {
                const int off = M.cind[j] - i;
                if (off < -32768 || off > 32767) return;
                cd[j] = (short)off;
            }
        cdv = dupload(cd);
        d.cd = cdv;
        int w = 0;
        for (int i = 0; i < M.n; i++) w = std::max(w, M.rptr[i + 1] - M.rptr[i]);
        if (w == 0 || w > kEllMax || (double)M.nnz() < 0.75 * (double)M.n * w) return;
        std::vector<short> ecd((size_t)w * M.n, 0);
        std::vector<int> eva((size_t)w * M.n, 0);
        for (int i = 0; i < M.n; i++)
            for (int j = M.rptr[i], k = 0; j < M.rptr[i + 1]; j++, k++) {
                ecd[(size_t)k * M.n + i] = cd[j];
                eva[(size_t)k * M.n + i] = M.val[j];
            }
        ell_cd = dupload(ecd);
        ell_va = dupload(eva);
        e = DEll{M.n, w, ell_cd, ell_va};
    }
    void release() {
        dfree(rp); dfree(ci); dfree(va); dfree(bi); dfree(db); dfree(cdv); dfree(ell_cd); dfree(ell_va);
        rp = ci = va = nullptr;
        bi = db = nullptr;
        cdv = nullptr;
        ell_cd = nullptr;
        ell_va = nullptr;
    }
};

struct DevBLevel {
    int n_all = 0, n_smooth = 0;
    bool one_colour = false;  // LD is the diagonal alone (one colour): the sweep can be fused
    DevBMat A, LD, U, P, R;
    int *colour_rows = nullptr;
    std::vector<int> colour_ptr;
    int *row_sys = nullptr;       // system of each row of this level
    int *row_sys_next = nullptr;  // ... and of level l+1 (rows of R)
    // cluster sweep: groups of systems, each walking its own colours
    // (use_cluster 0: one launch per colour, 1: k_bsweep_cluster, 2: k_bsweep_packed)
    int use_cluster = 0, ngroups = 0;
    int *gc_ptr = nullptr, *cbound = nullptr, *grows = nullptr;
    int *sw_ptr = nullptr;          // packed form: items of (colour, CTA) run k * kClusterCtas + q
    int4 *pk_items = nullptr;
    int2 *pk_ents = nullptr;
    // use_cluster 3: k_bcolour_packed over LD packed in colour order (colour k: colour_ptr[k] ..)
    int4 *cp_items = nullptr;
    int2 *cp_ents = nullptr;
};

struct BatchEngine::Impl {
    Ctx &c;
    int S, Rn, Dmax, smooth_iter, m = 0;
    std::shared_ptr<BatchHierarchy> h;
    std::vector<DevBLevel> lv;
    std::vector<int> n_level;
    bool fuse_jac = true;  // one-colour levels' sweeps fused into the neighbouring SpMVs
    std::vector<int *> ee, xx, rr, tmp;  // per level (ee/xx index l = 0 unused)
    std::vector<int *> row_sys;          // per level 0 .. Dmax
    BLuDesc *d_lu = nullptr;
    int nlu = 0;
    size_t lu_smem = 0;
    size_t lu_csmem = 0;   // the cluster form's shared memory
    int lu_cluster = 0;    // 1: coarse LU through k_blu_cluster
    int *Lcat = nullptr, *Ucat = nullptr, *dcat = nullptr;
    DevCsr Af;
    std::vector<BTile> tiles_h;
    BTile *tiles = nullptr;
    BTile *stiles = nullptr;  // tiles of at most kStreamThreads rows (stream SpMV + dot)
    int nstiles = 0;
    int *tile_ptr = nullptr;
    int ntiles = 0;
    unsigned *pflag = nullptr;       // per pair: status raised outside the preconditioner (fatal for a cycle)
    unsigned *pflag_prec = nullptr;  // per pair: int32 wraps inside the V-cycle (reported)
    unsigned *cur_pflag = nullptr;   // the array the launches of the moment report into
    // Krylov state (allocated for the largest m used)
    int *V = nullptr, *Z = nullptr;
    long long *H = nullptr, *cs = nullptr, *sn = nullptr, *e = nullptr;
    double *y = nullptr, *rvec = nullptr, *nrm = nullptr, *npart = nullptr, *e0 = nullptr;
    unsigned long long *acc = nullptr;
    BPair *pairs = nullptr;
    BInfo *info_d = nullptr, *info_h = nullptr;
    std::vector<cudaGraphExec_t> graphs;
    CycleGraph cyc;         // a whole restart cycle, steps gated on the device
    bool graph_pdl = true;  // the PDL setting the graphs were captured with
    // the Arnoldi step's A Z_j fused with its first dot (tuned apart from the
    // V-cycle's A: its tiles and reductions favour other lanes per row)
    int dot_group = -1;  // -1: the level-0 A's lanes per row
    bool dot_d16 = false;
    bool dot_ell = false;  // the Arnoldi SpMV + dot over the level-0 A's ELL copy
    // persistent coarse tail (k_btail): levels tail_from .. Dmax-1 and the LU in
    // one cooperative launch (0: off)
    int tail_from = 0;
    TailStep *d_steps = nullptr;
    int nsteps = 0;
    unsigned *tail_bar = nullptr;  // grid barrier: arrivals (reset before each launch)
    int tail_grid = 0;             // CTAs of the tail (at most one per SM)
    // the stand-alone V-cycle (precondition) replayed from a graph captured for one in/out pair
    cudaGraphExec_t vc_graph = nullptr;
    const int *vc_in = nullptr;
    int *vc_out = nullptr;
    long long vc_launches = 0;
    std::vector<long long> graph_launches;
    size_t N0 = 0;  // level-0 rows
    // cold timing: a buffer three times the L2 read before every timed call
    int4 *flush_buf = nullptr;
    size_t flush_n = 0;
    unsigned *flush_sink = nullptr;

    Impl(Ctx &ctx, std::shared_ptr<BatchHierarchy> hh, int nrhs) : c(ctx), h(hh) {
        S = h->S;
        Rn = nrhs;
        Dmax = h->Dmax;
        smooth_iter = h->hi.empty() ? 1 : h->hi[0]->smooth_iter;
        n_level = h->n_level;
        N0 = (size_t)n_level[0];
        lv.resize(Dmax);
        for (int l = 0; l < Dmax; l++) {
            const BatchLevel &L = h->lv[l];
            DevBLevel &d = lv[l];
            d.n_all = L.n_all;
            d.n_smooth = L.n_smooth;
            d.A.up(L.A, true);
            d.LD.up(L.LD);
            d.U.up(L.U, true);
            d.P.up(L.P);
            d.R.up(L.R);
            // the colour pass reads a row's LD entries minus the diagonal (no stream form)
            d.LD.group = pick_group(L.LD.n ? (double)(L.LD.nnz() - L.LD.n) / L.LD.n : 1.0);
            d.colour_rows = L.colour_rows.empty() ? nullptr : dupload(L.colour_rows);
            d.colour_ptr = L.colour_ptr;
            // one colour: every LD row holds its diagonal alone, so row i's
            // entry is entry i (what the fused sweep step reads)
            d.one_colour = L.LD.n > 0 && L.LD.nnz() == L.LD.n;
            for (int i = 0; d.one_colour && i < L.LD.n; i++)
                d.one_colour = L.LD.rptr[i] == i && L.LD.cind[i] == i;
        }
        for (int l = 0; l < Dmax; l++) build_cluster_groups(l);
        for (int l = 0; l < Dmax; l++) build_colour_pack(l);
        for (int l = 0; l <= Dmax; l++) row_sys.push_back(dupload(h->row_sys[l]));
        for (int l = 0; l < Dmax; l++) {
            lv[l].row_sys = row_sys[l];
            lv[l].row_sys_next = row_sys[l + 1];
        }
        auto vec = [&](int rows) { return (int *)dmalloc(sizeof(int) * (size_t)std::max(rows, 1) * Rn); };
        ee.assign(Dmax + 1, nullptr);
        xx.assign(Dmax + 1, nullptr);
        rr.assign(Dmax, nullptr);
        tmp.assign(Dmax, nullptr);
        for (int l = 1; l <= Dmax; l++) {
            ee[l] = vec(n_level[l]);
            xx[l] = vec(n_level[l]);
        }
        for (int l = 0; l < Dmax; l++) {
            rr[l] = vec(n_level[l]);
            tmp[l] = vec(n_level[l]);
        }
        // coarsest LU factors of every system, concatenated
        std::vector<BLuDesc> desc;
        std::vector<int> Lh, Uh, dh;
        size_t maxn = 0;
        for (const BatchLU &lu : h->lu) {
            BLuDesc d{};
            d.n = lu.n;
            d.sys = lu.sys;
            d.bitL = lu.bitL;
            d.bitU = lu.bitU;
            d.dbitU = lu.dbitU;
            d.mat_off = (long long)Lh.size();
            d.d_off = (long long)dh.size();
            d.in = ee[lu.level] + (size_t)lu.offset * Rn;
            d.out = xx[lu.level] + (size_t)lu.offset * Rn;
            Lh.insert(Lh.end(), lu.L.begin(), lu.L.end());
            Uh.insert(Uh.end(), lu.U.begin(), lu.U.end());
            dh.insert(dh.end(), lu.dinv.begin(), lu.dinv.end());
            maxn = std::max(maxn, (size_t)lu.n);
            desc.push_back(d);
        }
        nlu = (int)desc.size();
        lu_smem = (sizeof(long long) + sizeof(int)) * maxn * Rn;
        if (lu_smem > 227 * 1024) throw CudaError{"a coarsest level is too large for the batched LU kernel"};
        {
            const size_t np = (maxn + 31) / 32, own = (np + kLuCtas - 1) / kLuCtas;
            lu_csmem = ((sizeof(int) * maxn * Rn + 15) & ~(size_t)15) + sizeof(long long) * own * 32 * Rn;
        }
        // one cluster per system: worth it when the systems leave SMs idle
        lu_cluster = nlu > 0 && nlu * kLuCtas <= c.num_sms;
        Lcat = dupload(Lh);
        Ucat = dupload(Uh);
        dcat = dupload(dh);
        d_lu = dupload(desc);
        Af = upload_csr_f64(h->Af);
        // tiles over the level-0 rows, never straddling two systems
        std::vector<int> tp(1, 0);
        for (int s = 0; s < S; s++) {
            const int off = h->offset[0][s], n = h->n_sys[s];
            for (int r0 = 0; r0 < n; r0 += kTileRows)
                tiles_h.push_back(BTile{s, off + r0, off + std::min(n, r0 + kTileRows), r0 == 0});
            tp.push_back((int)tiles_h.size());
        }
        ntiles = (int)tiles_h.size();
        tiles = dupload(tiles_h);
        std::vector<BTile> st;
        for (int s = 0; s < S; s++) {
            const int off = h->offset[0][s], n = h->n_sys[s];
            for (int r0 = 0; r0 < n; r0 += kStreamThreads)
                st.push_back(BTile{s, off + r0, off + std::min(n, r0 + kStreamThreads), r0 == 0});
        }
        nstiles = (int)st.size();
        stiles = dupload(st);
        tile_ptr = dupload(tp);
        pflag = (unsigned *)dmalloc(sizeof(unsigned) * (size_t)S * Rn * 2);
        SAGB_CUDA(cudaMemset(pflag, 0, sizeof(unsigned) * (size_t)S * Rn * 2));
        pflag_prec = pflag + (size_t)S * Rn;
        cur_pflag = pflag;
        rvec = (double *)dmalloc(sizeof(double) * N0 * Rn);
        nrm = (double *)dmalloc(sizeof(double) * (size_t)S * Rn);
        e0 = (double *)dmalloc(sizeof(double) * (size_t)S * Rn);
        npart = (double *)dmalloc(sizeof(double) * (size_t)ntiles * Rn);
        pairs = (BPair *)dmalloc(sizeof(BPair) * (size_t)S * Rn);
        SAGB_CUDA(cudaMemset(pairs, 0, sizeof(BPair) * (size_t)S * Rn));
        info_d = (BInfo *)dmalloc(sizeof(BInfo));
        SAGB_CUDA(cudaMallocHost(&info_h, sizeof(BInfo)));
        static bool attr = false;
        if (!attr) {
            SAGB_CUDA(cudaFuncSetAttribute(k_blu<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
            SAGB_CUDA(cudaFuncSetAttribute(k_blu<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
            SAGB_CUDA(cudaFuncSetAttribute(k_blu<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
            SAGB_CUDA(cudaFuncSetAttribute(k_blu_cluster<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
            SAGB_CUDA(cudaFuncSetAttribute(k_blu_cluster<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
            SAGB_CUDA(cudaFuncSetAttribute(k_blu_cluster<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
            SAGB_CUDA(cudaFuncSetAttribute(k_btail<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem));
            SAGB_CUDA(cudaFuncSetAttribute(k_btail<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem));
            SAGB_CUDA(cudaFuncSetAttribute(k_btail<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTailSmem));
            attr = true;
        }
    }

    // Groups of the systems that smooth at level l, balanced by LD entries, one
    // cluster each; rows of a group listed colour by colour.  The cluster sweep
    // is the default where colours are small (many colours per row count).
    void build_cluster_groups(int l) {
        const BatchLevel &L = h->lv[l];
        DevBLevel &d = lv[l];
        std::vector<int> sys;
        for (int s = 0; s < S; s++)
            if (h->depth[s] > l) sys.push_back(s);
        if (sys.empty()) return;
        std::vector<long long> work(sys.size());
        for (size_t k = 0; k < sys.size(); k++) work[k] = h->hi[sys[k]]->LD[l].nnz();
        std::vector<size_t> idx(sys.size());
        for (size_t k = 0; k < idx.size(); k++) idx[k] = k;
        std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return work[a] > work[b]; });
        const int G = std::max(1, std::min((int)sys.size(), 2 * c.num_sms / kClusterCtas));
        std::vector<long long> load(G, 0);
        std::vector<std::vector<int>> members(G);
        for (size_t k : idx) {
            const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
            load[g] += work[k];
            members[g].push_back(sys[k]);
        }
        std::vector<int> gc(1, 0), cb, rows;
        for (int g = 0; g < G; g++) {
            std::sort(members[g].begin(), members[g].end());
            int nc = 0;
            for (int s : members[g])
                for (int cc : h->hi[s]->colour[l]) nc = std::max(nc, cc + 1);
            for (int k = 0; k < nc; k++) {
                cb.push_back((int)rows.size());
                for (int s : members[g]) {
                    const std::vector<int> &col = h->hi[s]->colour[l];
                    const int off = h->offset[l][s];
                    for (int i = 0; i < (int)col.size(); i++)
                        if (col[i] == k) rows.push_back(off + i);
                }
            }
            cb.push_back((int)rows.size());
            gc.push_back((int)cb.size());
        }
        // gc[g]..gc[g+1]-1 index cb; colours of group g = gc[g+1] - gc[g] - 1
        d.ngroups = G;
        d.gc_ptr = dupload(gc);
        d.cbound = dupload(cb);
        d.grows = dupload(rows);
        const int ncol = (int)L.colour_ptr.size() - 1;
        d.use_cluster = ncol > 0 && (double)L.n_smooth / ncol < 16384.0;
        if (ncol > 0 && (double)L.n_smooth / ncol < 65536.0) build_packed(l, gc, cb, rows);
    }

    // LD packed in the colour row order for k_bcolour_packed (up to 2^30 entries
    // of LD, 8 GB; left out, like the cluster pack, when a row does not fit the
    // item format)
    static bool pack_rows(const BatchCsr &LD, const int *rows, size_t nrows, std::vector<int4> &items,
                          std::vector<int2> &ents) {
        for (size_t k = 0; k < nrows; k++) {
            const int row = rows[k];
            const int e0 = LD.rptr[row], dp = LD.rptr[row + 1] - 1;
            const int len = dp - e0, bit = LD.bit[row], dbit = LD.dbit[row];
            if (len < 0 || len >= (1 << 20) || bit < 0 || bit > 63 || dbit < 0 || dbit > 63 ||
                ents.size() + (size_t)len >= (size_t)1 << 31)
                return false;
            const unsigned meta = (unsigned)len | (unsigned)bit << 20 | (unsigned)dbit << 26;
            items.push_back(make_int4(row, (int)ents.size(), LD.val[dp], (int)meta));
            for (int e = e0; e < dp; e++) ents.push_back(make_int2(LD.cind[e], LD.val[e]));
        }
        return true;
    }

    void build_colour_pack(int l) {
        const BatchLevel &L = h->lv[l];
        DevBLevel &d = lv[l];
        if (L.colour_rows.empty() || L.LD.nnz() > (int64_t(1) << 30)) return;
        std::vector<int4> items;
        std::vector<int2> ents;
        items.reserve(L.colour_rows.size());
        if (!pack_rows(L.LD, L.colour_rows.data(), L.colour_rows.size(), items, ents)) return;
        d.cp_items = dupload(items);
        d.cp_ents = ents.empty() ? (int2 *)dmalloc(sizeof(int2)) : dupload(ents);
    }

    // the packed copy of LD read by k_bsweep_packed (rows of each colour dealt
    // to the cluster's CTAs in turn); left out when a row does not fit the
    // item format, and the level then keeps the other two forms
    void build_packed(int l, const std::vector<int> &gc, const std::vector<int> &cb, const std::vector<int> &rows) {
        const BatchCsr &LD = h->lv[l].LD;
        DevBLevel &d = lv[l];
        const size_t K = cb.size();
        std::vector<char> is_end(K, 0);  // cb entries that close a group (no rows of their own)
        for (size_t g = 0; g + 1 < gc.size(); g++) is_end[gc[g + 1] - 1] = 1;
        std::vector<int> sw(K * kClusterCtas + 1, 0);
        std::vector<int4> items;
        std::vector<int2> ents;
        items.reserve(rows.size());
        for (size_t kk = 0; kk < K; kk++)
            for (int q = 0; q < kClusterCtas; q++) {
                sw[kk * kClusterCtas + q] = (int)items.size();
                if (is_end[kk]) continue;
                for (int i = cb[kk] + q; i < cb[kk + 1]; i += kClusterCtas)
                    if (!pack_rows(LD, &rows[i], 1, items, ents)) return;
            }
        sw[K * kClusterCtas] = (int)items.size();
        if (items.empty()) return;
        d.sw_ptr = dupload(sw);
        d.pk_items = dupload(items);
        d.pk_ents = ents.empty() ? (int2 *)dmalloc(sizeof(int2)) : dupload(ents);
        if (d.use_cluster) d.use_cluster = 2;
    }

    void free_krylov() {
        dfree(V); dfree(Z); dfree(H); dfree(cs); dfree(sn); dfree(e); dfree(y); dfree(acc);
        V = Z = nullptr;
        H = cs = sn = e = nullptr;
        y = nullptr;
        acc = nullptr;
        clear_graphs();
    }

    void clear_graphs() {
        cyc.clear();
        for (auto g : graphs)
            if (g) cudaGraphExecDestroy(g);
        graphs.clear();
        graph_launches.clear();
        if (vc_graph) cudaGraphExecDestroy(vc_graph);
        vc_graph = nullptr;
    }

    // Milliseconds per call of fn the way the solver runs it: max(reps, 5)
    // calls captured in one CUDA graph (launch gaps and programmatic overlap
    // as in the Arnoldi-step graphs), the fastest of three launches after a
    // warm-up launch; or reps calls on the stream after one warm-up call when
    // graphs are off.
    template <typename F>
    float timed(F &&fn, int reps, cudaEvent_t e0, cudaEvent_t e1) {
        const long long before = c.launches;
        float ms = 0;
        int n = reps;
        if (c.use_graphs) {
            n = std::max(reps, 5);
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge;
            SAGB_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            try {
                for (int k = 0; k < n; k++) fn();
            } catch (...) {
                cudaStreamEndCapture(c.stream, &g);
                if (g) cudaGraphDestroy(g);
                c.launches = before;
                throw;
            }
            SAGB_CUDA(cudaStreamEndCapture(c.stream, &g));
            SAGB_CUDA(cudaGraphInstantiate(&ge, g, 0));
            cudaGraphDestroy(g);
            SAGB_CUDA(cudaGraphLaunch(ge, c.stream));
            ms = 1e30f;
            for (int t = 0; t < 3; t++) {  // the fastest of three launches
                float one = 0;
                SAGB_CUDA(cudaEventRecord(e0, c.stream));
                SAGB_CUDA(cudaGraphLaunch(ge, c.stream));
                SAGB_CUDA(cudaEventRecord(e1, c.stream));
                SAGB_CUDA(cudaEventSynchronize(e1));
                SAGB_CUDA(cudaEventElapsedTime(&one, e0, e1));
                ms = std::min(ms, one);
            }
            cudaGraphExecDestroy(ge);
        } else {
            fn();
            SAGB_CUDA(cudaEventRecord(e0, c.stream));
            for (int k = 0; k < n; k++) fn();
            SAGB_CUDA(cudaEventRecord(e1, c.stream));
            SAGB_CUDA(cudaEventSynchronize(e1));
            SAGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        }
        c.launches = before;
        return ms / n;
    }

    void ensure_flush_buf() {  // outside any stream capture
        if (flush_buf) return;
        int l2 = 0;
        SAGB_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c.device));
        flush_n = 3 * (size_t)std::max(l2, 1 << 20) / sizeof(int4);
        flush_buf = (int4 *)dmalloc(flush_n * sizeof(int4));
        flush_sink = (unsigned *)dmalloc(sizeof(unsigned));
        SAGB_CUDA(cudaMemset(flush_buf, 0, flush_n * sizeof(int4)));
    }
    void l2_flush() {
        k_l2_flush<<<c.num_sms * 4, 512, 0, c.stream>>>(flush_buf, flush_n, flush_sink);
    }

    // milliseconds per call with the L2 flushed before every call: the time of
    // flush + call, less the flush's own (a call then reads its operator from
    // HBM, as in the solver's V-cycle, which streams ~1 GB between two uses)
    template <typename F>
    float timed_cold(F &&fn, int reps, cudaEvent_t e0, cudaEvent_t e1) {
        ensure_flush_buf();
        const float both = timed([&] {
            l2_flush();
            fn();
        }, reps, e0, e1);
        const float alone = timed([&] { l2_flush(); }, reps, e0, e1);
        return std::max(both - alone, 0.0f);
    }

    // precondition(): the V-cycle from a captured graph (re-captured when the
    // vectors, the launch shapes or the PDL setting change)
    void vcycle_graph(const int *in, int *out) {
        if (!c.use_graphs) return vcycle(in, out);
        if (graph_pdl != c.use_pdl) {
            clear_graphs();
            graph_pdl = c.use_pdl;
        }
        if (vc_graph && (vc_in != in || vc_out != out)) {
            cudaGraphExecDestroy(vc_graph);
            vc_graph = nullptr;
        }
        if (!vc_graph) {
            cudaGraph_t g = nullptr;
            const long long before = c.launches;
            SAGB_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            try {
                vcycle(in, out);
            } catch (...) {
                cudaStreamEndCapture(c.stream, &g);
                if (g) cudaGraphDestroy(g);
                c.launches = before;
                throw;
            }
            SAGB_CUDA(cudaStreamEndCapture(c.stream, &g));
            SAGB_CUDA(cudaGraphInstantiate(&vc_graph, g, 0));
            cudaGraphDestroy(g);
            vc_launches = c.launches - before;
            c.launches = before;
            vc_in = in;
            vc_out = out;
        }
        SAGB_CUDA(cudaGraphLaunch(vc_graph, c.stream));
        c.launches += vc_launches;
    }

    ~Impl() {
        free_krylov();
        for (auto &d : lv) {
            d.A.release(); d.LD.release(); d.U.release(); d.P.release(); d.R.release();
            dfree(d.colour_rows);
            dfree(d.gc_ptr);
            dfree(d.cbound);
            dfree(d.grows);
            dfree(d.sw_ptr);
            dfree(d.pk_items);
            dfree(d.pk_ents);
            dfree(d.cp_items);
            dfree(d.cp_ents);
        }
        for (auto p : row_sys) dfree(p);
        for (auto p : ee) dfree(p);
        for (auto p : xx) dfree(p);
        for (auto p : rr) dfree(p);
        for (auto p : tmp) dfree(p);
        dfree(d_lu); dfree(Lcat); dfree(Ucat); dfree(dcat);
        dfree(d_steps); dfree(tail_bar);
        Af.release();
        dfree(tiles); dfree(stiles); dfree(tile_ptr); dfree(pflag); dfree(rvec); dfree(nrm); dfree(e0); dfree(npart);
        dfree(pairs); dfree(info_d);
        dfree(flush_buf); dfree(flush_sink);
        if (info_h) cudaFreeHost(info_h);
    }

    // ------------------------------------------------------- dispatch helpers
    template <typename F>
    void by_r(F &&f) {
        if (Rn == 4) f(std::integral_constant<int, 4>());
        else if (Rn == 2) f(std::integral_constant<int, 2>());
        else f(std::integral_constant<int, 1>());
    }
    template <typename F>
    static void by_g(int G, F &&f) {
        switch (G) {
            case 1: f(std::integral_constant<int, 1>()); break;
            case 2: f(std::integral_constant<int, 2>()); break;
            case 4: f(std::integral_constant<int, 4>()); break;
            case 8: f(std::integral_constant<int, 8>()); break;
            case 16: f(std::integral_constant<int, 16>()); break;
            default: f(std::integral_constant<int, 32>()); break;
        }
    }

    // one kernel of the V-cycle on the library stream: programmatic dependent
    // launch when enabled, a thread-block cluster when cluster > 1
    template <typename... KArgs, typename... Args>
    void launch(void (*k)(KArgs...), int grid, int block, size_t smem, int cluster, Args... args) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(block);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = c.stream;
        cudaLaunchAttribute at[2];
        int na = 0;
        if (c.use_pdl) {
            at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            at[na].val.programmaticStreamSerializationAllowed = 1;
            na++;
        }
        if (cluster > 1) {
            at[na].id = cudaLaunchAttributeClusterDimension;
            at[na].val.clusterDim.x = cluster;
            at[na].val.clusterDim.y = 1;
            at[na].val.clusterDim.z = 1;
            na++;
        }
        cfg.attrs = at;
        cfg.numAttrs = na;
        SAGB_CUDA(cudaLaunchKernelEx(&cfg, k, args...));
        c.launches++;
    }

    // jac: JAC_NONE, or JAC_PRE with mode SET / JAC_POST with mode RESID (the
    // one-colour smoother step in the epilogue, J its level's diagonal)
    void bspmv(const DevBMat &M, const int *x, int *y, int mode, const int *z, const int *row_sys,
               int jac = JAC_NONE, const BJac &J = BJac{}) {
        if (M.d.n == 0) return;
        if (M.ell && M.ell_va) {
            const int blocks = (M.d.n + kBThreads - 1) / kBThreads;
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                auto k = jac == JAC_PRE ? k_bspmv_ell<R, SPMV_SET, JAC_PRE>
                         : jac == JAC_POST ? k_bspmv_ell<R, SPMV_RESID, JAC_POST>
                         : mode == SPMV_SET ? k_bspmv_ell<R, SPMV_SET>
                         : mode == SPMV_RESID ? k_bspmv_ell<R, SPMV_RESID> : k_bspmv_ell<R, SPMV_ADD>;
                launch(k, blocks, kBThreads, 0, 1, M.d, M.e, x, y, z, row_sys, cur_pflag, c.d_flags, J);
            });
            return;
        }
        if (M.group == 0) {
            const int blocks = (M.d.n + kStreamThreads - 1) / kStreamThreads;
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                auto k = jac == JAC_PRE ? k_bspmv_stream<R, SPMV_SET, JAC_PRE>
                         : jac == JAC_POST ? k_bspmv_stream<R, SPMV_RESID, JAC_POST>
                         : mode == SPMV_SET ? k_bspmv_stream<R, SPMV_SET>
                         : mode == SPMV_RESID ? k_bspmv_stream<R, SPMV_RESID> : k_bspmv_stream<R, SPMV_ADD>;
                launch(k, blocks, kStreamThreads, 0, 1, M.d, x, y, z, row_sys, cur_pflag, c.d_flags, J);
            });
            return;
        }
        const long long threads = (long long)M.d.n * M.group;
        const int blocks = (int)((threads + kBThreads - 1) / kBThreads);
        const bool d16 = M.d16 && M.cdv;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            by_g(M.group, [&](auto GG) {
                constexpr int G = decltype(GG)::value;
                auto pick = [&](auto D) {
                    constexpr bool D16 = decltype(D)::value;
                    return jac == JAC_PRE ? k_bspmv<R, G, SPMV_SET, D16, JAC_PRE>
                           : jac == JAC_POST ? k_bspmv<R, G, SPMV_RESID, D16, JAC_POST>
                           : mode == SPMV_SET ? k_bspmv<R, G, SPMV_SET, D16>
                           : mode == SPMV_RESID ? k_bspmv<R, G, SPMV_RESID, D16> : k_bspmv<R, G, SPMV_ADD, D16>;
                };
                auto k = d16 ? pick(std::true_type()) : pick(std::false_type());
                launch(k, blocks, kBThreads, 0, 1, M.d, x, y, z, row_sys, cur_pflag, c.d_flags, J);
            });
        });
    }

    // the one-colour step of level l (LD is its diagonal: row i's entry is i)
    BJac jac_of(int l, int *x2 = nullptr) const {
        const DevBMat &LD = lv[l].LD;
        return BJac{LD.d.val, LD.d.bit, LD.d.dbit, LD.d.n, x2};
    }

    void sweep(int l, const int *in, int *out) {
        const DevBLevel &L = lv[l];
        if (L.use_cluster == 3 && L.cp_items) {
            const int nc = (int)L.colour_ptr.size() - 1;
            for (int k = 0; k < nc; k++) {
                const int a = L.colour_ptr[k], b = L.colour_ptr[k + 1];
                if (b == a) continue;
                const long long threads = (long long)(b - a) * L.LD.group;
                const int blocks = (int)((threads + kBThreads - 1) / kBThreads);
                by_r([&](auto RR) {
                    constexpr int R = decltype(RR)::value;
                    by_g(L.LD.group, [&](auto GG) {
                        constexpr int G = decltype(GG)::value;
                        launch(k_bcolour_packed<R, G>, blocks, kBThreads, 0, 1, a, b, (const int4 *)L.cp_items,
                               (const int2 *)L.cp_ents, in, out, (const int *)L.row_sys, cur_pflag, c.d_flags);
                    });
                });
            }
            return;
        }
        if (L.use_cluster == 2 && L.pk_items && L.ngroups > 0) {
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                by_g(L.LD.group, [&](auto GG) {
                    constexpr int G = decltype(GG)::value;
                    launch(k_bsweep_packed<R, G>, L.ngroups * kClusterCtas, pk_threads<R>(), 0, kClusterCtas,
                           (const int *)L.gc_ptr, (const int *)L.sw_ptr, (const int4 *)L.pk_items,
                           (const int2 *)L.pk_ents, in, out, (const int *)L.row_sys, cur_pflag, c.d_flags);
                });
            });
            return;
        }
        if (L.use_cluster && L.ngroups > 0) {
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                by_g(L.LD.group, [&](auto GG) {
                    constexpr int G = decltype(GG)::value;
                    launch(k_bsweep_cluster<R, G>, L.ngroups * kClusterCtas, kBThreads, 0, kClusterCtas,
                           (const int *)L.gc_ptr, (const int *)L.cbound, (const int *)L.grows, L.LD.d, in, out,
                           (const int *)L.row_sys, cur_pflag, c.d_flags);
                });
            });
            return;
        }
        const int nc = (int)L.colour_ptr.size() - 1;
        for (int k = 0; k < nc; k++) {
            const int a = L.colour_ptr[k], cnt = L.colour_ptr[k + 1] - a;
            if (cnt == 0) continue;
            const long long threads = (long long)cnt * L.LD.group;
            const int blocks = (int)((threads + kBThreads - 1) / kBThreads);
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                by_g(L.LD.group, [&](auto GG) {
                    constexpr int G = decltype(GG)::value;
                    launch(k_bcolour<R, G>, blocks, kBThreads, 0, 1, cnt, (const int *)(L.colour_rows + a), L.LD.d, in,
                           out, (const int *)L.row_sys, cur_pflag, c.d_flags);
                });
            });
        }
    }

    void smooth(int l, const int *in, int *out, bool inited) {
        int k0 = 0;
        if (!inited) {
            sweep(l, in, out);
            k0 = 1;
        }
        for (int k = k0; k < smooth_iter; k++) {
            bspmv(lv[l].U, out, tmp[l], SPMV_RESID, in, lv[l].row_sys);
            sweep(l, tmp[l], out);
        }
    }

    // LUflex::Solve of every system (one CTA each, or one cluster each)
    void lu(unsigned *pf) {
        if (!nlu) return;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            if (lu_cluster)
                launch(k_blu_cluster<R>, nlu * kLuCtas, kLuCThreads, lu_csmem, kLuCtas, (const BLuDesc *)d_lu,
                       (const int *)Lcat, (const int *)Ucat, (const int *)dcat, pf, c.d_flags);
            else
                launch(k_blu<R>, nlu, kBLuThreads, lu_smem, 1, (const BLuDesc *)d_lu, (const int *)Lcat,
                       (const int *)Ucat, (const int *)dcat, pf, c.d_flags);
        });
    }

    // the steps of levels t .. Dmax-1 and the LU, in the order vcycle_body runs
    // them; false when a level lacks the colour-ordered packed LD
    bool build_tail(int t, int grid = 0) {
        if (t < 1 || t >= Dmax || lu_smem > (size_t)kTailSmem) return false;
        for (int l = t; l < Dmax; l++)
            if (!lv[l].cp_items) return false;
        std::vector<TailStep> st;
        auto colours = [&](int l, const int *in, int *out) {
            const DevBLevel &L = lv[l];
            for (size_t k = 0; k + 1 < L.colour_ptr.size(); k++) {
                if (L.colour_ptr[k + 1] == L.colour_ptr[k]) continue;
                TailStep q{};
                q.kind = TK_COLOUR;
                q.G = std::max(1, L.LD.group);
                q.ib = L.colour_ptr[k];
                q.ie = L.colour_ptr[k + 1];
                q.items = L.cp_items;
                q.ents = L.cp_ents;
                q.z = in;
                q.y = out;
                q.row_sys = L.row_sys;
                st.push_back(q);
            }
        };
        auto spmv = [&](const DevBMat &M, const int *x, int *y, int kind, const int *z, const int *row_sys) {
            if (M.d.n == 0) return;
            TailStep q{};
            q.kind = kind;
            q.G = std::max(1, M.group);
            q.M = M.d;
            q.x = x;
            q.y = y;
            q.z = z;
            q.row_sys = row_sys;
            st.push_back(q);
        };
        for (int l = t; l < Dmax; l++) {
            colours(l, ee[l], xx[l]);
            for (int k = 1; k < smooth_iter; k++) {
                spmv(lv[l].U, xx[l], tmp[l], TK_RESID, ee[l], lv[l].row_sys);
                colours(l, tmp[l], xx[l]);
            }
            spmv(lv[l].A, xx[l], rr[l], TK_RESID, ee[l], lv[l].row_sys);
            spmv(lv[l].R, rr[l], ee[l + 1], TK_SET, nullptr, lv[l].row_sys_next);
        }
        if (nlu) {
            TailStep q{};
            q.kind = TK_LU;
            st.push_back(q);
        }
        for (int l = Dmax - 1; l >= t; l--) {
            spmv(lv[l].P, xx[l + 1], xx[l], TK_ADD, nullptr, lv[l].row_sys);
            for (int k = 0; k < smooth_iter; k++) {
                spmv(lv[l].U, xx[l], tmp[l], TK_RESID, ee[l], lv[l].row_sys);
                colours(l, tmp[l], xx[l]);
            }
        }
        int per_sm = 0;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            SAGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_btail<R>, kTailThreads, lu_smem));
        });
        if (per_sm < 1) return false;
        dfree(d_steps);
        d_steps = dupload(st);
        nsteps = (int)st.size();
        // at most one CTA per SM, all resident (cooperative launch); fewer CTAs
        // make the barrier cheaper where the coarse levels have little work
        tail_grid = grid > 0 ? std::min(grid, c.num_sms) : c.num_sms;
        if (!tail_bar) tail_bar = (unsigned *)dmalloc(sizeof(unsigned) * 2);
        tail_from = t;
        clear_graphs();
        return true;
    }

    void drop_tail() {
        tail_from = 0;
        clear_graphs();
    }

    void launch_tail(unsigned extra = 0, unsigned long long limit_ns = kSpinLimitNs) {
        SAGB_CUDA(cudaMemsetAsync(tail_bar, 0, sizeof(unsigned) * 2, c.stream));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(tail_grid);
        cfg.blockDim = dim3(kTailThreads);
        cfg.dynamicSmemBytes = lu_smem;
        cfg.stream = c.stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            SAGB_CUDA(cudaLaunchKernelEx(&cfg, k_btail<R>, (const TailStep *)d_steps, nsteps, (const BLuDesc *)d_lu,
                                         nlu, (const int *)Lcat, (const int *)Ucat, (const int *)dcat, tail_bar,
                                         cur_pflag, c.d_flags, c.d_flags_main, extra, limit_ns));
        });
        c.launches++;
    }

    // intAMGflex::Precondition (INTAMG.hpp:269-293) for the whole batch; int32
    // wraps inside it go to the preconditioner's status arrays (FGMRES is
    // flexible, so they cost convergence speed, not correctness)
    void vcycle(const int *in, int *out) {
        PrecFlags guard(c);
        cur_pflag = pflag_prec;
        vcycle_body(in, out);
        cur_pflag = pflag;
    }

    // a level whose sweeps are fused into its neighbours' SpMVs (one colour,
    // one smoothing step, outside the persistent tail): its pre-smoothing
    // sweep in the restriction that produces its e, its post-smoothing sweep
    // in its U residual, whose result (in tmp) the interpolation above reads
    bool fused_pre(int l, int t) const { return fuse_jac && smooth_iter == 1 && l >= 1 && l < t && lv[l].one_colour; }
    bool fused_post(int l, int t) const { return fused_pre(l, t) && lv[l].n_all == lv[l].n_smooth; }

    void vcycle_body(const int *in, int *out) {
        const int t = tail_from > 0 && d_steps ? tail_from : Dmax;
        for (int l = 0; l < t; l++) {
            const int *e_l = l == 0 ? in : ee[l];
            int *x_l = l == 0 ? out : xx[l];
            if (!fused_pre(l, t)) smooth(l, e_l, x_l, false);
            bspmv(lv[l].A, x_l, rr[l], SPMV_RESID, e_l, lv[l].row_sys);
            if (fused_pre(l + 1, t))
                bspmv(lv[l].R, rr[l], ee[l + 1], SPMV_SET, nullptr, lv[l].row_sys_next, JAC_PRE,
                      jac_of(l + 1, xx[l + 1]));
            else
                bspmv(lv[l].R, rr[l], ee[l + 1], SPMV_SET, nullptr, lv[l].row_sys_next);
        }
        if (t < Dmax) launch_tail();
        else lu(cur_pflag);
        for (int l = t - 1; l >= 0; l--) {
            const int *e_l = l == 0 ? in : ee[l];
            int *x_l = l == 0 ? out : xx[l];
            bspmv(lv[l].P, fused_post(l + 1, t) ? tmp[l + 1] : xx[l + 1], x_l, SPMV_ADD, nullptr, lv[l].row_sys);
            if (fused_post(l, t))
                bspmv(lv[l].U, x_l, tmp[l], SPMV_RESID, e_l, lv[l].row_sys, JAC_POST, jac_of(l));
            else
                smooth(l, e_l, x_l, true);
        }
    }

    // ----------------------------------------------------------- Krylov
    void ensure_krylov(int mm) {
        if (mm == m && V) return;
        free_krylov();
        m = mm;
        const size_t P = (size_t)S * Rn;
        V = (int *)dmalloc(sizeof(int) * N0 * Rn * (m + 1));
        Z = (int *)dmalloc(sizeof(int) * N0 * Rn * (m + 1));
        H = (long long *)dmalloc(sizeof(long long) * P * (m + 1) * m);
        cs = (long long *)dmalloc(sizeof(long long) * P * m);
        sn = (long long *)dmalloc(sizeof(long long) * P * m);
        e = (long long *)dmalloc(sizeof(long long) * P * (m + 1));
        y = (double *)dmalloc(sizeof(double) * P * m);
        acc = (unsigned long long *)dmalloc(sizeof(unsigned long long) * P * (m + 2));
        SAGB_CUDA(cudaMemset(H, 0, sizeof(long long) * P * (m + 1) * m));
        SAGB_CUDA(cudaMemset(V, 0, sizeof(int) * N0 * Rn * (m + 1)));
        SAGB_CUDA(cudaMemset(Z, 0, sizeof(int) * N0 * Rn * (m + 1)));
    }

    void pair_norms(const double *v) {
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            k_bnorm_part<R><<<ntiles, kBThreads, 0, c.stream>>>(tiles, v, npart);
        });
        const int P = S * Rn;
        k_bnorm_fin<<<(P + 7) / 8, 256, 0, c.stream>>>(S, Rn, tile_ptr, npart, nrm);
        c.launches += 2;
    }

    // w = A z with the first Gram-Schmidt dot (v0 . w) per pair into acc
    void spmv_dot(const int *z, int *w, const int *v0, unsigned long long *accp, int mm) {
        const DevBMat &A0 = lv[0].A;
        const int g = dot_group >= 0 ? dot_group : A0.group;
        const bool d16 = dot_d16 && A0.cdv && g > 0;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            if (dot_ell && A0.ell_va) {
                launch(k_bspmv_dot_ell<R>, ntiles * kTileSub, kBThreads, 0, 1, (const BTile *)tiles, A0.d, A0.e, z, w,
                       v0, accp, mm, pflag, c.d_flags);
            } else if (g == 0) {
                launch(k_bspmv_dot_stream<R>, nstiles, kStreamThreads, 0, 1, (const BTile *)stiles, A0.d, z, w, v0,
                       accp, mm, pflag, c.d_flags);
            } else {
                by_g(g, [&](auto GG) {
                    constexpr int G = decltype(GG)::value;
                    launch(d16 ? k_bspmv_dot<R, G, true> : k_bspmv_dot<R, G, false>, ntiles, kBThreads, 0, 1,
                           (const BTile *)tiles, A0.d, z, w, v0, (const BPair *)pairs, accp, mm, pflag, c.d_flags);
                });
            }
        });
    }

    // d2h: read the step status back (per-step mode); has_next: end with the
    // kernel that opens step j+1 of the cycle graph when a pair is still active
    void arnoldi_step(int j, bool d2h = true, cudaGraphConditionalHandle next = 0, bool has_next = false) {
        const int P = S * Rn;
        const size_t vs = N0 * Rn;
        int *Vj = V + (size_t)j * vs, *Zj = Z + (size_t)j * vs, *w = V + (size_t)(j + 1) * vs;
        // the Arnoldi kernels wait for their predecessor at their first
        // instruction: programmatic launch only hides the launch latency
        launch(k_binfo_reset, 1, 1, 0, 1, info_d);
        vcycle(Vj, Zj);
        spmv_dot(Zj, w, V, acc, m);
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            for (int k = 0; k <= j; k++) {
                if (k < j)
                    launch(k_bmgs<R, false>, ntiles, kBThreads, 0, 1, (const BTile *)tiles, k, j, m, vs,
                           (const int *)V, w, (const BPair *)pairs, acc, H);
                else
                    launch(k_bmgs<R, true>, ntiles, kBThreads, 0, 1, (const BTile *)tiles, k, j, m, vs,
                           (const int *)V, w, (const BPair *)pairs, acc, H);
            }
        });
        launch(k_bgivens, (P + 127) / 128, 128, 0, 1, P, j, m, pairs, H, cs, sn, e, acc, pflag, info_d);
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            launch(k_bscal<R>, ntiles, kBThreads, 0, 1, (const BTile *)tiles, j, (const BPair *)pairs, w);
        });
        if (has_next) launch(k_cycle_next, 1, 32, 0, 1, (const int *)&info_d->n_active, next);
        if (d2h) SAGB_CUDA(cudaMemcpyAsync(info_h, info_d, sizeof(BInfo), cudaMemcpyDeviceToHost, c.stream));
    }

    // the Arnoldi steps of one restart cycle: one graph launch whose steps
    // after the first run only while a pair is active (no host round trip),
    // or step by step with a status read after each; returns true when the
    // cycle graph ran (its launches are counted once the pairs are read back)
    bool cycle_steps() {
        if (c.use_graphs && c.cycle_graph && !cyc.refused) {
            if (graph_pdl != c.use_pdl) {
                clear_graphs();
                graph_pdl = c.use_pdl;
            }
            if (!cyc.exec || cyc.m != m)
                build_cycle_graph(c, m, cyc, [&](int j, cudaGraphConditionalHandle nx, bool has) {
                    arnoldi_step(j, false, nx, has);
                });
            if (cyc.exec) {
                SAGB_CUDA(cudaGraphLaunch(cyc.exec, c.stream));
                return true;
            }
        }
        for (int j = 0; j < m; j++) {
            step(j);
            if (info_h->n_active == 0) break;
        }
        return false;
    }

    void step(int j) {
        if (graph_pdl != c.use_pdl) {
            clear_graphs();
            graph_pdl = c.use_pdl;
        }
        if (!c.use_graphs) {
            arnoldi_step(j);
        } else {
            if ((int)graphs.size() <= j) {
                graphs.resize(j + 1, nullptr);
                graph_launches.resize(j + 1, 0);
            }
            if (!graphs[j]) {
                cudaGraph_t g = nullptr;
                const long long before = c.launches;
                SAGB_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
                try {
                    arnoldi_step(j);
                } catch (...) {
                    cudaStreamEndCapture(c.stream, &g);
                    throw;
                }
                SAGB_CUDA(cudaStreamEndCapture(c.stream, &g));
                SAGB_CUDA(cudaGraphInstantiate(&graphs[j], g, 0));
                cudaGraphDestroy(g);
                graph_launches[j] = c.launches - before;
                c.launches = before;
            }
            SAGB_CUDA(cudaGraphLaunch(graphs[j], c.stream));
            c.launches += graph_launches[j];
        }
        SAGB_CUDA(cudaStreamSynchronize(c.stream));
    }

    void residual(const double *b, const double *x) {
        const int n = (int)N0;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            k_bresid_f64<R><<<(n + 127) / 128, 128, 0, c.stream>>>(n, Af.rptr, Af.cind, (const double *)Af.val, x, b,
                                                                  rvec);
        });
        c.launches++;
        pair_norms(rvec);
    }

    // Restarted::Solve per pair (irsolver.hpp:27-43), all pairs in lockstep
    void solve(const KrylovParams &kp, const int *bits_sys, const double *b, const double *nrm_b, double *x,
               BatchStats &st) {
        const int P = S * Rn;
        ensure_krylov(kp.m);
        st = BatchStats();
        st.iters.assign(P, 0);
        st.converged.assign(P, 0);
        st.fallbacks.assign(P, 0);
        st.final_bit.assign(P, 0);
        st.explicit_res.assign(P, 0.0);
        std::vector<BPair> hp(P);
        std::vector<double> nb(P);
        SAGB_CUDA(cudaMemcpy(nb.data(), nrm_b, sizeof(double) * P, cudaMemcpyDefault));
        std::vector<int> bit(P), done(P, 0), discarded(P, 0);
        std::vector<double> prev(P, 0.0), hn(P);
        if (kp.m > 64) throw CudaError{"restart length above 64"};
        for (int p = 0; p < P; p++) bit[p] = bits_sys[p / Rn];
        SAGB_CUDA(cudaMemsetAsync(pflag, 0, sizeof(unsigned) * P * 2, c.stream));
        for (int outer = 0; outer < kp.max_outer; outer++) {
            residual(b, x);
            SAGB_CUDA(cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * P, cudaMemcpyDeviceToHost, c.stream));
            SAGB_CUDA(cudaStreamSynchronize(c.stream));
            int ncycle = 0;
            for (int p = 0; p < P; p++) {
                hp[p] = BPair();
                hp[p].bit = bit[p];
                hp[p].nrm_b = nb[p];
                if (done[p]) continue;
                const double nr = hn[p];
                st.explicit_res[p] = nr / nb[p];
                if (kp.explicit_check && outer > 0 && !discarded[p] && nr <= kp.eps * nb[p]) {
                    done[p] = 1;
                    st.converged[p] = 1;
                    continue;
                }
                if (!discarded[p] && std::fabs(nr - prev[p]) / nr < 1.0e-8) {  // stagnation (irsolver.hpp:35)
                    done[p] = 1;
                    st.iters[p] = 0;
                    continue;
                }
                prev[p] = nr;
                discarded[p] = 0;
                hp[p].active = 1;
                ncycle++;
            }
            if (ncycle == 0) break;
            st.restarts++;
            // status bits of the previous cycle (including those raised on
            // the vectors of pairs that had already stopped) are dropped
            SAGB_CUDA(cudaMemsetAsync(pflag, 0, sizeof(unsigned) * P * 2, c.stream));
            SAGB_CUDA(cudaMemcpyAsync(pairs, hp.data(), sizeof(BPair) * P, cudaMemcpyHostToDevice, c.stream));
            SAGB_CUDA(cudaMemcpyAsync(e0, nrm, sizeof(double) * P, cudaMemcpyDeviceToDevice, c.stream));
            k_bbegin<<<(P + 127) / 128, 128, 0, c.stream>>>(P, e0, kp.eps, pairs, e, acc, m, kp.cycle_bits);
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                k_bv0<R><<<ntiles * kTileSub, kBThreads, 0, c.stream>>>(tiles, rvec, pairs, V);
            });
            c.launches += 2;
            const bool in_graph = cycle_steps();
            st.cycle_graphs += in_graph;
            k_btrsv<<<(P + 127) / 128, 128, 0, c.stream>>>(P, m, pairs, H, e, y);
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                k_bxupd<R><<<ntiles * kTileSub, kBThreads, 0, c.stream>>>(tiles, m, N0 * Rn, pairs, y, Z, x);
            });
            c.launches += 2;
            SAGB_CUDA(cudaMemcpyAsync(hp.data(), pairs, sizeof(BPair) * P, cudaMemcpyDeviceToHost, c.stream));
            SAGB_CUDA(cudaStreamSynchronize(c.stream));
            if (in_graph) {  // the steps that ran: as many as the longest pair took
                int steps = 0;
                for (int p = 0; p < P; p++) steps = std::max(steps, hp[p].jn);
                for (int j = 0; j < steps && j < (int)cyc.step_launches.size(); j++) c.launches += cyc.step_launches[j];
            }
            for (int p = 0; p < P; p++) {
                if (done[p] || !(hp[p].jn > 0)) continue;
                if (hp[p].bad) {
                    // cycle discarded (x untouched): one fractional bit less
                    st.flags |= hp[p].bad;
                    discarded[p] = 1;
                    if (!kp.fallback || bit[p] <= 1) {
                        done[p] = 1;
                        continue;
                    }
                    bit[p]--;
                    st.fallbacks[p]++;
                    continue;
                }
                st.iters[p] += hp[p].jn;
                if (hp[p].conv && !kp.explicit_check) {
                    done[p] = 1;
                    st.converged[p] = 1;
                }
            }
        }
        {
            std::vector<unsigned> pp(P);
            SAGB_CUDA(cudaMemcpyAsync(pp.data(), pflag_prec, sizeof(unsigned) * P, cudaMemcpyDeviceToHost, c.stream));
            SAGB_CUDA(cudaStreamSynchronize(c.stream));
            for (unsigned f : pp)
                if (f & ST_OVERFLOW) st.flags |= ST_PREC_OVF;
        }
        if (tail_from > 0) {
            unsigned mainf = 0;
            SAGB_CUDA(cudaMemcpy(&mainf, c.d_flags_main, sizeof(unsigned), cudaMemcpyDeviceToHost));
            if (mainf & ST_TIMEOUT) throw CudaError{"the V-cycle's persistent coarse tail timed out at a grid barrier"};
        }
        // the last cycle's update has not been checked yet
        residual(b, x);
        SAGB_CUDA(cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * P, cudaMemcpyDeviceToHost, c.stream));
        SAGB_CUDA(cudaStreamSynchronize(c.stream));
        for (int p = 0; p < P; p++) {
            st.explicit_res[p] = hn[p] / nb[p];
            st.final_bit[p] = bit[p];
            if (!done[p] && kp.explicit_check && hn[p] <= kp.eps * nb[p]) st.converged[p] = 1;
            if (!st.converged[p]) st.iters[p] = 0;
        }
    }
};

BatchEngine::BatchEngine(Ctx &c, std::shared_ptr<BatchHierarchy> h, int nrhs)
    : impl_(new Impl(c, std::move(h), nrhs)) {}
BatchEngine::~BatchEngine() { delete impl_; }
int BatchEngine::nrhs() const { return impl_->Rn; }
size_t BatchEngine::rows() const { return impl_->N0; }
void BatchEngine::precondition(const int *in, int *out) { impl_->vcycle_graph(in, out); }
void BatchEngine::pair_norms(const double *v, double *out_dev) {
    impl_->pair_norms(v);
    SAGB_CUDA(cudaMemcpyAsync(out_dev, impl_->nrm, sizeof(double) * (size_t)impl_->S * impl_->Rn,
                              cudaMemcpyDefault, impl_->c.stream));
}
void BatchEngine::solve(const KrylovParams &kp, const int *bits_sys, const double *b, const double *nrm_b, double *x,
                        BatchStats &st) {
    impl_->solve(kp, bits_sys, b, nrm_b, x, st);
    last_cycle_graphs_ = st.cycle_graphs;
}
void BatchEngine::set_groups(int level, int op, int group) {
    if (level < 0 || level >= impl_->Dmax) throw CudaError{"no such level"};
    DevBLevel &L = impl_->lv[level];
    DevBMat *M = op == 0 ? &L.A : op == 1 ? &L.LD : op == 2 ? &L.U : op == 3 ? &L.P : &L.R;
    M->group = group;
    impl_->clear_graphs();
}
int BatchEngine::sweep_form(int level, int set) {
    if (level < 0 || level >= impl_->Dmax) throw CudaError{"no such level"};
    DevBLevel &L = impl_->lv[level];
    if (set >= 0) {
        if (set > 3 || ((set == 1 || set == 2) && L.ngroups == 0) || (set == 2 && !L.pk_items) ||
            (set == 3 && !L.cp_items))
            throw CudaError{"sweep form not available at this level"};
        L.use_cluster = set;
        impl_->clear_graphs();
    }
    return L.use_cluster;
}
int BatchEngine::ell(int level, int op, int set) {
    if (level < 0 || level >= impl_->Dmax || (op != 0 && op != 2)) throw CudaError{"no such operator"};
    DevBMat &M = op == 0 ? impl_->lv[level].A : impl_->lv[level].U;
    if (set >= 0) {
        if (set > 0 && !M.ell_va) throw CudaError{"this operator has no ELL copy"};
        M.ell = set > 0;
        if (level == 0 && op == 0) impl_->dot_ell = M.ell;
        impl_->clear_graphs();
    }
    return M.ell && M.ell_va ? 1 : 0;
}
int BatchEngine::fused_sweeps(int set) {
    Impl &I = *impl_;
    if (set >= 0) {
        I.fuse_jac = set > 0;
        I.clear_graphs();
    }
    const int t = I.tail_from > 0 && I.d_steps ? I.tail_from : I.Dmax;
    int n = 0;
    for (int l = 0; l < I.Dmax; l++) n += I.fused_pre(l, t);
    return n;
}
int BatchEngine::compressed(int level, int op, int set) {
    if (level < 0 || level >= impl_->Dmax || (op != 0 && op != 2)) throw CudaError{"no such operator"};
    DevBMat &M = op == 0 ? impl_->lv[level].A : impl_->lv[level].U;
    if (set >= 0) {
        if (set > 0 && !M.cdv) throw CudaError{"this operator has no compressed columns"};
        M.d16 = set > 0;
        impl_->clear_graphs();
    }
    return M.d16 && M.cdv ? 1 : 0;
}
unsigned BatchEngine::tail_selftest(int level, double timeout_ms) {
    Impl &I = *impl_;
    const int keep_from = I.tail_from, keep_grid = I.tail_grid;
    if (!I.build_tail(level)) throw CudaError{"no persistent tail from this level"};
    unsigned before = 0, after = 0;
    SAGB_CUDA(cudaStreamSynchronize(I.c.stream));
    SAGB_CUDA(cudaMemcpy(&before, I.c.d_flags_main, sizeof(unsigned), cudaMemcpyDeviceToHost));
    // one launch whose first grid barrier expects one CTA more than the grid has
    {
        PrecFlags guard(I.c);
        I.cur_pflag = I.pflag_prec;
        I.launch_tail(1u, (unsigned long long)(timeout_ms * 1e6));
        I.cur_pflag = I.pflag;
    }
    unsigned tail_status = 0;
    SAGB_CUDA(cudaMemcpyAsync(&tail_status, I.tail_bar + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, I.c.stream));
    SAGB_CUDA(cudaStreamSynchronize(I.c.stream));
    SAGB_CUDA(cudaMemcpy(&after, I.c.d_flags_main, sizeof(unsigned), cudaMemcpyDeviceToHost));
    // the status word as it was, and the tail as it was
    SAGB_CUDA(cudaMemcpy(I.c.d_flags_main, &before, sizeof(unsigned), cudaMemcpyHostToDevice));
    SAGB_CUDA(cudaMemset(I.pflag, 0, sizeof(unsigned) * (size_t)I.S * I.Rn * 2));
    if (keep_from > 0) I.build_tail(keep_from, keep_grid);
    else I.drop_tail();
    return (tail_status | after) & ST_TIMEOUT;
}

int BatchEngine::tail(int set, int grid) {
    Impl &I = *impl_;
    if (set == 0) I.drop_tail();
    else if (set > 0 && !I.build_tail(set, grid)) throw CudaError{"no persistent tail from this level"};
    return I.tail_from;
}
int BatchEngine::group(int level, int op) const {
    const DevBLevel &L = impl_->lv[level];
    const DevBMat *M = op == 0 ? &L.A : op == 1 ? &L.LD : op == 2 ? &L.U : op == 3 ? &L.P : &L.R;
    return M->group;
}
int BatchEngine::depth() const { return impl_->Dmax; }

void BatchEngine::level_op(int level, int op, const int *in, int *out) {
    Impl &I = *impl_;
    if (level < 0 || level >= I.Dmax || op < 0 || op > 4) throw CudaError{"no such operator"};
    DevBLevel &L = I.lv[level];
    if (op == 1) return I.sweep(level, in, out);
    const DevBMat &M = op == 0 ? L.A : op == 2 ? L.U : op == 3 ? L.P : L.R;
    I.bspmv(M, in, out, SPMV_SET, nullptr, op == 4 ? L.row_sys_next : L.row_sys);
}

float BatchEngine::time_op(int level, int op, const int *in, int *out, int reps, bool cold) {
    Impl &I = *impl_;
    if (reps < 1 || op < 0 || op > 6 || (op <= 4 && (level < 0 || level >= I.Dmax)))
        throw CudaError{"no such operator"};
    cudaEvent_t e0, e1;
    SAGB_CUDA(cudaEventCreate(&e0));
    SAGB_CUDA(cudaEventCreate(&e1));
    float ms = 0;
    try {
        auto body = [&] {
            if (op == 5) I.lu(I.pflag);
            else if (op == 6) I.vcycle(in, out);
            else level_op(level, op, in, out);
        };
        ms = cold ? I.timed_cold(body, reps, e0, e1) : I.timed(body, reps, e0, e1);
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms;
}

void BatchEngine::coarse_solve() {
    Impl &I = *impl_;
    I.lu(I.pflag);
}

void BatchEngine::level_info(int level, int op, int *n, int *m, int64_t *nnz, int *ncolours) const {
    const Impl &I = *impl_;
    if (level < 0 || level >= I.Dmax || op < 0 || op > 4) throw CudaError{"no such operator"};
    const BatchLevel &L = I.h->lv[level];
    const BatchCsr &M = op == 0 ? L.A : op == 1 ? L.LD : op == 2 ? L.U : op == 3 ? L.P : L.R;
    if (n) *n = M.n;
    if (m) *m = M.m;
    if (nnz) *nnz = M.nnz();
    if (ncolours) *ncolours = (int)L.colour_ptr.size() - 1;
}

// Autotuner: for every level operator, time each candidate lanes-per-row
// value on the current vectors and keep the fastest (the SpMV and the colour
// sweep have the same results for every value).
void BatchEngine::autotune(int reps) {
    Impl &I = *impl_;
    Ctx &c = I.c;
    cudaEvent_t e0, e1;
    SAGB_CUDA(cudaEventCreate(&e0));
    SAGB_CUDA(cudaEventCreate(&e1));
    int *xa = (int *)dmalloc(sizeof(int) * I.N0 * I.Rn), *xb = (int *)dmalloc(sizeof(int) * I.N0 * I.Rn);
    SAGB_CUDA(cudaMemset(xa, 0, sizeof(int) * I.N0 * I.Rn));
    SAGB_CUDA(cudaMemset(xb, 0, sizeof(int) * I.N0 * I.Rn));
    auto timeit = [&](auto &&fn) { return I.timed(fn, reps, e0, e1); };
    if (I.nlu) {
        // the coarse LU: one CTA per system or one cluster per system
        float bt[2] = {0, 0};
        for (int uc = 0; uc < 2; uc++) {
            I.lu_cluster = uc;
            bt[uc] = timeit([&] { I.lu(I.pflag); });
        }
        I.lu_cluster = bt[1] < bt[0];
    }
    const int cand[] = {0, 1, 2, 4, 8, 16, 32};  // 0: tile-staged stream (not for the colour sweep)
    for (int l = 0; l < I.Dmax; l++) {
        DevBLevel &L = I.lv[l];
        for (int op = 0; op < 5; op++) {
            DevBMat *M = op == 0 ? &L.A : op == 1 ? &L.LD : op == 2 ? &L.U : op == 3 ? &L.P : &L.R;
            if (M->d.n == 0) continue;
            if (op == 1) {
                // the sweep form first: one launch per colour, or one cluster
                // launch per level (plain or packed); each form at its best group
                float bt[4] = {1e30f, 1e30f, 1e30f, 1e30f};
                int bg[4] = {M->group, M->group, M->group, M->group};
                const bool avail[4] = {true, L.ngroups > 0, L.ngroups > 0 && L.pk_items != nullptr,
                                       L.cp_items != nullptr};
                const int nform = 4;
                for (int uc = 0; uc < nform; uc++) {
                    if (!avail[uc]) continue;
                    L.use_cluster = uc;
                    for (int g : cand) {
                        if (g == 0) continue;
                        M->group = g;
                        const float ms = timeit([&] { I.sweep(l, xa, xb); });
                        if (ms < bt[uc]) {
                            bt[uc] = ms;
                            bg[uc] = g;
                        }
                    }
                }
                int best_form = 0;
                for (int uc = 1; uc < nform; uc++)
                    if (bt[uc] < bt[best_form]) best_form = uc;
                L.use_cluster = best_form;
                M->group = bg[best_form];
                continue;
            }
            float best = 1e30f;
            int bestg = M->group;
            bool bestd = false;
            M->ell = false;
            for (int dd = 0; dd < (M->cdv ? 2 : 1); dd++)
                for (int g : cand) {
                    if (dd && g == 0) continue;  // the compressed columns are read by the lane kernels
                    M->group = g;
                    M->d16 = dd;
                    const float ms = timeit([&] { I.bspmv(*M, xa, xb, SPMV_SET, nullptr, L.row_sys); });
                    if (ms < best) {
                        best = ms;
                        bestg = g;
                        bestd = dd;
                    }
                }
            M->group = bestg;
            M->d16 = bestd;
            if (M->ell_va) {  // the ELL copy, where the operator has one
                M->ell = true;
                const float ms = timeit([&] { I.bspmv(*M, xa, xb, SPMV_SET, nullptr, L.row_sys); });
                M->ell = ms < best;
            }
        }
    }
    {
        // the persistent coarse tail: from which level on (or none), by V-cycle time
        I.drop_tail();
        float best = timeit([&] { I.vcycle(xa, xb); });
        int bestt = 0, bestg = 0;
        try {
            // from the coarsest level up; stop once a start level is no better
            // than the one below it (the tail only pays where levels are tiny)
            float prev = best;
            for (int t = I.Dmax - 1; t >= 1; t--) {
                bool any = false;
                float here = 1e30f;
                for (int g : {32, 0}) {
                    if (!I.build_tail(t, g)) break;
                    any = true;
                    const float ms = timeit([&] { I.vcycle(xa, xb); });
                    here = std::min(here, ms);
                    if (ms < best) {
                        best = ms;
                        bestt = t;
                        bestg = g;
                    }
                }
                if (!any || here >= prev) break;
                prev = here;
            }
        } catch (const CudaError &) {
            bestt = 0;  // the cooperative launch is not available here: no tail
            cudaGetLastError();
        }
        if (bestt > 0) I.build_tail(bestt, bestg);
        else I.drop_tail();
    }
    {
        // the Arnoldi SpMV + first dot, on its own (acc for one column, m = 1)
        unsigned long long *acct = (unsigned long long *)dmalloc(sizeof(unsigned long long) * (size_t)I.S * I.Rn * 3);
        SAGB_CUDA(cudaMemset(acct, 0, sizeof(unsigned long long) * (size_t)I.S * I.Rn * 3));
        float best = 1e30f;
        int bestg = I.lv[0].A.group;
        bool bestd = false;
        for (int dd = 0; dd < (I.lv[0].A.cdv ? 2 : 1); dd++)
            for (int g : cand) {
                if (dd && g == 0) continue;
                I.dot_group = g;
                I.dot_d16 = dd;
                const float ms = timeit([&] { I.spmv_dot(xa, xb, xa, acct, 1); });
                if (ms < best) {
                    best = ms;
                    bestg = g;
                    bestd = dd;
                }
            }
        I.dot_group = bestg;
        I.dot_d16 = bestd;
        I.dot_ell = false;
        if (I.lv[0].A.ell_va) {
            I.dot_ell = true;
            const float ms = timeit([&] { I.spmv_dot(xa, xb, xa, acct, 1); });
            I.dot_ell = ms < best;
        }
        dfree(acct);
    }
    SAGB_CUDA(cudaMemsetAsync(I.pflag, 0, sizeof(unsigned) * (size_t)I.S * I.Rn * 2, c.stream));
    SAGB_CUDA(cudaMemsetAsync(c.d_flags, 0, sizeof(unsigned), c.stream));
    SAGB_CUDA(cudaStreamSynchronize(c.stream));
    dfree(xa);
    dfree(xb);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    I.clear_graphs();
}

}  // namespace sagb
