// Batched FP64-AMG-FGMRES and FP32-mixed AMG-FGMRES: the floating-point
// siblings of the batched integer engine (batch.cu), on the same systems,
// coarsening, level order, colour caps, coarsest-level size and launch model,
// so that the integer solver is compared with an FP64 solver that runs the
// same GPU design.
//
// Per system and right-hand side ("pair") the arithmetic is that of the
// reference's floating-point classes with the multicolour smoother:
//   * V-cycle: dfAMG::Precondition (INTAMG.hpp:86-134): pre-smoothing,
//     r = in - A x, restriction, the coarsest LU<T> (lu.hpp:11-39), then
//     interpolation, x += P x_c, post-smoothing (tmp = in - U x, x = LD^-1 tmp).
//   * sweep: ldtri::CSR<T>::SpTRSV (ldtri.hpp:47-57) row rule
//     out_i = (in_i - sum_j l_ij out_j) * dinv_i, rows in colour order, one
//     launch per colour (rows of a colour read only earlier colours).
//   * FGMRES<double> (gmres.hpp:19-98) / FGMRES<float> (gmres.hpp:101-180):
//     e0 = ||r|| (FP64, stored as T), V0 = (T)(r / e0), modified Gram-Schmidt
//     with T dot products, Givens rotations in T, convergence on
//     |e_{j+1}| <= ||b|| eps, x += y_k Z_k (AxpyFD for float).
//   * Restarted (irsolver.hpp:27-43) per pair on the host, FP64 residuals
//     of every pair from one launch.
// Dot products and norms are sums in a fixed order (per tile, then per pair
// over its tiles), so results do not depend on timing; they differ from the
// reference's sequential sums in the last bits, as any parallel order does.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <type_traits>

#include "../sagb_internal.hpp"
#include "common.cuh"
#include "cycle_graph.cuh"

namespace sagb {
namespace {

constexpr int kFThreads = 256;
constexpr int kFTileRows = 2048;
constexpr int kFLuThreads = 512;
constexpr int kFPkU = 4;  // entries per lane fetched before the launch wait

// ------------------------------------------------------------ vector access
// Rows interleave the R right-hand sides (v[row * R + r]): one 8/16/32-byte
// access per row.  MODE 0: read-only cache (data written by earlier launches),
// 1: plain coherent load (written earlier in the same sweep), 2: through L2.
template <int MODE, typename V>
__device__ __forceinline__ V ldv(const V *p) {
    if constexpr (MODE == 0) return __ldg(p);
    else if constexpr (MODE == 2) return __ldcg(p);
    else return *p;
}

template <typename T, int R, int MODE = 0>
__device__ __forceinline__ void fld(const T *x, int row, T (&v)[R]) {
    if constexpr (std::is_same<T, double>::value) {
        if constexpr (R == 4) {
            const double2 *p = reinterpret_cast<const double2 *>(x) + 2 * (size_t)row;
            const double2 a = ldv<MODE>(p), b = ldv<MODE>(p + 1);
            v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
        } else if constexpr (R == 2) {
            const double2 a = ldv<MODE>(reinterpret_cast<const double2 *>(x) + row);
            v[0] = a.x; v[1] = a.y;
        } else {
            v[0] = ldv<MODE>(x + row);
        }
    } else {
        if constexpr (R == 4) {
            const float4 a = ldv<MODE>(reinterpret_cast<const float4 *>(x) + row);
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        } else if constexpr (R == 2) {
            const float2 a = ldv<MODE>(reinterpret_cast<const float2 *>(x) + row);
            v[0] = a.x; v[1] = a.y;
        } else {
            v[0] = ldv<MODE>(x + row);
        }
    }
}

template <typename T, int R>
__device__ __forceinline__ void fst(T *x, int row, const T (&v)[R]) {
    if constexpr (std::is_same<T, double>::value) {
        if constexpr (R == 4) {
            double2 *p = reinterpret_cast<double2 *>(x) + 2 * (size_t)row;
            p[0] = make_double2(v[0], v[1]);
            p[1] = make_double2(v[2], v[3]);
        } else if constexpr (R == 2) {
            reinterpret_cast<double2 *>(x)[row] = make_double2(v[0], v[1]);
        } else {
            x[row] = v[0];
        }
    } else {
        if constexpr (R == 4) reinterpret_cast<float4 *>(x)[row] = make_float4(v[0], v[1], v[2], v[3]);
        else if constexpr (R == 2) reinterpret_cast<float2 *>(x)[row] = make_float2(v[0], v[1]);
        else x[row] = v[0];
    }
}

template <typename T, int R, int G>
__device__ __forceinline__ void lane_reduce(T (&a)[R]) {
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) a[r] += __shfl_xor_sync(0xffffffffu, a[r], o);
}

template <typename T>
struct FMat {
    int n;
    const int *rptr, *cind;
    const T *val;
};

// acc += sum_j a_ij x_j over entries [j0, e1) of a row, lanes G apart, four
// entries a lane in flight (MODE: how x is read)
template <typename T, int R, int G, int MODE>
__device__ __forceinline__ void row_acc(const int *__restrict__ cind, const T *__restrict__ val, int j0, int e1,
                                        const T *x, T (&acc)[R]) {
    int j = j0;
    for (; j + 3 * G < e1; j += 4 * G) {
        int cc[4];
        T vv[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            cc[q] = __ldg(cind + j + q * G);
            vv[q] = __ldg(val + j + q * G);
        }
        T xv[4][R];
#pragma unroll
        for (int q = 0; q < 4; q++) fld<T, R, MODE>(x, cc[q], xv[q]);
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] += vv[q] * xv[q][r];
    }
    if (j < e1) {  // the last 1-3 entries of this lane in one predicated round
        int cc[3];
        T vv[3];
#pragma unroll
        for (int q = 0; q < 3; q++) {
            const int jj = j + q * G;
            cc[q] = jj < e1 ? __ldg(cind + jj) : -1;
            vv[q] = jj < e1 ? __ldg(val + jj) : T(0);
        }
#pragma unroll
        for (int q = 0; q < 3; q++) {
            if (cc[q] < 0) continue;
            T xv[R];
            fld<T, R, MODE>(x, cc[q], xv);
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] += vv[q] * xv[r];
        }
    }
}

// ------------------------------------------------------------------ SpMV
// The one-colour smoother step fused into a level SpMV's epilogue (as in the
// integer engine): where a level's split kept one colour, LD is its diagonal
// and a sweep is out_i = (in_i - 0) * dinv_i (ldtri::CSR<T>, ldtri.hpp:49-58,
// with no off-diagonal term).  jac 1: y = R r and x2 = step(y) on the next
// level's smoothing rows; jac 2: y = step(z - U x).
template <typename T>
struct FJac {
    const T *dinv;  // the one-colour LD's values (its inverted diagonal), one per row
    int n;          // jac 1: rows of y that smooth (a prefix)
    T *x2;          // jac 1: the step's output
};

// y = A x (SPMV_SET), y = z - A x (SPMV_RESID) or y = y + A x (SPMV_ADD):
// CSR<T>::SpMV (spmat.hpp:43-52) with Sub / Add (blas1.hpp:62-72)
template <typename T, int R, int G>
__global__ void __launch_bounds__(kFThreads)
k_fspmv(FMat<T> A, const T *__restrict__ x, T *__restrict__ y, const T *__restrict__ z, int mode, int jac,
        FJac<T> J) {
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * kFThreads + threadIdx.x;
    const int row = (int)(tid / G), lane = (int)(tid % G);
    const bool ok = row < A.n;
    const int e0 = ok ? __ldg(A.rptr + row) : 0, e1 = ok ? __ldg(A.rptr + row + 1) : 0;
    constexpr int kPre = 4;  // entries per lane fetched before the wait (more cost occupancy)
    int cc[kPre];
    T vv[kPre];
#pragma unroll
    for (int q = 0; q < kPre; q++) {  // static: fetched before the wait
        const int j = e0 + lane + q * G;
        cc[q] = j < e1 ? __ldg(A.cind + j) : -1;
        vv[q] = j < e1 ? __ldg(A.val + j) : T(0);
    }
    pdl_wait();
    T acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
#pragma unroll
    for (int q = 0; q < kPre; q++) {
        if (cc[q] < 0) continue;
        T xv[R];
        fld<T, R, 0>(x, cc[q], xv);
#pragma unroll
        for (int r = 0; r < R; r++) acc[r] += vv[q] * xv[r];
    }
    if (e1 - e0 > kPre * G) row_acc<T, R, G, 0>(A.cind, A.val, e0 + lane + kPre * G, e1, x, acc);
    lane_reduce<T, R, G>(acc);
    if (lane == 0 && ok) {
        T out[R];
        if (mode == SPMV_RESID) {
            T zz[R];
            fld<T, R, 0>(z, row, zz);
#pragma unroll
            for (int r = 0; r < R; r++) out[r] = zz[r] - acc[r];
        } else if (mode == SPMV_ADD) {
            T yy[R];
            fld<T, R, 1>(y, row, yy);
#pragma unroll
            for (int r = 0; r < R; r++) out[r] = acc[r] + yy[r];
        } else {
#pragma unroll
            for (int r = 0; r < R; r++) out[r] = acc[r];
        }
        if (jac == 2) {
            const T dinv = __ldg(J.dinv + row);
#pragma unroll
            for (int r = 0; r < R; r++) out[r] = (out[r] - T(0)) * dinv;
        }
        fst<T, R>(y, row, out);
        if (jac == 1 && row < J.n) {
            const T dinv = __ldg(J.dinv + row);
            T x2[R];
#pragma unroll
            for (int r = 0; r < R; r++) x2[r] = (out[r] - T(0)) * dinv;
            fst<T, R>(J.x2, row, x2);
        }
    }
}

// --------------------------------------------------------- colour sweeps
// One colour over the batched LD (rows through the colour's row list)
template <typename T, int R, int G>
__global__ void __launch_bounds__(kFThreads)
k_fcolour(int cnt, const int *__restrict__ rows, FMat<T> LD, const T *__restrict__ in, T *out) {
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * kFThreads + threadIdx.x;
    const int k = (int)(tid / G), lane = (int)(tid % G);
    int row = -1, e0 = 0, dpos = 0;
    if (k < cnt) {
        row = __ldg(rows + k);
        e0 = __ldg(LD.rptr + row);
        dpos = __ldg(LD.rptr + row + 1) - 1;
    }
    pdl_wait();
    T acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
    if (k < cnt) row_acc<T, R, G, 1>(LD.cind, LD.val, e0 + lane, dpos, out, acc);
    lane_reduce<T, R, G>(acc);
    if (lane == 0 && k < cnt) {
        const T dinv = __ldg(LD.val + dpos);
        T iv[R], res[R];
        fld<T, R, 0>(in, row, iv);
#pragma unroll
        for (int r = 0; r < R; r++) res[r] = (iv[r] - acc[r]) * dinv;
        fst<T, R>(out, row, res);
    }
}

// One colour over LD packed at setup in colour-row order: item {row, first
// entry, entries, -} with its inverse diagonal, entries {column} / {value} of
// the strictly lower part; the item and each lane's first entries are fetched
// before the launch wait, so a colour waits for one round trip of the earlier
// colours' values.
template <typename T, int R, int G>
__global__ void __launch_bounds__(kFThreads)
k_fcolour_packed(int ib, int ie, const int4 *__restrict__ items, const T *__restrict__ idinv,
                 const int *__restrict__ ecol, const T *__restrict__ eval, const T *__restrict__ in, T *out) {
    pdl_trigger();
    const long long tid = (long long)blockIdx.x * kFThreads + threadIdx.x;
    const int lane = (int)(tid % G);
    const long long it = ib + tid / G;
    const bool ok = it < ie;
    const int4 hd = ok ? __ldg(items + it) : make_int4(0, 0, 0, 0);
    const T dinv = ok ? __ldg(idinv + it) : T(0);
    int cc[kFPkU];
    T vv[kFPkU];
#pragma unroll
    for (int u = 0; u < kFPkU; u++) {
        const int j = lane + u * G;
        cc[u] = j < hd.z ? __ldg(ecol + hd.y + j) : -1;
        vv[u] = j < hd.z ? __ldg(eval + hd.y + j) : T(0);
    }
    pdl_wait();
    T iv[R];
    if (ok) fld<T, R, 0>(in, hd.x, iv);
    T acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0;
#pragma unroll
    for (int u = 0; u < kFPkU; u++) {
        if (cc[u] < 0) continue;
        T xv[R];
        fld<T, R, 1>(out, cc[u], xv);
#pragma unroll
        for (int r = 0; r < R; r++) acc[r] += vv[u] * xv[r];
    }
    if (hd.z > kFPkU * G) row_acc<T, R, G, 1>(ecol + hd.y, eval + hd.y, lane + kFPkU * G, hd.z, out, acc);
    lane_reduce<T, R, G>(acc);
    if (lane == 0 && ok) {
        T res[R];
#pragma unroll
        for (int r = 0; r < R; r++) res[r] = (iv[r] - acc[r]) * dinv;
        fst<T, R>(out, hd.x, res);
    }
}

// ------------------------------------------------------------ coarse LU
template <typename T>
struct FLuDesc {
    int n, sys;
    long long mat_off, d_off;
    const T *in;
    T *out;
};

// LU<T>::Solve (lu.hpp:35-38) for every system: ltri forward
// (x_i = in_i - sum_{j<i} l_ij x_j) then dutri backward
// (x_i = (t_i - sum_{j>i} u_ij x_j) * dinv_i), one CTA per system, 32-row
// panels: warps reduce panel rows against the solved part, warp 0 solves the
// diagonal block from registers.
template <typename T, int R>
__global__ void __launch_bounds__(kFLuThreads, 1)
k_flu(const FLuDesc<T> *__restrict__ desc, const T *__restrict__ Lcat, const T *__restrict__ Ucat,
      const T *__restrict__ dcat) {
    pdl_trigger();
    pdl_wait();
    extern __shared__ __align__(16) unsigned char fsm[];
    const FLuDesc<T> d = desc[blockIdx.x];
    const int n = d.n;
    T *t = reinterpret_cast<T *>(fsm);
    T *x = t + (size_t)n * R;
    const T *L = Lcat + d.mat_off, *U = Ucat + d.mat_off, *dinv = dcat + d.d_off;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = kFLuThreads / 32;
    for (int i = tid; i < n * R; i += kFLuThreads) t[i] = d.in[i];
    __syncthreads();
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int kb = min(32, n - k0);
        for (int pr = warp; k0 > 0 && pr < kb; pr += NW) {
            const T *row = L + (size_t)(k0 + pr) * n;
            T acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            for (int c = lane; c < k0; c += 32) {
                const T v = __ldg(row + c);
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] += v * x[c * R + r];
            }
            lane_reduce<T, R, 32>(acc);
            if (lane == 0)
#pragma unroll
                for (int r = 0; r < R; r++) t[(k0 + pr) * R + r] -= acc[r];
        }
        __syncthreads();
        if (warp == 0) {
            T blk[32];
            const T *row = L + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) blk[c] = (lane < kb && c < lane) ? __ldg(row + c) : T(0);
            T tr[R];
#pragma unroll
            for (int r = 0; r < R; r++) tr[r] = lane < kb ? t[(k0 + lane) * R + r] : T(0);
#pragma unroll
            for (int c = 0; c < 32; c++) {
                if (c < kb) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const T xc = __shfl_sync(0xffffffffu, tr[r], c);
                        if (lane > c) tr[r] -= blk[c] * xc;
                        if (lane == c) x[(k0 + c) * R + r] = xc;
                    }
                }
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < n * R; i += kFLuThreads) t[i] = x[i];
    __syncthreads();
    for (int k1 = n; k1 > 0; k1 -= 32) {
        const int kb = min(32, k1);
        const int k0 = k1 - kb;
        for (int pr = warp; k1 < n && pr < kb; pr += NW) {
            const T *row = U + (size_t)(k0 + pr) * n;
            T acc[R];
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = 0;
            for (int c = k1 + lane; c < n; c += 32) {
                const T v = __ldg(row + c);
#pragma unroll
                for (int r = 0; r < R; r++) acc[r] += v * x[c * R + r];
            }
            lane_reduce<T, R, 32>(acc);
            if (lane == 0)
#pragma unroll
                for (int r = 0; r < R; r++) t[(k0 + pr) * R + r] -= acc[r];
        }
        __syncthreads();
        if (warp == 0) {
            T blk[32];
            const T *row = U + (size_t)(k0 + lane) * n + k0;
#pragma unroll
            for (int c = 0; c < 32; c++) blk[c] = (lane < kb && c > lane && c < kb) ? __ldg(row + c) : T(0);
            T tr[R];
#pragma unroll
            for (int r = 0; r < R; r++) tr[r] = lane < kb ? t[(k0 + lane) * R + r] : T(0);
            const T dv = lane < kb ? __ldg(dinv + k0 + lane) : T(0);
#pragma unroll
            for (int c = 31; c >= 0; c--) {
                if (c < kb) {
#pragma unroll
                    for (int r = 0; r < R; r++) {
                        const T xc = __shfl_sync(0xffffffffu, tr[r] * dv, c);
                        if (lane < c) tr[r] -= blk[c] * xc;
                        if (lane == c) x[(k0 + c) * R + r] = xc;
                    }
                }
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < n * R; i += kFLuThreads) d.out[i] = x[i];
}

// ============================================================== Krylov

struct FTile {
    int sys, row0, row1, first;  // rows [row0, row1) of one system
};

struct FPair {
    double e0, e_inv, nrm_b, crit, relres;  // crit = ||b|| eps
    int active, jn, conv;
    unsigned bad;
};

struct FInfo {
    int n_active;
    unsigned flags;
};

// fixed-order block sum of R values; the result is valid in every thread
template <typename T, int R>
__device__ __forceinline__ void block_sum_all(T (&v)[R], T (*sh)[R]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    lane_reduce<T, R, 32>(v);
    if (lane == 0)
#pragma unroll
        for (int r = 0; r < R; r++) sh[warp][r] = v[r];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int r = 0; r < R; r++) {
            T s = 0;
            for (int w = 0; w < kFThreads / 32; w++) s += sh[w][r];
            sh[0][r] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = sh[0][r];
    __syncthreads();
}

// the per-pair sum of slot `slot` over the system's tiles, in a fixed order
// (every CTA of the system computes the same value)
template <typename T, int R>
__device__ __forceinline__ void system_sum(const T *__restrict__ part, int slot, int ntiles, int t0, int t1,
                                           T (&h)[R], T (*sh)[R]) {
    const T *ps = part + (size_t)slot * ntiles * R;
#pragma unroll
    for (int r = 0; r < R; r++) h[r] = 0;
    for (int k = t0 + threadIdx.x; k < t1; k += kFThreads)
#pragma unroll
        for (int r = 0; r < R; r++) h[r] += ps[(size_t)k * R + r];
    block_sum_all<T, R>(h, sh);
}

// e[0] = (T) ||r||, e_inv = 1 / e[0] (gmres.hpp:50-51, 131-132)
template <typename T>
__global__ void k_fbegin(int P, const double *__restrict__ nrm, double eps, FPair *pairs, T *e, int m) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    FPair &q = pairs[p];
    q.jn = 0;
    q.conv = 0;
    q.bad = 0;
    q.crit = q.nrm_b * eps;
    if (!q.active) return;
    const T e0 = (T)nrm[p];
    e[(size_t)p * (m + 1)] = e0;
    q.e0 = (double)e0;
    q.e_inv = 1.0 / (double)e0;
}

// the elementwise Krylov kernels run one row per thread: block b covers rows
// row0 + (b % kFTileSub) * kFThreads + [0, kFThreads) of tile b / kFTileSub
constexpr int kFTileSub = kFTileRows / kFThreads;

template <typename T, int R>
__global__ void __launch_bounds__(kFThreads)
k_fv0(const FTile *__restrict__ tiles, const double *__restrict__ rv, const FPair *__restrict__ pairs,
      T *__restrict__ V0) {
    const FTile t = tiles[blockIdx.x / kFTileSub];
    const int i = t.row0 + (blockIdx.x % kFTileSub) * kFThreads + threadIdx.x;
    if (i >= t.row1) return;
#pragma unroll
    for (int r = 0; r < R; r++)
        if (pairs[t.sys * R + r].active)
            V0[(size_t)i * R + r] = (T)(__ldg(rv + (size_t)i * R + r) * pairs[t.sys * R + r].e_inv);
}

// w = A z on one tile's rows, part[0][tile] = V0 . w
template <typename T, int R, int G>
__global__ void __launch_bounds__(kFThreads)
k_fspmv_dot(const FTile *__restrict__ tiles, FMat<T> A, const T *__restrict__ z, T *__restrict__ w,
            const T *__restrict__ v0, T *__restrict__ part) {
    pdl_trigger();
    pdl_wait();
    __shared__ T sh[kFThreads / 32][R];
    const FTile t = tiles[blockIdx.x];
    const int lane = threadIdx.x % G;
    T dot[R];
#pragma unroll
    for (int r = 0; r < R; r++) dot[r] = 0;
    for (int row0 = t.row0; row0 < t.row1; row0 += kFThreads / G) {
        const int row = row0 + threadIdx.x / G;
        T a[R];
#pragma unroll
        for (int r = 0; r < R; r++) a[r] = 0;
        if (row < t.row1) row_acc<T, R, G, 0>(A.cind, A.val, __ldg(A.rptr + row) + lane, __ldg(A.rptr + row + 1), z, a);
        lane_reduce<T, R, G>(a);
        if (lane == 0 && row < t.row1) {
            T vv[R];
            fld<T, R, 0>(v0, row, vv);
#pragma unroll
            for (int r = 0; r < R; r++) dot[r] += vv[r] * a[r];
            fst<T, R>(w, row, a);
        }
    }
    block_sum_all<T, R>(dot, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) part[(size_t)blockIdx.x * R + r] = dot[r];
}

// MGS pass k of step j: h = V_k . w (slot k summed over the system's tiles),
// H[j][k] = h, w += (-h) V_k (Axpy, gmres.hpp:60-61), then slot k+1 = V_{k+1} . w
// or, in the last pass, w . w
template <typename T, int R, bool LAST>
__global__ void __launch_bounds__(kFThreads)
k_fmgs(const FTile *__restrict__ tiles, const int *__restrict__ tile_ptr, int ntiles, int k, int j, int m,
       size_t vstride, const T *__restrict__ V, T *__restrict__ w, const FPair *__restrict__ pairs, T *part, T *H) {
    pdl_trigger();
    pdl_wait();
    __shared__ T sh[kFThreads / 32][R];
    const FTile t = tiles[blockIdx.x];
    T h[R];
    system_sum<T, R>(part, k, ntiles, tile_ptr[t.sys], tile_ptr[t.sys + 1], h, sh);
    bool act[R];
    T a[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = t.sys * R + r;
        act[r] = pairs[p].active != 0;
        if (t.first && threadIdx.x == 0 && act[r]) H[(size_t)p * (m + 1) * m + (size_t)j * (m + 1) + k] = h[r];
        a[r] = -h[r];
    }
    const T *vk = V + (size_t)k * vstride;
    const T *vk1 = V + (size_t)(k + 1) * vstride;
    T sum[R];
#pragma unroll
    for (int r = 0; r < R; r++) sum[r] = 0;
    for (int i = t.row0 + threadIdx.x; i < t.row1; i += kFThreads) {
        T wv[R], v[R], v1[R];
        fld<T, R, 1>(w, i, wv);
        fld<T, R, 0>(vk, i, v);
        if (!LAST) fld<T, R, 0>(vk1, i, v1);
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (!act[r]) continue;
            wv[r] += a[r] * v[r];
            sum[r] += LAST ? wv[r] * wv[r] : v1[r] * wv[r];
        }
        fst<T, R>(w, i, wv);
    }
    block_sum_all<T, R>(sum, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) part[((size_t)(k + 1) * ntiles + blockIdx.x) * R + r] = sum[r];
}

// per pair (one warp): H_{j+1,j} = ||w||, 1 / H_{j+1,j}, Grot of the earlier
// rotations, Ggen, e update and the convergence test (gmres.hpp:63-80)
template <typename T>
__global__ void k_fgivens(int P, int R, int j, int m, int ntiles, const int *__restrict__ tile_ptr, FPair *pairs,
                          const T *__restrict__ part, T *Hall, T *call, T *sall, T *eall, T *ascal, FInfo *info) {
    pdl_trigger();
    pdl_wait();
    const int p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (p >= P) return;
    FPair &q = pairs[p];
    if (!q.active) return;
    const int s = p / R, r = p % R;
    const T *ps = part + (size_t)(j + 1) * ntiles * R;
    T nsq = 0;
    for (int k = tile_ptr[s] + lane; k < tile_ptr[s + 1]; k += 32) nsq += ps[(size_t)k * R + r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nsq += __shfl_xor_sync(0xffffffffu, nsq, o);
    if (lane) return;
    T *Hj = Hall + (size_t)p * (m + 1) * m + (size_t)j * (m + 1);
    T *c = call + (size_t)p * m, *sn = sall + (size_t)p * m, *e = eall + (size_t)p * (m + 1);
    Hj[j + 1] = (T)sqrt(nsq);
    unsigned bad = 0;
    if (!(Hj[j + 1] > T(0))) bad |= ST_DIVZERO;  // zero or NaN
    ascal[p] = (T)1 / Hj[j + 1];
    for (int k = 0; k < j; k++) {
        const T tt = Hj[k];
        Hj[k] = c[k] * tt - sn[k] * Hj[k + 1];
        Hj[k + 1] = sn[k] * tt + c[k] * Hj[k + 1];
    }
    const T aa = Hj[j], bb = Hj[j + 1];
    const T rr = (T)sqrt(aa * aa + bb * bb);
    c[j] = aa / rr;
    sn[j] = -bb / rr;
    Hj[j] = rr;
    Hj[j + 1] = 0;
    e[j + 1] = sn[j] * e[j];
    e[j] = c[j] * e[j];
    const double en = fabs((double)e[j + 1]);
    q.relres = en / q.nrm_b;
    q.jn = j + 1;
    if (bad || !(en == en)) {
        q.bad = bad | ST_DIVZERO;
        q.active = 0;
    } else if (en <= q.crit) {
        q.conv = 1;
        q.active = 0;
    } else if (j + 1 < m) {
        atomicAdd(&info->n_active, 1);
    }
}

// V_{j+1} = w / H_{j+1,j} (Scal, gmres.hpp:64) for the pairs that took step j
template <typename T, int R>
__global__ void k_fscal(const FTile *__restrict__ tiles, int j, const FPair *__restrict__ pairs,
                        const T *__restrict__ ascal, T *__restrict__ w) {
    pdl_trigger();
    pdl_wait();
    const FTile t = tiles[blockIdx.x];
    T a[R];
    bool act[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int p = t.sys * R + r;
        act[r] = pairs[p].jn == j + 1 && !pairs[p].bad;
        a[r] = act[r] ? ascal[p] : T(1);
    }
    for (int i = t.row0 + threadIdx.x; i < t.row1; i += blockDim.x) {
        T wv[R];
        fld<T, R, 1>(w, i, wv);
#pragma unroll
        for (int r = 0; r < R; r++)
            if (act[r]) wv[r] *= a[r];
        fst<T, R>(w, i, wv);
    }
}

__global__ void k_finfo_reset(FInfo *info) {
    pdl_trigger();
    pdl_wait();
    info->n_active = 0;
}

// blas2::Trsv (blas2.hpp:25-34) per pair
template <typename T>
__global__ void k_ftrsv(int P, int m, const FPair *__restrict__ pairs, const T *Hall, const T *eall, T *yall) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    const FPair &q = pairs[p];
    const int jn = q.jn;
    if (jn == 0 || q.bad) return;
    const T *H = Hall + (size_t)p * (m + 1) * m;
    const T *e = eall + (size_t)p * (m + 1);
    T *y = yall + (size_t)p * m;
    for (int i = jn - 1; i >= 0; i--) {
        T t = e[i];
        for (int k = jn - 1; k > i; k--) t -= H[(size_t)k * (m + 1) + i] * y[k];
        y[i] = t / H[(size_t)i * (m + 1) + i];
    }
}

// x += y_k Z_k, k = 0 .. jn-1 in order (Axpy<double>, or AxpyFD for float:
// x += (double)(y_k * z), blas1.hpp:98-101)
template <typename T, int R>
__global__ void __launch_bounds__(kFThreads)
k_fxupd(const FTile *__restrict__ tiles, int m, size_t vstride, const FPair *__restrict__ pairs,
        const T *__restrict__ yall, const T *__restrict__ Z, double *__restrict__ x) {
    const FTile t = tiles[blockIdx.x / kFTileSub];
    __shared__ T sy[R][64];
    __shared__ int sjn[R];
    if (threadIdx.x < R) {
        const FPair &q = pairs[t.sys * R + threadIdx.x];
        sjn[threadIdx.x] = q.jn > 0 && !q.bad ? q.jn : 0;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < R * m; idx += blockDim.x) {
        const int r = idx / m, k = idx % m;
        sy[r][k] = k < sjn[r] ? yall[(size_t)(t.sys * R + r) * m + k] : T(0);
    }
    __syncthreads();
    const int i = t.row0 + (blockIdx.x % kFTileSub) * kFThreads + threadIdx.x;
    if (i >= t.row1) return;
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int jn = sjn[r];
        if (!jn) continue;
        double xi = x[(size_t)i * R + r];
        for (int k = 0; k < jn; k++) xi += (double)(sy[r][k] * __ldg(Z + (size_t)k * vstride + (size_t)i * R + r));
        x[(size_t)i * R + r] = xi;
    }
}

// r = b - A x in FP64, every right-hand side (irsolver.hpp:32-33)
template <int R>
__global__ void k_fresid(int n, const int *__restrict__ rptr, const int *__restrict__ cind,
                         const double *__restrict__ val, const double *__restrict__ x, const double *__restrict__ b,
                         double *__restrict__ rv) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    double acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) acc[r] = 0.0;
    const int e1 = rptr[row + 1];
    for (int j0 = rptr[row]; j0 < e1; j0 += 8) {  // eight entries' loads issued together, summed in order
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
    for (int r = 0; r < R; r++) rv[(size_t)row * R + r] = b[(size_t)row * R + r] - acc[r];
}

// per-tile sums of squares, then per pair over its tiles (fixed order)
template <int R>
__global__ void __launch_bounds__(kFThreads) k_fnorm_part(const FTile *__restrict__ tiles, const double *__restrict__ v,
                                                          double *__restrict__ part) {
    __shared__ double sh[kFThreads / 32][R];
    const FTile t = tiles[blockIdx.x];
    double s[R];
#pragma unroll
    for (int r = 0; r < R; r++) s[r] = 0;
    for (int i = t.row0 + threadIdx.x; i < t.row1; i += kFThreads)
#pragma unroll
        for (int r = 0; r < R; r++) {
            const double q = v[(size_t)i * R + r];
            s[r] += q * q;
        }
    block_sum_all<double, R>(s, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int r = 0; r < R; r++) part[(size_t)blockIdx.x * R + r] = s[r];
}

// one warp per pair, lanes over the system's tiles, a fixed shuffle tree
__global__ void k_fnorm_fin(int S, int R, const int *__restrict__ tile_ptr, const double *__restrict__ part,
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

template <typename T>
struct DevFMat {
    FMat<T> d{};
    int group = 1;
    int *rp = nullptr, *ci = nullptr;
    T *va = nullptr;
    int64_t nnz = 0;
    void up(const BatchCsrT<T> &M) {
        rp = dupload(M.rptr);
        ci = dupload(M.cind);
        va = dupload(M.val);
        nnz = M.nnz();
        d = FMat<T>{M.n, rp, ci, va};
        group = pick_group(M.n ? (double)M.nnz() / M.n : 1.0);
    }
    void release() {
        dfree(rp); dfree(ci); dfree(va);
        rp = ci = nullptr;
        va = nullptr;
    }
};

template <typename T>
struct DevFLevel {
    int n_all = 0, n_smooth = 0;
    bool one_colour = false;  // LD is the diagonal alone (one colour): the sweep can be fused
    DevFMat<T> A, LD, U, P, R;
    int *colour_rows = nullptr;
    std::vector<int> colour_ptr;
    int packed = 1;  // 1: sweep over the colour-ordered pack, 0: over the CSR through the row lists
    int4 *items = nullptr;
    T *idinv = nullptr;
    int *ecol = nullptr;
    T *eval = nullptr;
};

template <int V>
using IC = std::integral_constant<int, V>;

}  // namespace

// --------------------------------------------------------------- the engine
class BatchFpEngine::Base {
  public:
    virtual ~Base() {}
    virtual void precondition(const void *in, void *out) = 0;
    virtual void solve(const KrylovParams &kp, const double *b, const double *nrm_b, double *x, BatchStats &st) = 0;
    virtual void autotune(int reps) = 0;
    virtual float time_vcycle(int reps) = 0;
    virtual int fused_sweeps(int set) = 0;
    virtual int depth() const = 0;
    virtual size_t rows() const = 0;
};

namespace {

template <typename T>
class FpImpl : public BatchFpEngine::Base {
  public:
    Ctx &c;
    std::shared_ptr<BatchHierarchy> h;
    int S, Rn, Dmax, smooth_iter, m = 0;
    size_t N0;
    std::vector<int> n_level;
    std::vector<DevFLevel<T>> lv;
    std::vector<T *> ee, xx, rr, tmp;
    bool fuse_jac = true;
    FLuDesc<T> *d_lu = nullptr;
    int nlu = 0;
    size_t lu_smem = 0;
    T *Lcat = nullptr, *Ucat = nullptr, *dcat = nullptr;
    DevCsr Af;
    std::vector<FTile> tiles_h;
    FTile *tiles = nullptr;
    int *tile_ptr = nullptr;
    int ntiles = 0;
    int dot_group = -1;
    // Krylov state
    T *V = nullptr, *Z = nullptr, *H = nullptr, *cs = nullptr, *sn = nullptr, *e = nullptr, *y = nullptr;
    T *part = nullptr, *ascal = nullptr;
    double *rvec = nullptr, *nrm = nullptr, *npart = nullptr;
    FPair *pairs = nullptr;
    FInfo *info_d = nullptr, *info_h = nullptr;
    std::vector<cudaGraphExec_t> graphs;
    std::vector<long long> graph_launches;
    CycleGraph cyc;
    bool graph_pdl = true;
    cudaGraphExec_t vc_graph = nullptr;
    const T *vc_in = nullptr;
    T *vc_out = nullptr;
    long long vc_launches = 0;

    FpImpl(Ctx &ctx, std::shared_ptr<BatchHierarchy> hh, int nrhs, int threads) : c(ctx), h(hh) {
        S = h->S;
        Rn = nrhs;
        Dmax = h->Dmax;
        smooth_iter = h->sm.iter;
        n_level = h->n_level;
        N0 = (size_t)n_level[0];
        const BatchFp<T> F = build_batch_fp<T>(*h, threads);
        lv.resize(Dmax);
        for (int l = 0; l < Dmax; l++) {
            const BatchLevelT<T> &L = F.lv[l];
            DevFLevel<T> &d = lv[l];
            d.n_all = h->lv[l].n_all;
            d.n_smooth = h->lv[l].n_smooth;
            d.A.up(L.A);
            d.LD.up(L.LD);
            d.U.up(L.U);
            d.P.up(L.P);
            d.R.up(L.R);
            d.LD.group = pick_group(L.LD.n ? (double)(L.LD.nnz() - L.LD.n) / L.LD.n : 1.0);
            d.colour_rows = dupload(L.colour_rows);
            d.colour_ptr = L.colour_ptr;
            d.one_colour = L.LD.n > 0 && L.LD.nnz() == L.LD.n;
            for (int i = 0; d.one_colour && i < L.LD.n; i++)
                d.one_colour = L.LD.rptr[i] == i && L.LD.cind[i] == i;
            pack(L, d);
        }
        auto vec = [&](int rows) { return (T *)dmalloc(sizeof(T) * (size_t)std::max(rows, 1) * Rn); };
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
        std::vector<FLuDesc<T>> desc;
        std::vector<T> Lh, Uh, dh;
        size_t maxn = 0;
        for (const BatchLUT<T> &lu : F.lu) {
            FLuDesc<T> d{};
            d.n = lu.n;
            d.sys = lu.sys;
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
        lu_smem = 2 * sizeof(T) * maxn * Rn;
        if (lu_smem > 227 * 1024) throw CudaError{"a coarsest level is too large for the batched FP LU kernel"};
        Lcat = dupload(Lh);
        Ucat = dupload(Uh);
        dcat = dupload(dh);
        d_lu = dupload(desc);
        Af = upload_csr_f64(h->Af);
        std::vector<int> tp(1, 0);
        for (int s = 0; s < S; s++) {
            const int off = h->offset[0][s], n = h->n_sys[s];
            for (int r0 = 0; r0 < n; r0 += kFTileRows)
                tiles_h.push_back(FTile{s, off + r0, off + std::min(n, r0 + kFTileRows), r0 == 0});
            tp.push_back((int)tiles_h.size());
        }
        ntiles = (int)tiles_h.size();
        tiles = dupload(tiles_h);
        tile_ptr = dupload(tp);
        rvec = (double *)dmalloc(sizeof(double) * N0 * Rn);
        nrm = (double *)dmalloc(sizeof(double) * (size_t)S * Rn);
        npart = (double *)dmalloc(sizeof(double) * (size_t)ntiles * Rn);
        pairs = (FPair *)dmalloc(sizeof(FPair) * (size_t)S * Rn);
        SAGB_CUDA(cudaMemset(pairs, 0, sizeof(FPair) * (size_t)S * Rn));
        ascal = (T *)dmalloc(sizeof(T) * (size_t)S * Rn);
        info_d = (FInfo *)dmalloc(sizeof(FInfo));
        SAGB_CUDA(cudaMallocHost(&info_h, sizeof(FInfo)));
        SAGB_CUDA(cudaFuncSetAttribute(k_flu<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        SAGB_CUDA(cudaFuncSetAttribute(k_flu<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        SAGB_CUDA(cudaFuncSetAttribute(k_flu<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    }

    // LD in colour-row order: items {row, first entry, entries, 0}, the
    // inverse diagonal per item, the strictly lower entries as columns and values
    void pack(const BatchLevelT<T> &L, DevFLevel<T> &d) {
        const size_t nrows = L.colour_rows.size();
        std::vector<int4> items(nrows);
        std::vector<T> idv(nrows);
        std::vector<int> ec;
        std::vector<T> ev;
        ec.reserve(L.LD.nnz());
        ev.reserve(L.LD.nnz());
        for (size_t k = 0; k < nrows; k++) {
            const int row = L.colour_rows[k];
            const int a = L.LD.rptr[row], b = L.LD.rptr[row + 1] - 1;  // the last entry is dinv
            if (ec.size() > (size_t)INT32_MAX - (size_t)(b - a)) {
                d.packed = 0;
                return;
            }
            items[k] = make_int4(row, (int)ec.size(), b - a, 0);
            idv[k] = L.LD.val[b];
            for (int j = a; j < b; j++) {
                ec.push_back(L.LD.cind[j]);
                ev.push_back(L.LD.val[j]);
            }
        }
        d.items = dupload(items);
        d.idinv = dupload(idv);
        d.ecol = dupload(ec);
        d.eval = dupload(ev);
    }

    void free_krylov() {
        dfree(V); dfree(Z); dfree(H); dfree(cs); dfree(sn); dfree(e); dfree(y); dfree(part);
        V = Z = H = cs = sn = e = y = part = nullptr;
        clear_graphs();
    }
    void clear_graphs() {
        cyc.clear();
        for (auto &g : graphs)
            if (g) cudaGraphExecDestroy(g);
        graphs.clear();
        graph_launches.clear();
        if (vc_graph) cudaGraphExecDestroy(vc_graph);
        vc_graph = nullptr;
    }

    ~FpImpl() override {
        free_krylov();
        for (auto &d : lv) {
            d.A.release(); d.LD.release(); d.U.release(); d.P.release(); d.R.release();
            dfree(d.colour_rows); dfree(d.items); dfree(d.idinv); dfree(d.ecol); dfree(d.eval);
        }
        for (auto p : ee) dfree(p);
        for (auto p : xx) dfree(p);
        for (auto p : rr) dfree(p);
        for (auto p : tmp) dfree(p);
        dfree(d_lu); dfree(Lcat); dfree(Ucat); dfree(dcat);
        Af.release();
        dfree(tiles); dfree(tile_ptr); dfree(rvec); dfree(nrm); dfree(npart); dfree(pairs); dfree(ascal);
        dfree(info_d);
        if (info_h) cudaFreeHost(info_h);
    }

    int depth() const override { return Dmax; }
    size_t rows() const override { return N0; }

    // ------------------------------------------------------- dispatch
    template <typename F>
    void by_r(F &&f) {
        if (Rn == 4) f(IC<4>());
        else if (Rn == 2) f(IC<2>());
        else f(IC<1>());
    }
    template <typename F>
    static void by_g(int G, F &&f) {
        switch (G) {
            case 1: f(IC<1>()); break;
            case 2: f(IC<2>()); break;
            case 4: f(IC<4>()); break;
            case 8: f(IC<8>()); break;
            case 16: f(IC<16>()); break;
            default: f(IC<32>()); break;
        }
    }
    template <typename... KArgs, typename... Args>
    void launch(void (*k)(KArgs...), int grid, int block, size_t smem, Args... args) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3(block);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = c.stream;
        cudaLaunchAttribute at[1];
        int na = 0;
        if (c.use_pdl) {
            at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            at[na].val.programmaticStreamSerializationAllowed = 1;
            na++;
        }
        cfg.attrs = at;
        cfg.numAttrs = na;
        SAGB_CUDA(cudaLaunchKernelEx(&cfg, k, args...));
        c.launches++;
    }

    void spmv(const DevFMat<T> &M, const T *x, T *y, int mode, const T *z, int jac = 0, FJac<T> J = FJac<T>{}) {
        if (M.d.n == 0) return;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            by_g(M.group, [&](auto GG) {
                constexpr int G = decltype(GG)::value;
                const long long thr = (long long)M.d.n * G;
                launch(k_fspmv<T, R, G>, (int)((thr + kFThreads - 1) / kFThreads), kFThreads, 0, M.d, x, y, z, mode,
                       jac, J);
            });
        });
    }

    void sweep(int l, const T *in, T *out) {
        DevFLevel<T> &L = lv[l];
        const int nc = (int)L.colour_ptr.size() - 1;
        for (int k = 0; k < nc; k++) {
            const int a = L.colour_ptr[k], b = L.colour_ptr[k + 1];
            if (b == a) continue;
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                by_g(L.LD.group, [&](auto GG) {
                    constexpr int G = decltype(GG)::value;
                    const int blocks = (int)(((long long)(b - a) * G + kFThreads - 1) / kFThreads);
                    if (L.packed && L.items)
                        launch(k_fcolour_packed<T, R, G>, blocks, kFThreads, 0, a, b, (const int4 *)L.items,
                               (const T *)L.idinv, (const int *)L.ecol, (const T *)L.eval, in, out);
                    else
                        launch(k_fcolour<T, R, G>, blocks, kFThreads, 0, b - a, (const int *)(L.colour_rows + a),
                               L.LD.d, in, out);
                });
            });
        }
    }

    // SOR::Smooth in colour order (stationary.hpp:239-262): pre-smoothing
    // out = LD^-1 in; post-smoothing tmp = in - U out, out = LD^-1 tmp
    void smooth(int l, const T *in, T *out, bool inited) {
        int k0 = 0;
        if (!inited) {
            sweep(l, in, out);
            k0 = 1;
        }
        for (int k = k0; k < smooth_iter; k++) {
            spmv(lv[l].U, out, tmp[l], SPMV_RESID, in);
            sweep(l, tmp[l], out);
        }
    }

    void lu() {
        if (!nlu) return;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            launch(k_flu<T, R>, nlu, kFLuThreads, lu_smem, (const FLuDesc<T> *)d_lu, (const T *)Lcat,
                   (const T *)Ucat, (const T *)dcat);
        });
    }

    // one-colour levels below the finest with their sweeps fused into the
    // neighbouring SpMVs (pre: the restriction producing e; post: the U
    // residual, result in tmp, which the interpolation above reads)
    bool fused_pre(int l) const { return fuse_jac && smooth_iter == 1 && l >= 1 && l < Dmax && lv[l].one_colour; }
    bool fused_post(int l) const { return fused_pre(l) && lv[l].n_all == lv[l].n_smooth; }
    FJac<T> jac_of(int l, T *x2 = nullptr) const { return FJac<T>{lv[l].LD.d.val, lv[l].LD.d.n, x2}; }
    int fused_sweeps(int set) override {
        if (set >= 0) {
            fuse_jac = set > 0;
            clear_graphs();
        }
        int n = 0;
        for (int l = 0; l < Dmax; l++) n += fused_pre(l);
        return n;
    }

    // dfAMG::Precondition (INTAMG.hpp:86-134) for the whole batch
    void vcycle(const T *in, T *out) {
        for (int l = 0; l < Dmax; l++) {
            const T *e_l = l == 0 ? in : ee[l];
            T *x_l = l == 0 ? out : xx[l];
            if (!fused_pre(l)) smooth(l, e_l, x_l, false);
            spmv(lv[l].A, x_l, rr[l], SPMV_RESID, e_l);
            if (fused_pre(l + 1)) spmv(lv[l].R, rr[l], ee[l + 1], SPMV_SET, nullptr, 1, jac_of(l + 1, xx[l + 1]));
            else spmv(lv[l].R, rr[l], ee[l + 1], SPMV_SET, nullptr);
        }
        lu();
        for (int l = Dmax - 1; l >= 0; l--) {
            const T *e_l = l == 0 ? in : ee[l];
            T *x_l = l == 0 ? out : xx[l];
            spmv(lv[l].P, fused_post(l + 1) ? tmp[l + 1] : xx[l + 1], x_l, SPMV_ADD, nullptr);
            if (fused_post(l)) spmv(lv[l].U, x_l, tmp[l], SPMV_RESID, e_l, 2, jac_of(l));
            else smooth(l, e_l, x_l, true);
        }
    }

    template <typename F>
    void captured(cudaGraphExec_t &ge, long long &count, F &&body) {
        cudaGraph_t g = nullptr;
        const long long before = c.launches;
        SAGB_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        try {
            body();
        } catch (...) {
            cudaStreamEndCapture(c.stream, &g);
            if (g) cudaGraphDestroy(g);
            c.launches = before;
            throw;
        }
        SAGB_CUDA(cudaStreamEndCapture(c.stream, &g));
        SAGB_CUDA(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
        count = c.launches - before;
        c.launches = before;
    }

    void precondition(const void *in_, void *out_) override {
        const T *in = (const T *)in_;
        T *out = (T *)out_;
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
            captured(vc_graph, vc_launches, [&] { vcycle(in, out); });
            vc_in = in;
            vc_out = out;
        }
        SAGB_CUDA(cudaGraphLaunch(vc_graph, c.stream));
        c.launches += vc_launches;
    }

    // ----------------------------------------------------------- Krylov
    void ensure_krylov(int mm) {
        if (mm == m && V) return;
        free_krylov();
        m = mm;
        const size_t P = (size_t)S * Rn;
        V = (T *)dmalloc(sizeof(T) * N0 * Rn * (m + 1));
        Z = (T *)dmalloc(sizeof(T) * N0 * Rn * (m + 1));
        H = (T *)dmalloc(sizeof(T) * P * (m + 1) * m);
        cs = (T *)dmalloc(sizeof(T) * P * m);
        sn = (T *)dmalloc(sizeof(T) * P * m);
        e = (T *)dmalloc(sizeof(T) * P * (m + 1));
        y = (T *)dmalloc(sizeof(T) * P * m);
        part = (T *)dmalloc(sizeof(T) * (size_t)(m + 1) * ntiles * Rn);
        SAGB_CUDA(cudaMemset(H, 0, sizeof(T) * P * (m + 1) * m));
        SAGB_CUDA(cudaMemset(V, 0, sizeof(T) * N0 * Rn * (m + 1)));
        SAGB_CUDA(cudaMemset(Z, 0, sizeof(T) * N0 * Rn * (m + 1)));
    }

    void pair_norms(const double *v) {
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            k_fnorm_part<R><<<ntiles, kFThreads, 0, c.stream>>>(tiles, v, npart);
        });
        const int P = S * Rn;
        k_fnorm_fin<<<(P + 7) / 8, 256, 0, c.stream>>>(S, Rn, tile_ptr, npart, nrm);
        c.launches += 2;
    }

    void residual(const double *b, const double *x) {
        const int n = (int)N0;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            k_fresid<R><<<(n + 127) / 128, 128, 0, c.stream>>>(n, Af.rptr, Af.cind, (const double *)Af.val, x, b,
                                                               rvec);
        });
        c.launches++;
        pair_norms(rvec);
    }

    void spmv_dot(const T *z, T *w, const T *v0) {
        const DevFMat<T> &A0 = lv[0].A;
        const int g = dot_group > 0 ? dot_group : A0.group;
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            by_g(g, [&](auto GG) {
                constexpr int G = decltype(GG)::value;
                launch(k_fspmv_dot<T, R, G>, ntiles, kFThreads, 0, (const FTile *)tiles, A0.d, z, w, v0, part);
            });
        });
    }

    void arnoldi_step(int j, bool d2h = true, cudaGraphConditionalHandle next = 0, bool has_next = false) {
        const int P = S * Rn;
        const size_t vs = N0 * Rn;
        T *Vj = V + (size_t)j * vs, *Zj = Z + (size_t)j * vs, *w = V + (size_t)(j + 1) * vs;
        launch(k_finfo_reset, 1, 1, 0, info_d);
        vcycle(Vj, Zj);
        spmv_dot(Zj, w, V);
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            for (int k = 0; k <= j; k++) {
                if (k < j)
                    launch(k_fmgs<T, R, false>, ntiles, kFThreads, 0, (const FTile *)tiles, (const int *)tile_ptr,
                           ntiles, k, j, m, vs, (const T *)V, w, (const FPair *)pairs, part, H);
                else
                    launch(k_fmgs<T, R, true>, ntiles, kFThreads, 0, (const FTile *)tiles, (const int *)tile_ptr,
                           ntiles, k, j, m, vs, (const T *)V, w, (const FPair *)pairs, part, H);
            }
        });
        launch(k_fgivens<T>, (P + 3) / 4, 128, 0, P, Rn, j, m, ntiles, (const int *)tile_ptr, pairs,
               (const T *)part, H, cs, sn, e, ascal, info_d);
        by_r([&](auto RR) {
            constexpr int R = decltype(RR)::value;
            launch(k_fscal<T, R>, ntiles, kFThreads, 0, (const FTile *)tiles, j, (const FPair *)pairs,
                   (const T *)ascal, w);
        });
        if (has_next) launch(k_cycle_next, 1, 32, 0, (const int *)&info_d->n_active, next);
        if (d2h) SAGB_CUDA(cudaMemcpyAsync(info_h, info_d, sizeof(FInfo), cudaMemcpyDeviceToHost, c.stream));
    }

    // the steps of one restart cycle as one graph gated on the device (see
    // cycle_graph.cuh), or step by step; true when the graph ran
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
            if (!graphs[j]) captured(graphs[j], graph_launches[j], [&] { arnoldi_step(j); });
            SAGB_CUDA(cudaGraphLaunch(graphs[j], c.stream));
            c.launches += graph_launches[j];
        }
        SAGB_CUDA(cudaStreamSynchronize(c.stream));
    }

    // Restarted::Solve per pair (irsolver.hpp:27-43), all pairs in lockstep
    void solve(const KrylovParams &kp, const double *b, const double *nrm_b, double *x, BatchStats &st) override {
        const int P = S * Rn;
        if (kp.m > 64) throw CudaError{"restart length above 64"};
        ensure_krylov(kp.m);
        st = BatchStats();
        st.iters.assign(P, 0);
        st.converged.assign(P, 0);
        st.fallbacks.assign(P, 0);
        st.final_bit.assign(P, 0);
        st.explicit_res.assign(P, 0.0);
        std::vector<FPair> hp(P);
        std::vector<double> nb(P), hn(P), prev(P, 0.0);
        std::vector<int> done(P, 0);
        SAGB_CUDA(cudaMemcpy(nb.data(), nrm_b, sizeof(double) * P, cudaMemcpyDefault));
        for (int outer = 0; outer < kp.max_outer; outer++) {
            residual(b, x);
            SAGB_CUDA(cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * P, cudaMemcpyDeviceToHost, c.stream));
            SAGB_CUDA(cudaStreamSynchronize(c.stream));
            int ncycle = 0;
            for (int p = 0; p < P; p++) {
                hp[p] = FPair();
                hp[p].nrm_b = nb[p];
                if (done[p]) continue;
                const double nr = hn[p];
                st.explicit_res[p] = nr / nb[p];
                if (kp.explicit_check && outer > 0 && nr <= kp.eps * nb[p]) {
                    done[p] = 1;
                    st.converged[p] = 1;
                    continue;
                }
                if (std::fabs(nr - prev[p]) / nr < 1.0e-8) {  // stagnation (irsolver.hpp:35)
                    done[p] = 1;
                    st.iters[p] = 0;
                    continue;
                }
                prev[p] = nr;
                hp[p].active = 1;
                ncycle++;
            }
            if (ncycle == 0) break;
            st.restarts++;
            SAGB_CUDA(cudaMemcpyAsync(pairs, hp.data(), sizeof(FPair) * P, cudaMemcpyHostToDevice, c.stream));
            k_fbegin<T><<<(P + 127) / 128, 128, 0, c.stream>>>(P, nrm, kp.eps, pairs, e, m);
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                k_fv0<T, R><<<ntiles * kFTileSub, kFThreads, 0, c.stream>>>(tiles, rvec, pairs, V);
            });
            c.launches += 2;
            const bool in_graph = cycle_steps();
            st.cycle_graphs += in_graph;
            k_ftrsv<T><<<(P + 127) / 128, 128, 0, c.stream>>>(P, m, pairs, H, e, y);
            by_r([&](auto RR) {
                constexpr int R = decltype(RR)::value;
                k_fxupd<T, R><<<ntiles * kFTileSub, kFThreads, 0, c.stream>>>(tiles, m, N0 * Rn, pairs, y, Z, x);
            });
            c.launches += 2;
            SAGB_CUDA(cudaMemcpyAsync(hp.data(), pairs, sizeof(FPair) * P, cudaMemcpyDeviceToHost, c.stream));
            SAGB_CUDA(cudaStreamSynchronize(c.stream));
            if (in_graph) {
                int steps = 0;
                for (int p = 0; p < P; p++) steps = std::max(steps, hp[p].jn);
                for (int j = 0; j < steps && j < (int)cyc.step_launches.size(); j++) c.launches += cyc.step_launches[j];
            }
            for (int p = 0; p < P; p++) {
                if (done[p] || !(hp[p].jn > 0)) continue;
                if (hp[p].bad) {
                    st.flags |= hp[p].bad;
                    done[p] = 1;
                    continue;
                }
                st.iters[p] += hp[p].jn;
                if (hp[p].conv && !kp.explicit_check) {
                    done[p] = 1;
                    st.converged[p] = 1;
                }
            }
        }
        residual(b, x);
        SAGB_CUDA(cudaMemcpyAsync(hn.data(), nrm, sizeof(double) * P, cudaMemcpyDeviceToHost, c.stream));
        SAGB_CUDA(cudaStreamSynchronize(c.stream));
        for (int p = 0; p < P; p++) {
            st.explicit_res[p] = hn[p] / nb[p];
            if (!done[p] && kp.explicit_check && hn[p] <= kp.eps * nb[p]) st.converged[p] = 1;
            if (!st.converged[p]) st.iters[p] = 0;
        }
    }

    // ----------------------------------------------------------- tuning
    template <typename F>
    float timed(F &&fn, int reps, cudaEvent_t e0, cudaEvent_t e1) {
        float ms = 1e30f;
        const int n = std::max(reps, 5);
        if (c.use_graphs) {
            cudaGraphExec_t ge;
            long long cnt = 0;
            captured(ge, cnt, [&] {
                for (int k = 0; k < n; k++) fn();
            });
            SAGB_CUDA(cudaGraphLaunch(ge, c.stream));
            for (int t = 0; t < 3; t++) {
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
            const long long before = c.launches;
            fn();
            SAGB_CUDA(cudaEventRecord(e0, c.stream));
            for (int k = 0; k < n; k++) fn();
            SAGB_CUDA(cudaEventRecord(e1, c.stream));
            SAGB_CUDA(cudaEventSynchronize(e1));
            SAGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            c.launches = before;
        }
        return ms / n;
    }

    // lanes per row of every operator and the sweep form of every level,
    // each timed as the solver runs it; results do not depend on the choice
    // beyond the order of FP sums inside a row
    void autotune(int reps) override {
        cudaEvent_t e0, e1;
        SAGB_CUDA(cudaEventCreate(&e0));
        SAGB_CUDA(cudaEventCreate(&e1));
        T *xa = (T *)dmalloc(sizeof(T) * N0 * Rn), *xb = (T *)dmalloc(sizeof(T) * N0 * Rn);
        SAGB_CUDA(cudaMemset(xa, 0, sizeof(T) * N0 * Rn));
        SAGB_CUDA(cudaMemset(xb, 0, sizeof(T) * N0 * Rn));
        const int cand[] = {1, 2, 4, 8, 16, 32};
        for (int l = 0; l < Dmax; l++) {
            DevFLevel<T> &L = lv[l];
            for (int op = 0; op < 5; op++) {
                DevFMat<T> *M = op == 0 ? &L.A : op == 1 ? &L.LD : op == 2 ? &L.U : op == 3 ? &L.P : &L.R;
                if (M->d.n == 0) continue;
                float best = 1e30f;
                int bestg = M->group, bestf = L.packed;
                const int nform = op == 1 && L.items ? 2 : 1;
                for (int f = 0; f < nform; f++) {
                    if (op == 1) L.packed = nform == 2 ? f : 0;
                    for (int g : cand) {
                        M->group = g;
                        const float ms = timed([&] {
                            if (op == 1) sweep(l, xa, xb);
                            else spmv(*M, xa, xb, SPMV_SET, nullptr);
                        }, reps, e0, e1);
                        if (ms < best) {
                            best = ms;
                            bestg = g;
                            bestf = op == 1 ? L.packed : bestf;
                        }
                    }
                }
                M->group = bestg;
                if (op == 1) L.packed = bestf;
            }
        }
        {
            ensure_krylov(std::max(m, 1));
            float best = 1e30f;
            int bestg = lv[0].A.group;
            for (int g : cand) {
                dot_group = g;
                const float ms = timed([&] { spmv_dot(xa, xb, xa); }, reps, e0, e1);
                if (ms < best) {
                    best = ms;
                    bestg = g;
                }
            }
            dot_group = bestg;
        }
        SAGB_CUDA(cudaStreamSynchronize(c.stream));
        dfree(xa);
        dfree(xb);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        clear_graphs();
    }

    float time_vcycle(int reps) override {
        cudaEvent_t e0, e1;
        SAGB_CUDA(cudaEventCreate(&e0));
        SAGB_CUDA(cudaEventCreate(&e1));
        T *xa = (T *)dmalloc(sizeof(T) * N0 * Rn), *xb = (T *)dmalloc(sizeof(T) * N0 * Rn);
        SAGB_CUDA(cudaMemset(xa, 0, sizeof(T) * N0 * Rn));
        const float ms = timed([&] { vcycle(xa, xb); }, reps, e0, e1);
        dfree(xa);
        dfree(xb);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return ms;
    }
};

}  // namespace

BatchFpEngine::BatchFpEngine(Ctx &c, std::shared_ptr<BatchHierarchy> h, int vt, int nrhs, int threads) : vt_(vt) {
    if (vt == VT_F64) impl_ = std::make_unique<FpImpl<double>>(c, h, nrhs, threads);
    else if (vt == VT_F32) impl_ = std::make_unique<FpImpl<float>>(c, h, nrhs, threads);
    else throw CudaError{"the floating-point batch takes SA_F64 or SA_F32"};
}
BatchFpEngine::~BatchFpEngine() = default;
void BatchFpEngine::precondition(const void *in, void *out) { impl_->precondition(in, out); }
void BatchFpEngine::solve(const KrylovParams &kp, const double *b, const double *nrm_b, double *x, BatchStats &st) {
    impl_->solve(kp, b, nrm_b, x, st);
    last_cycle_graphs_ = st.cycle_graphs;
}
void BatchFpEngine::autotune(int reps) { impl_->autotune(reps); }
float BatchFpEngine::time_vcycle(int reps) { return impl_->time_vcycle(reps); }
int BatchFpEngine::fused_sweeps(int set) { return impl_->fused_sweeps(set); }
int BatchFpEngine::depth() const { return impl_->depth(); }
size_t BatchFpEngine::rows() const { return impl_->rows(); }

}  // namespace sagb
