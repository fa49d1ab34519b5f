// GPU Ruge-Stueben setup: the levels of helper::multigrid::get_amg_set
// (helper_multigrid.hpp:34-63) with the strength split, both transposes, the
// direct interpolation and the two products of the Galerkin operator on the
// device; the greedy C/F selection (first_pass, second_pass), a sequential
// bucket algorithm, stays on the host.
//
// Every value equals the host setup's bit for bit: each FP64 operation is the
// host's operation in the host's order, written with the round-to-nearest
// intrinsics so that the compiler cannot contract a multiply and an add, and
// every output row is ordered as the host orders it.
//
//   strength        one thread a row: the row maximum, theta * max, the split
//   transposes      counts, prefix sums, scattered fill, then each row sorted
//                   by column (the host fills rows in increasing source order)
//   interpolation   one thread a fine row: the weak-row sum, sum_{k in C_i} a_mk
//                   by the host's merge, then w_ij in the host's order
//   products        C[:, c] = sum_k right[k, c] * left[:, k] in k order, one
//                   team (a warp, or a CTA for long columns) a column: a shared
//                   hash table keyed by row accumulates y + alpha * x in k
//                   order (the rows of one left column are distinct, so no two
//                   lanes of a step touch one entry), then the nonzero entries
//                   are ranked by row; the longest columns keep their table
//                   in global memory (one table per CTA)
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../host/amg_setup.hpp"
#include "../sagb_internal.hpp"
#include "common.cuh"

namespace sagb {
namespace {

constexpr int kRsThreads = 256;

struct DMat {  // FP64 CSR (or compressed columns) on the device
    int n = 0, m = 0;
    long long nnz = 0;
    int *rptr = nullptr, *cind = nullptr;
    double *val = nullptr;
    void release() {
        dfree(rptr);
        dfree(cind);
        dfree(val);
        rptr = cind = nullptr;
        val = nullptr;
    }
};

template <typename T>
T *dnew(size_t n) {
    return (T *)dmalloc(sizeof(T) * std::max<size_t>(n, 1));
}
template <typename T>
void up(Ctx &c, T *d, const T *h, size_t n) {
    if (n) SAGB_CUDA(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, c.stream));
}
template <typename T>
void down(Ctx &c, T *h, const T *d, size_t n) {
    if (n) SAGB_CUDA(cudaMemcpyAsync(h, d, sizeof(T) * n, cudaMemcpyDeviceToHost, c.stream));
}
void sync(Ctx &c) { SAGB_CUDA(cudaStreamSynchronize(c.stream)); }
int blocks_for(long long n) { return (int)std::max<long long>(1, (n + kRsThreads - 1) / kRsThreads); }

// row pointers from per-row counts (host prefix sum; the setup is not latency bound)
std::vector<int> scan_counts(Ctx &c, const int *d_cnt, int n, int *d_rptr) {
    std::vector<int> cnt(n), rp(n + 1, 0);
    down(c, cnt.data(), d_cnt, n);
    sync(c);
    long long acc = 0;
    for (int i = 0; i < n; i++) {
        acc += cnt[i];
        if (acc > INT_MAX) throw SetupError{"GPU setup: more than 2^31 entries in one operator"};
        rp[i + 1] = (int)acc;
    }
    up(c, d_rptr, rp.data(), n + 1);
    sync(c);
    return rp;
}

DMat upload(Ctx &c, const CsrD &A) {
    DMat d;
    d.n = A.n;
    d.m = A.m;
    d.nnz = A.nnz();
    d.rptr = dnew<int>(A.n + 1);
    d.cind = dnew<int>(d.nnz);
    d.val = dnew<double>(d.nnz);
    up(c, d.rptr, A.rptr.data(), A.n + 1);
    up(c, d.cind, A.cind.data(), d.nnz);
    up(c, d.val, A.val.data(), d.nnz);
    sync(c);
    return d;
}

CsrD download(Ctx &c, const DMat &d) {
    CsrD A;
    A.n = d.n;
    A.m = d.m;
    A.rptr.resize(d.n + 1);
    A.cind.resize(d.nnz);
    A.val.resize(d.nnz);
    down(c, A.rptr.data(), d.rptr, d.n + 1);
    down(c, A.cind.data(), d.cind, d.nnz);
    down(c, A.val.data(), d.val, d.nnz);
    sync(c);
    return A;
}

// ------------------------------------------------------------------ strength
// get_strong_weak_set (helper_multigrid.hpp:67-108)
__global__ void k_rs_strong_count(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                  const double *__restrict__ v, double theta, double *__restrict__ thr,
                                  int *__restrict__ scnt, int *__restrict__ wcnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double mx = 0;
    for (int j = rp[i]; j < rp[i + 1]; j++)
        if (ci[j] != i && fabs(v[j]) > mx) mx = fabs(v[j]);
    const double t = __dmul_rn(theta, mx);
    int s = 0;
    for (int j = rp[i]; j < rp[i + 1]; j++)
        if (ci[j] != i && fabs(v[j]) >= t) s++;
    thr[i] = t;
    scnt[i] = s;
    wcnt[i] = rp[i + 1] - rp[i] - s;
}

__global__ void k_rs_strong_fill(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                                 const double *__restrict__ v, const double *__restrict__ thr,
                                 const int *__restrict__ srp, int *__restrict__ sci, double *__restrict__ sv,
                                 const int *__restrict__ wrp, int *__restrict__ wci, double *__restrict__ wv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int a = srp[i], b = wrp[i];
    const double t = thr[i];
    for (int j = rp[i]; j < rp[i + 1]; j++) {
        if (ci[j] != i && fabs(v[j]) >= t) {
            sci[a] = ci[j];
            sv[a++] = v[j];
        } else {
            wci[b] = ci[j];
            wv[b++] = v[j];
        }
    }
}

// ---------------------------------------------------------------- transposes
__global__ void k_rs_count_cols(long long nnz, const int *__restrict__ ci, int *__restrict__ cnt) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < nnz) atomicAdd(cnt + ci[e], 1);
}

__global__ void k_rs_tr_fill(int n, const int *__restrict__ rp, const int *__restrict__ ci,
                             const double *__restrict__ v, int *__restrict__ cursor, int *__restrict__ tci,
                             double *__restrict__ tv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int j = rp[i]; j < rp[i + 1]; j++) {
        const int p = atomicAdd(cursor + ci[j], 1);
        tci[p] = i;
        if (v) tv[p] = v[j];
    }
}

// each row ordered by column (columns of a row are distinct)
__global__ void k_rs_sort_rows(int n, const int *__restrict__ rp, int *__restrict__ ci, double *__restrict__ v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int a = rp[i] + 1; a < rp[i + 1]; a++) {
        const int key = ci[a];
        const double kv = v ? v[a] : 0.0;
        int b = a - 1;
        while (b >= rp[i] && ci[b] > key) {
            ci[b + 1] = ci[b];
            if (v) v[b + 1] = v[b];
            b--;
        }
        ci[b + 1] = key;
        if (v) v[b + 1] = kv;
    }
}

// rows x cols (n x m) -> m x n, rows in increasing source order
DMat transpose(Ctx &c, const DMat &A, bool values) {
    DMat T;
    T.n = A.m;
    T.m = A.n;
    T.nnz = A.nnz;
    T.rptr = dnew<int>(T.n + 1);
    T.cind = dnew<int>(T.nnz);
    T.val = values ? dnew<double>(T.nnz) : nullptr;
    int *cnt = dnew<int>(T.n);
    SAGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * std::max(T.n, 1), c.stream));
    if (A.nnz) k_rs_count_cols<<<blocks_for(A.nnz), kRsThreads, 0, c.stream>>>(A.nnz, A.cind, cnt);
    scan_counts(c, cnt, T.n, T.rptr);
    SAGB_CUDA(cudaMemcpyAsync(cnt, T.rptr, sizeof(int) * T.n, cudaMemcpyDeviceToDevice, c.stream));
    if (A.n) k_rs_tr_fill<<<blocks_for(A.n), kRsThreads, 0, c.stream>>>(A.n, A.rptr, A.cind, values ? A.val : nullptr,
                                                                      cnt, T.cind, T.val);
    if (T.n) k_rs_sort_rows<<<blocks_for(T.n), kRsThreads, 0, c.stream>>>(T.n, T.rptr, T.cind, T.val);
    SAGB_CUDA(cudaGetLastError());
    sync(c);
    dfree(cnt);
    return T;
}

// ------------------------------------------------------------- interpolation
// sepalate_strong_to_coarse_fine + get_interpolation_matrix
// (helper_multigrid.hpp:419-532), the host's interpolation() step for step.
// part: the S-entry indices of row i, strong coarse ones first (ncs of them),
// then strong fine ones, each in row order.
__global__ void k_rs_interp(int n, const int *__restrict__ Arp, const int *__restrict__ Aci,
                            const double *__restrict__ Av, const int *__restrict__ Srp, const int *__restrict__ Sci,
                            const double *__restrict__ Sv, const int *__restrict__ Wrp,
                            const double *__restrict__ Wv, const int *__restrict__ isc, const int *__restrict__ colmap,
                            const int *__restrict__ ncs_row, const int *__restrict__ part,
                            const long long *__restrict__ amj_off, double *__restrict__ amj_all,
                            double *__restrict__ amk_all, const int *__restrict__ Prp, int *__restrict__ Pci,
                            double *__restrict__ Pv, unsigned *__restrict__ warn_row,
                            int *__restrict__ first_stop) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (isc[i]) {
        Pci[Prp[i]] = colmap[i];
        Pv[Prp[i]] = 1.0;
        return;
    }
    const int s0 = Srp[i], ncs = ncs_row[i], ncf = Srp[i + 1] - s0 - ncs;
    double deno = 0;
    for (int j = Wrp[i]; j < Wrp[i + 1]; j++) deno = __dadd_rn(deno, Wv[j]);
    double *amj = amj_all + amj_off[i];
    double *amk_m = amk_all + s0;
    for (long long t = 0; t < (long long)ncf * ncs; t++) amj[t] = 0.0;
    for (int q = 0; q < ncf && ncs > 0; q++) {
        const int mrow = Sci[part[s0 + ncs + q]];
        double amk = 0;
        bool hit = false;
        int a = Arp[mrow], k = 0;
        while (a < Arp[mrow + 1] && k < ncs) {
            const int ck = Sci[part[s0 + k]];
            if (Aci[a] < ck) {
                a++;
            } else if (Aci[a] == ck) {
                amk = __dadd_rn(amk, Av[a]);
                amj[(long long)q * ncs + k] = Av[a];
                hit = true;
                a++;
                k++;
            } else {
                k++;
            }
        }
        if (amk == 0) {
            if (hit) {
                warn_row[i] += (unsigned)ncs;  // "1 amk = 0" once per (j, m) pair
                amk = 0.00001;
            } else {
                atomicMin(first_stop, i);  // "2 amk = 0": the setup stops at the first such row
                return;
            }
        }
        amk_m[q] = amk;
    }
    for (int k = 0; k < ncs; k++) {
        const int e = part[s0 + k];
        double aij = Sv[e];
        for (int q = 0; q < ncf; q++) {
            const double vf = Sv[part[s0 + ncs + q]];
            aij = __dadd_rn(aij, __ddiv_rn(__dmul_rn(vf, amj[(long long)q * ncs + k]), amk_m[q]));
        }
        Pci[Prp[i] + k] = colmap[Sci[e]];
        Pv[Prp[i] + k] = __ddiv_rn(-aij, deno);
    }
}

// ------------------------------------------------------------------ products
__global__ void k_sp_bound(int ncols, const int *__restrict__ rp, const int *__restrict__ ri,
                           const int *__restrict__ lp, long long *__restrict__ bound) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    long long b = 0;
    for (int k = rp[c]; k < rp[c + 1]; k++) b += lp[ri[k] + 1] - lp[ri[k]];
    bound[c] = b;
}

template <int TEAM>
__device__ __forceinline__ void team_sync() {
    if (TEAM == 32) __syncwarp();
    else __syncthreads();
}

// One team of TEAM threads per column of the list; CAP hash slots per team
// (at least twice the column's product count, so a probe always ends within
// CAP steps).  Output: cnt[c] entries at s2[off[c] ...] in row order (s1 is the
// unsorted staging copy).
template <int LOG2CAP, int TEAM>
__global__ void __launch_bounds__(TEAM == 32 ? 128 : TEAM)
k_sp_cols(int ncols, const int *__restrict__ cols, const int *__restrict__ lp, const int *__restrict__ li,
          const double *__restrict__ lv, const int *__restrict__ rp, const int *__restrict__ ri,
          const double *__restrict__ rv, const long long *__restrict__ off, int *__restrict__ s1r,
          double *__restrict__ s1v, int *__restrict__ s2r, double *__restrict__ s2v, int *__restrict__ cnt,
          unsigned *__restrict__ err) {
    constexpr int CAP = 1 << LOG2CAP;
    extern __shared__ __align__(16) unsigned char sm[];
    const int teams = blockDim.x / TEAM, team = threadIdx.x / TEAM, tid = threadIdx.x % TEAM;
    double *vals = (double *)sm + (size_t)team * CAP;
    int *keys = (int *)(sm + sizeof(double) * (size_t)teams * CAP) + (size_t)team * CAP;
    int *nlist = (int *)(sm + (sizeof(double) + sizeof(int)) * (size_t)teams * CAP) + team;
    for (int w = blockIdx.x * teams + team; w < ncols; w += gridDim.x * teams) {
        const int c = cols[w];
        for (int s = tid; s < CAP; s += TEAM) {
            keys[s] = -1;
            vals[s] = 0.0;
        }
        if (tid == 0) *nlist = 0;
        team_sync<TEAM>();
        for (int k = rp[c]; k < rp[c + 1]; k++) {
            const int src = ri[k];
            const double alpha = rv[k];
            for (int t = lp[src] + tid; t < lp[src + 1]; t += TEAM) {
                const int row = li[t];
                const double p = __dmul_rn(alpha, lv[t]);
                int slot = (int)(((unsigned)row * 2654435761u) >> (32 - LOG2CAP));
                int probes = 0;
                for (; probes < CAP; probes++) {
                    const int kk = keys[slot];
                    if (kk == row) break;
                    if (kk == -1) {
                        const int prev = atomicCAS(keys + slot, -1, row);
                        if (prev == -1 || prev == row) break;
                    }
                    slot = (slot + 1) & (CAP - 1);
                }
                if (probes == CAP) {
                    atomicOr(err, 2u);  // cannot happen with CAP >= 2 * products
                    continue;
                }
                vals[slot] = __dadd_rn(vals[slot], p);
            }
            team_sync<TEAM>();
        }
        // the nonzero entries (an entry that ends at zero is dropped), unsorted
        const long long o = off[c];
        for (int s = tid; s < CAP; s += TEAM)
            if (keys[s] != -1 && vals[s] != 0.0) {
                const int p = atomicAdd(nlist, 1);
                s1r[o + p] = keys[s];
                s1v[o + p] = vals[s];
            }
        team_sync<TEAM>();
        const int nl = *nlist;
        for (int e = tid; e < nl; e += TEAM) {
            const int key = s1r[o + e];
            int rank = 0;
            for (int j = 0; j < nl; j++) rank += s1r[o + j] < key;
            s2r[o + rank] = key;
            s2v[o + rank] = s1v[o + e];
        }
        if (tid == 0) cnt[c] = nl;
        team_sync<TEAM>();
    }
}

// The same for columns whose table does not fit in shared memory: one CTA a
// column, its table (2^log2cap slots) in global memory, one table per CTA.
__global__ void __launch_bounds__(512)
k_sp_cols_global(int ncols, const int *__restrict__ cols, const int *__restrict__ lp, const int *__restrict__ li,
                 const double *__restrict__ lv, const int *__restrict__ rp, const int *__restrict__ ri,
                 const double *__restrict__ rv, const long long *__restrict__ off, int *__restrict__ s1r,
                 double *__restrict__ s1v, int *__restrict__ s2r, double *__restrict__ s2v, int *__restrict__ cnt,
                 int log2cap, int *__restrict__ gkeys, double *__restrict__ gvals, unsigned *__restrict__ err) {
    __shared__ int nlist;
    const int cap = 1 << log2cap;
    int *keys = gkeys + (size_t)blockIdx.x * cap;
    double *vals = gvals + (size_t)blockIdx.x * cap;
    const int tid = threadIdx.x, T = blockDim.x;
    for (int w = blockIdx.x; w < ncols; w += gridDim.x) {
        const int c = cols[w];
        for (int s = tid; s < cap; s += T) {
            keys[s] = -1;
            vals[s] = 0.0;
        }
        if (tid == 0) nlist = 0;
        __syncthreads();
        for (int k = rp[c]; k < rp[c + 1]; k++) {
            const int src = ri[k];
            const double alpha = rv[k];
            for (int t = lp[src] + tid; t < lp[src + 1]; t += T) {
                const int row = li[t];
                const double p = __dmul_rn(alpha, lv[t]);
                int slot = (int)(((unsigned)row * 2654435761u) >> (32 - log2cap));
                int probes = 0;
                for (; probes < cap; probes++) {
                    const int kk = keys[slot];
                    if (kk == row) break;
                    if (kk == -1) {
                        const int prev = atomicCAS(keys + slot, -1, row);
                        if (prev == -1 || prev == row) break;
                    }
                    slot = (slot + 1) & (cap - 1);
                }
                if (probes == cap) {
                    atomicOr(err, 2u);
                    continue;
                }
                vals[slot] = __dadd_rn(vals[slot], p);
            }
            __syncthreads();
        }
        const long long o = off[c];
        for (int s = tid; s < cap; s += T)
            if (keys[s] != -1 && vals[s] != 0.0) {
                const int p = atomicAdd(&nlist, 1);
                s1r[o + p] = keys[s];
                s1v[o + p] = vals[s];
            }
        __syncthreads();
        const int nl = nlist;
        for (int e = tid; e < nl; e += T) {
            const int key = s1r[o + e];
            int rank = 0;
            for (int j = 0; j < nl; j++) rank += s1r[o + j] < key;
            s2r[o + rank] = key;
            s2v[o + rank] = s1v[o + e];
        }
        if (tid == 0) cnt[c] = nl;
        __syncthreads();
    }
}

__global__ void k_sp_gather(int ncols, const int *__restrict__ cols, const long long *__restrict__ off,
                            const int *__restrict__ rptr, const int *__restrict__ s2r,
                            const double *__restrict__ s2v, int *__restrict__ oi, double *__restrict__ ov) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int w = (int)(t / 32), lane = (int)(t % 32);
    if (w >= ncols) return;
    const int c = cols[w];
    const long long o = off[c];
    for (int e = rptr[c] + lane; e < rptr[c + 1]; e += 32) {
        oi[e] = s2r[o + e - rptr[c]];
        ov[e] = s2v[o + e - rptr[c]];
    }
}

template <int LOG2CAP, int TEAM>
void launch_cols(Ctx &c, const std::vector<int> &list, const int *lp, const int *li, const double *lv, const int *rp,
                 const int *ri, const double *rv, const long long *off, int *s1r, double *s1v, int *s2r,
                 double *s2v, int *cnt, unsigned *err) {
    if (list.empty()) return;
    constexpr int CAP = 1 << LOG2CAP;
    const int threads = TEAM == 32 ? 128 : TEAM;
    const int teams = threads / TEAM;
    const size_t smem = (sizeof(double) + sizeof(int)) * (size_t)teams * CAP + sizeof(int) * teams;
    SAGB_CUDA(cudaFuncSetAttribute(k_sp_cols<LOG2CAP, TEAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int *dl = dnew<int>(list.size());
    up(c, dl, list.data(), list.size());
    const long long want = ((long long)list.size() + teams - 1) / teams;
    const int grid = (int)std::min<long long>(want, (long long)c.num_sms * 16);
    k_sp_cols<LOG2CAP, TEAM><<<grid, threads, smem, c.stream>>>((int)list.size(), dl, lp, li, lv, rp, ri, rv, off, s1r,
                                                                s1v, s2r, s2v, cnt, err);
    SAGB_CUDA(cudaGetLastError());
    sync(c);
    dfree(dl);
}

// out[:, c] = sum_k right[k, c] * left[:, k] (cscSpMM, helper_sparse.hpp:257-285)
// for c < R; left has L rows.  Returned as compressed columns in a DMat
// (n = R columns, m = L).
DMat product(Ctx &c, const int *lp, const int *li, const double *lv, int L, const int *rp, const int *ri,
             const double *rv, int R, unsigned *d_err) {
    DMat O;
    O.n = R;
    O.m = L;
    O.rptr = dnew<int>(R + 1);
    long long *bound = dnew<long long>(R);
    if (R) k_sp_bound<<<blocks_for(R), kRsThreads, 0, c.stream>>>(R, rp, ri, lp, bound);
    std::vector<long long> hb(R);
    down(c, hb.data(), bound, R);
    sync(c);
    // classes by table size (at least twice the column's products): warps up
    // to 2^11 slots, CTAs up to 2^13 in shared memory, longer in global memory
    std::vector<int> lists[8], glist;
    int glog2 = 0;
    std::vector<long long> off(R + 1, 0);
    for (int col = 0; col < R; col++) {
        const long long b = hb[col];
        off[col + 1] = off[col] + b;
        if (b == 0) continue;
        int lg = 6;
        while ((1LL << lg) < 2 * b) lg++;
        if (lg > 30) throw SetupError{"GPU setup: Galerkin column too long"};
        if (lg > 13) {
            glist.push_back(col);
            glog2 = std::max(glog2, lg);
        } else {
            lists[lg - 6].push_back(col);
        }
    }
    const long long total = off[R];
    long long *doff = dnew<long long>(R + 1);
    up(c, doff, off.data(), R + 1);
    int *s1r = dnew<int>(total), *s2r = dnew<int>(total);
    double *s1v = dnew<double>(total), *s2v = dnew<double>(total);
    int *cnt = dnew<int>(R);
    SAGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * std::max(R, 1), c.stream));
    launch_cols<6, 32>(c, lists[0], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<7, 32>(c, lists[1], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<8, 32>(c, lists[2], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<9, 32>(c, lists[3], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<10, 32>(c, lists[4], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<11, 32>(c, lists[5], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<12, 256>(c, lists[6], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    launch_cols<13, 256>(c, lists[7], lp, li, lv, rp, ri, rv, doff, s1r, s1v, s2r, s2v, cnt, d_err);
    if (!glist.empty()) {
        // one table per CTA, at most ~2 GB of tables
        const long long per = (1LL << glog2) * (long long)(sizeof(int) + sizeof(double));
        const int grid = (int)std::max<long long>(
            1, std::min<long long>({(long long)glist.size(), (long long)c.num_sms * 2, (2LL << 30) / per}));
        int *gk = dnew<int>((size_t)grid << glog2);
        double *gv = dnew<double>((size_t)grid << glog2);
        int *dl = dnew<int>(glist.size());
        up(c, dl, glist.data(), glist.size());
        k_sp_cols_global<<<grid, 512, 0, c.stream>>>((int)glist.size(), dl, lp, li, lv, rp, ri, rv, doff, s1r, s1v,
                                                     s2r, s2v, cnt, glog2, gk, gv, d_err);
        SAGB_CUDA(cudaGetLastError());
        sync(c);
        dfree(dl);
        dfree(gk);
        dfree(gv);
    }
    const std::vector<int> rptr = scan_counts(c, cnt, R, O.rptr);
    O.nnz = rptr[R];
    O.cind = dnew<int>(O.nnz);
    O.val = dnew<double>(O.nnz);
    std::vector<int> all;
    for (int k = 0; k < 8; k++) all.insert(all.end(), lists[k].begin(), lists[k].end());
    all.insert(all.end(), glist.begin(), glist.end());
    if (!all.empty()) {
        int *dl = dnew<int>(all.size());
        up(c, dl, all.data(), all.size());
        k_sp_gather<<<blocks_for((long long)all.size() * 32), kRsThreads, 0, c.stream>>>(
            (int)all.size(), dl, doff, O.rptr, s2r, s2v, O.cind, O.val);
        SAGB_CUDA(cudaGetLastError());
        sync(c);
        dfree(dl);
    }
    dfree(bound);
    dfree(doff);
    dfree(s1r);
    dfree(s2r);
    dfree(s1v);
    dfree(s2v);
    dfree(cnt);
    return O;
}

// one level: A (device) -> CA (device), P and R (host copies); the host's rs_level
void rs_level_gpu(Ctx &c, const DMat &A, double theta, DMat &CA, CsrD &P_h, CsrD &R_h) {
    if (theta <= 0 || 1 < theta) throw SetupError{"Theta must be in 0 < theta <= 1"};
    const int N = A.n;
    // strength split
    double *thr = dnew<double>(N);
    int *scnt = dnew<int>(N), *wcnt = dnew<int>(N);
    k_rs_strong_count<<<blocks_for(N), kRsThreads, 0, c.stream>>>(N, A.rptr, A.cind, A.val, theta, thr, scnt, wcnt);
    SAGB_CUDA(cudaGetLastError());
    DMat S, W;
    S.n = W.n = S.m = W.m = N;
    S.rptr = dnew<int>(N + 1);
    W.rptr = dnew<int>(N + 1);
    const std::vector<int> srp = scan_counts(c, scnt, N, S.rptr);
    const std::vector<int> wrp = scan_counts(c, wcnt, N, W.rptr);
    S.nnz = srp[N];
    W.nnz = wrp[N];
    S.cind = dnew<int>(S.nnz);
    S.val = dnew<double>(S.nnz);
    W.cind = dnew<int>(W.nnz);
    W.val = dnew<double>(W.nnz);
    k_rs_strong_fill<<<blocks_for(N), kRsThreads, 0, c.stream>>>(N, A.rptr, A.cind, A.val, thr, S.rptr, S.cind, S.val,
                                                                 W.rptr, W.cind, W.val);
    SAGB_CUDA(cudaGetLastError());
    DMat St = transpose(c, S, false);
    // C/F splitting on the host
    CsrD Sh;
    Sh.n = Sh.m = N;
    Sh.rptr = srp;
    Sh.cind.resize(S.nnz);
    Sh.val.resize(S.nnz);
    down(c, Sh.cind.data(), S.cind, S.nnz);
    down(c, Sh.val.data(), S.val, S.nnz);
    Pattern Sth;
    Sth.n = N;
    Sth.rptr.resize(N + 1);
    Sth.cind.resize(St.nnz);
    down(c, Sth.rptr.data(), St.rptr, N + 1);
    down(c, Sth.cind.data(), St.cind, St.nnz);
    sync(c);
    St.release();
    std::vector<int> is_coarse;
    rs_first_pass(Sh, Sth, is_coarse);
    rs_second_pass(Sh, is_coarse);
    // interpolation: per-row layout on the host, arithmetic on the device
    std::vector<int> colmap(N, -1), ncs(N, 0), part(S.nnz), prp(N + 1, 0);
    std::vector<long long> amj_off(N + 1, 0);
    int nc = 0;
    for (int i = 0; i < N; i++)
        if (is_coarse[i]) colmap[i] = nc++;
    for (int i = 0; i < N; i++) {
        int k = srp[i];
        for (int j = srp[i]; j < srp[i + 1]; j++)
            if (is_coarse[Sh.cind[j]]) part[k++] = j;
        ncs[i] = k - srp[i];
        for (int j = srp[i]; j < srp[i + 1]; j++)
            if (!is_coarse[Sh.cind[j]]) part[k++] = j;
        const int ncf = srp[i + 1] - srp[i] - ncs[i];
        const long long rows_i = is_coarse[i] ? 1 : ncs[i];
        if ((long long)prp[i] + rows_i > INT_MAX) throw SetupError{"GPU setup: interpolation too large"};
        prp[i + 1] = prp[i] + (int)rows_i;
        amj_off[i + 1] = amj_off[i] + (is_coarse[i] ? 0 : (long long)ncs[i] * ncf);
    }
    DMat P;
    P.n = N;
    P.m = nc;
    P.nnz = prp[N];
    P.rptr = dnew<int>(N + 1);
    P.cind = dnew<int>(P.nnz);
    P.val = dnew<double>(P.nnz);
    int *d_isc = dnew<int>(N), *d_col = dnew<int>(N), *d_ncs = dnew<int>(N), *d_part = dnew<int>(S.nnz);
    long long *d_amj_off = dnew<long long>(N + 1);
    double *d_amj = dnew<double>(amj_off[N]), *d_amk = dnew<double>(S.nnz);
    unsigned *d_warn = dnew<unsigned>(N);
    int *d_stop = dnew<int>(1);
    unsigned *d_err = dnew<unsigned>(1);
    SAGB_CUDA(cudaMemsetAsync(d_warn, 0, sizeof(unsigned) * N, c.stream));
    up(c, d_stop, &N, 1);
    up(c, P.rptr, prp.data(), N + 1);
    up(c, d_isc, is_coarse.data(), N);
    up(c, d_col, colmap.data(), N);
    up(c, d_ncs, ncs.data(), N);
    up(c, d_part, part.data(), S.nnz);
    up(c, d_amj_off, amj_off.data(), N + 1);
    k_rs_interp<<<blocks_for(N), kRsThreads, 0, c.stream>>>(N, A.rptr, A.cind, A.val, S.rptr, S.cind, S.val, W.rptr,
                                                            W.val, d_isc, d_col, d_ncs, d_part, d_amj_off, d_amj,
                                                            d_amk, P.rptr, P.cind, P.val, d_warn, d_stop);
    SAGB_CUDA(cudaGetLastError());
    // the host setup's messages in its order: the warnings of the rows up to
    // the first stopping row (helper_multigrid.hpp:511-518)
    std::vector<unsigned> warn(N);
    int first_stop = N;
    unsigned err = 0;
    down(c, warn.data(), d_warn, N);
    down(c, &first_stop, d_stop, 1);
    sync(c);
    for (int i = 0; i < N && i <= first_stop; i++)
        for (unsigned k = 0; k < warn[i]; k++) printf("1 amk = 0\n");
    if (first_stop < N) {
        printf("2 amk = 0\n");
        fflush(stdout);
        dfree(d_warn); dfree(d_stop); dfree(d_err);
        throw SetupError{"interpolation: fine row " + std::to_string(first_stop) +
                         " has a strong fine neighbour with no coupling to its coarse points (2 amk = 0)"};
    }
    dfree(thr); dfree(scnt); dfree(wcnt);
    dfree(d_isc); dfree(d_col); dfree(d_ncs); dfree(d_part); dfree(d_amj_off); dfree(d_amj); dfree(d_amk);
    dfree(d_warn);
    dfree(d_stop);
    S.release();
    W.release();
    // R = P^T and the Galerkin operator (get_coarse_matrix, helper_multigrid.hpp:564-586):
    // T = A^T P, then C = P^T T, read back as CSR
    DMat R = transpose(c, P, true);
    SAGB_CUDA(cudaMemsetAsync(d_err, 0, sizeof(unsigned), c.stream));
    DMat T = product(c, A.rptr, A.cind, A.val, A.n, R.rptr, R.cind, R.val, P.m, d_err);
    DMat C = product(c, P.rptr, P.cind, P.val, P.m, T.rptr, T.cind, T.val, P.m, d_err);
    down(c, &err, d_err, 1);
    sync(c);
    dfree(d_err);
    if (err) throw SetupError{"GPU setup: Galerkin product hash table overflow"};
    T.release();
    C.m = C.n = P.m;
    CA = C;
    P_h = download(c, P);
    R_h = download(c, R);
    P.release();
    R.release();
}

}  // namespace

RsChain rs_chain_gpu(Ctx &c, const CsrD &A, double theta, int max_levels, int coarse_size) {
    RsChain ch;
    DMat cur = upload(c, A);
    try {
        int depth = 0;
        while (true) {
            if (depth >= 1) {
                if (!(max_levels > depth && ch.CA[depth - 1].n > coarse_size)) break;
                if (coarse_size != 2000 && depth >= 2 && ch.CA[depth - 1].n * 10 > ch.CA[depth - 2].n * 9) break;
            }
            DMat ca;
            CsrD p, r;
            rs_level_gpu(c, cur, theta, ca, p, r);
            cur.release();
            cur = ca;
            ch.CA.push_back(download(c, cur));
            ch.P.push_back(std::move(p));
            ch.R.push_back(std::move(r));
            depth++;
        }
    } catch (...) {
        cur.release();
        throw;
    }
    cur.release();
    return ch;
}

}  // namespace sagb
