// Tile-staged CSR row sums for integer matrices with short rows.
//
// A CTA owns blockDim.x consecutive rows (one per thread).  Their entries form
// one contiguous range of the CSR arrays, which the CTA streams through shared
// memory in chunks with coalesced 16-byte loads; each thread then sums the
// part of its own row that lies in the chunk, gathering x through the
// read-only cache.  The matrix bytes thus move at full line utilisation even
// when rows are a few entries long, where a lane-per-entry kernel leaves most
// of each load idle.  Integer sums wrap like the reference's, so the result is
// the same as any other order.
#pragma once
#include "common.cuh"

namespace sagb {

constexpr int kStreamThreads = 256;
constexpr int kStreamCap = 2048;  // entries per chunk (16 KB of shared memory)

// x interleaves R right-hand sides: x[col * R + r]
template <int R>
__device__ __forceinline__ void gather_r(const int *__restrict__ x, int col, int (&v)[R]) {
    if constexpr (R == 4) {
        const int4 q = __ldg(reinterpret_cast<const int4 *>(x) + col);
        v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else if constexpr (R == 2) {
        const int2 q = __ldg(reinterpret_cast<const int2 *>(x) + col);
        v[0] = q.x; v[1] = q.y;
    } else {
        v[0] = __ldg(x + col);
    }
}

// Rows [r0, r1) with r1 - r0 <= blockDim.x: thread t adds the sum over row
// r0 + t of val * x to acc[r].  Every thread of the CTA must call it (it
// synchronises the CTA).  PDL: the first chunk of the matrix is staged before
// pdl_wait(), x is read after it.
template <int R, bool PDL = false>
__device__ __forceinline__ void stream_rows(int r0, int r1, const int *__restrict__ rptr,
                                            const int *__restrict__ cind, const int *__restrict__ val,
                                            const int *__restrict__ x, long long (&acc)[R]) {
    __shared__ int s_val[kStreamCap], s_col[kStreamCap];
    const int tid = threadIdx.x, bd = blockDim.x;
    const int row = r0 + tid;
    const int a = __ldg(rptr + r0), b = __ldg(rptr + r1);
    const int ra = row < r1 ? __ldg(rptr + row) : 0, rb = row < r1 ? __ldg(rptr + row + 1) : 0;
    if (PDL && a >= b) pdl_wait();  // no entries: nothing staged
    for (int base = a; base < b; base += kStreamCap) {
        const int cnt = min(kStreamCap, b - base);
        const int head = min(cnt, (4 - (base & 3)) & 3);
        for (int i = tid; i < head; i += bd) {
            s_val[i] = __ldg(val + base + i);
            s_col[i] = __ldg(cind + base + i);
        }
        const int nv = (cnt - head) >> 2;
        const int4 *v4 = reinterpret_cast<const int4 *>(val + base + head);
        const int4 *c4 = reinterpret_cast<const int4 *>(cind + base + head);
        for (int i = tid; i < nv; i += bd) {
            const int4 q = __ldg(v4 + i), p = __ldg(c4 + i);
            const int o = head + 4 * i;
            s_val[o] = q.x; s_val[o + 1] = q.y; s_val[o + 2] = q.z; s_val[o + 3] = q.w;
            s_col[o] = p.x; s_col[o + 1] = p.y; s_col[o + 2] = p.z; s_col[o + 3] = p.w;
        }
        for (int i = head + 4 * nv + tid; i < cnt; i += bd) {
            s_val[i] = __ldg(val + base + i);
            s_col[i] = __ldg(cind + base + i);
        }
        __syncthreads();
        if (PDL && base == a) pdl_wait();
        const int lo = max(ra, base), hi = min(rb, base + cnt);
        for (int j = lo; j < hi; j++) {
            const long long v = s_val[j - base];
            int xv[R];
            gather_r<R>(x, s_col[j - base], xv);
#pragma unroll
            for (int r = 0; r < R; r++) acc[r] = wadd(acc[r], v * (long long)xv[r]);
        }
        __syncthreads();
    }
}

}  // namespace sagb
