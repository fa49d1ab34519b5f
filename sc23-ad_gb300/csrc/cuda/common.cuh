// Device helpers shared by the sm_103a kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sagb {

// device status bits (sa_status flags in include/sagb.h)
enum : unsigned {
    ST_OVERFLOW = 1u,      // an integer result left the int32 range (wrapped as in the reference)
    ST_TIMEOUT = 2u,       // a bounded wait ran out (dependency never published)
    ST_DIVZERO = 4u,       // Hessenberg / Givens denominator was zero
    ST_NORM_OVF = 8u,      // int64 sum of squares wrapped (negative)
    ST_PREC_OVF = 16u,     // an int32 result wrapped inside the preconditioner (V-cycle)
};

// Time limit of every spin wait in device code (nanoseconds).
constexpr unsigned long long kSpinLimitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// two's-complement arithmetic (the reference relies on wrap-around)
__device__ __forceinline__ long long wadd(long long a, long long b) {
    return (long long)((unsigned long long)a + (unsigned long long)b);
}
__device__ __forceinline__ long long wsub(long long a, long long b) {
    return (long long)((unsigned long long)a - (unsigned long long)b);
}
__device__ __forceinline__ long long wmul(long long a, long long b) {
    return (long long)((unsigned long long)a * (unsigned long long)b);
}
__device__ __forceinline__ long long wshl(long long a, int s) { return (long long)((unsigned long long)a << s); }
__device__ __forceinline__ int lo32(long long v) { return (int)(unsigned)(unsigned long long)v; }
__device__ __forceinline__ bool fits32(long long v) { return v == (long long)(int)v; }

// (int)(double) as compiled by g++ on x86-64 (cvttsd2si): truncation toward
// zero, INT_MIN when out of range or NaN (CUDA's conversion saturates instead).
__device__ __forceinline__ int d2i_x86(double v) {
    if (!(v > -2147483649.0 && v < 2147483648.0)) return (int)0x80000000;
    return __double2int_rz(v);
}
__device__ __forceinline__ long long d2l_x86(double v) {
    if (!(v > -9223372036854775808.0 && v < 9223372036854775808.0)) return (long long)0x8000000000000000ull;
    return __double2ll_rz(v);
}

// ------------------------------------------- bulk copies and mbarriers (sm_90+)
__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// one-dimensional bulk copy global -> shared; addresses and size 16-byte aligned
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

template <typename T>
__device__ __forceinline__ T shfl_xor(T v, int o) {
    return __shfl_xor_sync(0xffffffffu, v, o);
}

// integer square root by Newton's method (blas1::int32::lsqrt, blas1.hpp:107-119)
__device__ __forceinline__ long long lsqrt_dev(long long x) {
    if (x <= 0) return 0;
    long long s = 1, t = x;
    while (s < t) { s <<= 1; t >>= 1; }
    do {
        t = s;
        s = (x / s + s) >> 1;
    } while (s < t);
    return t;
}


// Programmatic dependent launch.  The V-cycle's kernels are launched with the
// programmatic-serialization attribute: a kernel may start while the one
// before it drains, reads what does not change during the V-cycle (row
// pointers, row lists), then waits at pdl_wait() until the previous grid has
// completed and its writes are visible; nothing it reads or writes that the
// previous kernels produce or read is touched before that wait.  Each kernel
// lets its successor start as soon as all of its own CTAs are running.
// Launched without the attribute, both instructions have no effect.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

}  // namespace sagb
