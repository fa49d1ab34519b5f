"""sa_amg_sweep_noalloc: the Gauss-Seidel sweep for callers that cannot
allocate device memory while they solve (their GPU memory is already claimed by
another allocator, or they cannot afford the synchronisation cudaMalloc and
cudaFree imply).  Its scratch lives in a static device array instead of an
allocation; its output must be the regular sweep's, call after call.

Kept in a file of its own, collected last."""
import numpy as np
import pytest

import sagb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,dtype", [(sagb.INT, np.int32), (sagb.F64, np.float64)])
def test_noalloc_sweep_matches_sweep(prec, dtype):
    ctx = sagb.Context(0)
    # 40^3 = 64,000 rows: the fine level runs the multi-CTA kernel that needs
    # scratch, the coarse ones the shared-memory kernel
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, 40)
    xs, b = A.rhs(3)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    M = sagb.Amg(ctx, prec, r, c, v)
    rng = np.random.default_rng(11)
    for level in range(M.depth):
        n = M.level_info(sagb.OP_LD, level)[0]
        if prec == sagb.INT:
            x = rng.integers(-(1 << 29), 1 << 29, size=n).astype(dtype)
        else:
            x = rng.standard_normal(n).astype(dtype)
        dx = sagb.DeviceArray.from_host(ctx, x)
        dref = sagb.DeviceArray(ctx, n, dtype)
        dout = sagb.DeviceArray(ctx, n, dtype)
        sagb.check(sagb.lib().sa_amg_sweep(ctx.h, M.h, level, dx.ptr, dref.ptr))
        ref = dref.download()
        for _ in range(2):  # two calls in a row share the static scratch
            sagb.check(sagb.lib().sa_amg_sweep_noalloc(ctx.h, M.h, level, dx.ptr, dout.ptr))
            ctx.sync()
            np.testing.assert_array_equal(dout.download(), ref)
        for d in (dx, dref, dout):
            d.close()
    assert ctx.flags() == 0
    # host buffers would need staging (an allocation): rejected
    with pytest.raises(sagb.SagbError):
        sagb.check(sagb.lib().sa_amg_sweep_noalloc(ctx.h, M.h, 0, np.zeros(4).ctypes.data, np.zeros(4).ctypes.data))
    M.close()
    ctx.close()
