"""The GPU Ruge-Stueben setup against the host setup and the reference.

sa_setup_create_gpu runs each level's strength split, transposes,
interpolation and both Galerkin products on the GPU (the C/F splitting on the
host).  Its hierarchy must be the host setup's bit for bit: against the
reference's own hierarchies (the golden fixtures the host setup is pinned to)
and against the host setup on larger generated problems whose coarse Galerkin
columns exercise every product path (warp teams, CTA teams and the host loop
for the longest columns)."""
import numpy as np
import pytest

import oracle_ffi as of
import sagb

pytestmark = pytest.mark.gpu

GOLDEN = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14", "p3d16bj"]


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    yield c
    c.close()


def _params(case):
    return sagb.amg_params(smoother_blocks=40 if case.endswith("bj") else 0)


def _cmp(got, g, pfx, with_bits=True):
    r, c, v, bit, dbit, m = got
    meta = g[pfx + "_meta"]
    np.testing.assert_array_equal(r, g[pfx + "_rptr"], err_msg=pfx + " rptr")
    np.testing.assert_array_equal(c, g[pfx + "_cind"], err_msg=pfx + " cind")
    np.testing.assert_array_equal(v, g[pfx + "_val"], err_msg=pfx + " val")
    assert m == meta[1]
    if with_bits:
        assert (bit, dbit) == (meta[2], meta[3]), pfx


@pytest.mark.parametrize("case", GOLDEN)
def test_gpu_setup_matches_reference(ctx, case):
    g = of.load_golden(case)
    s = sagb.Setup(sagb.INT, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], _params(case), ctx=ctx)
    D = int(g["depth"][0])
    assert s.depth == D
    for i in range(D):
        if i < D - 1:
            _cmp(s.view(sagb.OP_CA, i), g, f"L{i}_CA")
        _cmp(s.view(sagb.OP_P, i), g, f"L{i}_P")
        _cmp(s.view(sagb.OP_R, i), g, f"L{i}_R")
        _cmp(s.view(sagb.OP_LD, i), g, f"S{i}_LD")
    _cmp(s.view(sagb.OP_LUL), g, "LU_L", with_bits=False)
    _cmp(s.view(sagb.OP_LUU), g, "LU_U")
    if "d_depth" in g:
        d = sagb.Setup(sagb.F64, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], _params(case), ctx=ctx)
        for i in range(int(g["d_depth"][0])):
            if i < D - 1:
                _cmp(d.view(sagb.OP_CA, i), g, f"d_L{i}_CA", with_bits=False)
            _cmp(d.view(sagb.OP_P, i), g, f"d_L{i}_P", with_bits=False)


def _views_equal(a, b):
    assert a.depth == b.depth
    ops = [sagb.OP_P, sagb.OP_R, sagb.OP_LD, sagb.OP_U]
    for i in range(a.depth):
        for op in ops + ([sagb.OP_CA] if i < a.depth - 1 else []):
            va, vb = a.view(op, i), b.view(op, i)
            for x, y in zip(va[:3], vb[:3]):
                np.testing.assert_array_equal(x, y, err_msg=f"op {op} level {i}")
            assert va[3:] == vb[3:], (op, i)
    for op in (sagb.OP_LUL, sagb.OP_LUU):
        va, vb = a.view(op), b.view(op)
        for x, y in zip(va[:3], vb[:3]):
            np.testing.assert_array_equal(x, y)


GENERATED = [(sagb.GEN_POISSON3D, 40, 0.0), (sagb.GEN_STENCIL27, 30, 0.0), (sagb.GEN_CONVDIFF3D, 28, 50.0),
             (sagb.GEN_VARCOEF3D, 24, 2.0), (sagb.GEN_ANISO2D, 160, 1e-3)]


@pytest.mark.parametrize("kind,n,prm", GENERATED)
@pytest.mark.parametrize("prec", [sagb.F64, sagb.INT])
def test_gpu_setup_matches_host(ctx, kind, n, prm, prec):
    A = sagb.HostCsr.generate(kind, n, prm, seed=3)
    xs, b = A.rhs(5)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    for params in (sagb.amg_params(), sagb.amg_params(multicolor=1, max_colours=8, coarse_colours=2, coarse_size=100)):
        host = sagb.Setup(prec, r, c, v, params)
        gpu = sagb.Setup(prec, r, c, v, params, ctx=ctx)
        _views_equal(host, gpu)


def test_batch_gpu_chain_matches_host(ctx):
    """sa_batch_create builds the chains of large systems on the GPU
    (SA_OPT_GPU_SETUP: here systems of 100000 rows or more): the batch's
    hierarchy and its V-cycle are those of the host-built batch."""
    systems = []
    for kind, n in ((sagb.GEN_POISSON3D, 48), (sagb.GEN_STENCIL27, 12)):
        A = sagb.HostCsr.generate(kind, n, 0.0, seed=2)
        xs, b = A.rhs(3)
        A.lmax1_scaling(b)
        systems.append(A.arrays())
    assert len(systems[0][0]) - 1 >= 100000
    ctx.set_option(sagb.OPT_GPU_SETUP, 100000)
    try:
        Bg = sagb.Batch(ctx, systems, 1)
        ctx.set_option(sagb.OPT_GPU_SETUP, 0)
        Bh = sagb.Batch(ctx, systems, 1)
    finally:
        ctx.set_option(sagb.OPT_GPU_SETUP, 1)
    for s in range(2):
        _views_equal(Bg.system_setup(s), Bh.system_setup(s))
    vin = np.random.default_rng(1).integers(-(1 << 28), 1 << 28, size=Bg.rows).astype(np.int32)
    np.testing.assert_array_equal(Bg.precondition(vin), Bh.precondition(vin))
    Bg.close()
    Bh.close()
