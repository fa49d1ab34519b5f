"""GPU parity of the multicolour smoother variant against the C oracle.

The multicolour split keeps the natural numbering; the sweep's schedule uses
the colours as its levels, so a sweep is one barrier per colour instead of one
per dependency level.  Integer results must equal the oracle's colour-ordered
sweep bit for bit; FP64 results bit for bit in the sequential-order mode."""
import ctypes as C

import numpy as np
import pytest

import oracle_ffi as of
import sagb
import setup_views as sv

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    yield c
    c.close()


def _problem(kind, n, param=0.0):
    A = sagb.HostCsr.generate(kind, n, param)
    xs, b = A.rhs(1)
    A.lmax1_scaling(b)
    return A, b


CASES = [(sagb.GEN_POISSON3D, 40, 0.0), (sagb.GEN_STENCIL27, 20, 0.0), (sagb.GEN_CONVDIFF3D, 24, 20.0)]


@pytest.mark.parametrize("kind,n,param", CASES)
def test_int_mc_sweep_and_vcycle_bit_exact(ctx, kind, n, param):
    A, b = _problem(kind, n, param)
    r, c, v = A.arrays()
    setup = sagb.Setup(sagb.INT, r, c, v, sagb.amg_params(multicolor=1))
    M = sagb.Amg(ctx, sagb.INT, setup=setup)
    keep = of.Keep()
    h = sv.oracle_amg(keep, setup)
    rng = np.random.default_rng(11)
    N = len(r) - 1
    for lv in range(setup.depth):
        col = setup.view(sagb.OP_COLOR, lv)
        nl = len(col)
        assert M.level_info(sagb.OP_LD, lv)[4] == col.max() + 1  # one sweep level per colour
        vin = rng.integers(-(1 << 28), 1 << 28, size=nl).astype(np.int32)
        ref = np.zeros_like(vin)
        of.lib().or_ldtri_order_i32(C.byref(h.LD[lv]), of.ptr(of.colour_order(col), of.i32p),
                                    of.ptr(vin, of.i32p), of.ptr(ref, of.i32p))
        np.testing.assert_array_equal(M.sweep(lv, vin), ref)
    vin = rng.integers(-(1 << 29), 1 << 29, size=N).astype(np.int32)
    ref = np.zeros_like(vin)
    of.lib().or_vcycle_i32(C.byref(h), of.ptr(vin, of.i32p), of.ptr(ref, of.i32p))
    np.testing.assert_array_equal(M.precondition(vin), ref)
    M.close()


def test_fp64_mc_vcycle(ctx):
    A, b = _problem(sagb.GEN_POISSON3D, 32)
    r, c, v = A.arrays()
    setup = sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=1))
    keep = of.Keep()
    h = sv.oracle_amg(keep, setup)
    ref = np.zeros(len(b))
    of.lib().or_vcycle_f64(C.byref(h), of.ptr(b, of.f64p), of.ptr(ref, of.f64p))
    ctx.set_option(sagb.OPT_FP_EXACT, 1)
    try:
        M = sagb.Amg(ctx, sagb.F64, setup=setup)
        np.testing.assert_array_equal(M.precondition(b), ref)
        M.close()
    finally:
        ctx.set_option(sagb.OPT_FP_EXACT, 0)
    M = sagb.Amg(ctx, sagb.F64, setup=setup)
    out = M.precondition(b)
    assert np.linalg.norm(out - ref) <= 1e-12 * np.linalg.norm(ref)
    M.close()


@pytest.mark.parametrize("kind,n", [(sagb.GEN_POISSON3D, 48), (sagb.GEN_STENCIL27, 32)])
def test_int_mc_solve_converges(ctx, kind, n):
    """int-AMG-FGMRES with the multicolour smoother reaches the reference's
    tolerance; its iteration count is reported next to the natural order's."""
    A, b = _problem(kind, n)
    r, c, v = A.arrays()
    nrm_b = float(np.linalg.norm(b))
    dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
    iA = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
    its = {}
    for mc in (0, 1):
        s_int = sagb.Setup(sagb.INT, r, c, v, sagb.amg_params(multicolor=mc))
        M = sagb.Amg(ctx, sagb.INT, setup=s_int)
        M64 = sagb.Amg(ctx, sagb.F64, setup=s_int.derive(sagb.F64))
        bits = sagb.rule_bits(ctx, M64, b, nrm_b)
        S = sagb.Solver(ctx, sagb.INT, dA, iA, M, sagb.solver_params(m=30, frac_bits=bits, explicit_stop=1))
        x = np.zeros(len(b))
        it, conv = S.solve(b, nrm_b, x)
        rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
        res = np.linalg.norm(b - np.bincount(rows, weights=v * x[c], minlength=len(b))) / nrm_b
        assert conv == 1 and res <= 1e-10, (mc, it, res)
        its[mc] = it
        S.close(); M.close(); M64.close()
    print("iterations natural/multicolour:", its)
    assert its[1] <= 2 * its[0] + 5
