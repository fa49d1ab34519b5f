"""GPU parity of the batched FP64 and FP32-mixed siblings (sa_batch_fp_*).

Per system and right-hand side the batched V-cycle must be the oracle's
dfAMG V-cycle (Library/preconditioner/INTAMG.hpp:86-134) with the multicolour
SOR sweep in the system's colour order, on the same hierarchy: within 1e-12
relative in FP64 (the GPU sums a row's products in lane order, the oracle in
index order) and within float rounding in FP32.  Whole solves must reach the
explicit residual and take the iterations of the oracle's Restarted(FGMRES<T>)
on the same hierarchy within one."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle_ffi as of
import sagb
import setup_views as sv

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    of.lib().or_set_threads(os.cpu_count() or 1)
    yield c
    c.close()


SYSTEMS = [(sagb.GEN_POISSON3D, 12, 0.0), (sagb.GEN_STENCIL27, 10, 0.0), (sagb.GEN_CONVDIFF3D, 14, 20.0),
           (sagb.GEN_POISSON2D, 40, 0.0), (sagb.GEN_POISSON3D, 17, 0.0), (sagb.GEN_VARCOEF3D, 13, 1.0)]


def _systems(specs, seed=1):
    out, bs = [], []
    for k, (kind, n, prm) in enumerate(specs):
        A = sagb.HostCsr.generate(kind, n, prm, seed=k + 1)
        _, b = A.rhs(seed + 100 * k)
        A.lmax1_scaling(b)
        out.append(A.arrays())
        bs.append(b)
    return out, bs


def _oracle_vcycle(h, x, prec):
    x = np.ascontiguousarray(x, np.float64 if prec == sagb.F64 else np.float32)
    ref = np.zeros_like(x)
    if prec == sagb.F64:
        of.lib().or_vcycle_f64(C.byref(h), of.ptr(x, of.f64p), of.ptr(ref, of.f64p))
    else:
        of.lib().or_vcycle_f32(C.byref(h), of.ptr(x, of.f32p), of.ptr(ref, of.f32p))
    return ref


def _check_vcycle(B, F, prec, nrhs, seed, tol):
    dt = np.float64 if prec == sagb.F64 else np.float32
    vin = np.random.default_rng(seed).uniform(-1, 1, size=B.rows * nrhs).astype(dt)
    out = F.precondition(vin).reshape(B.rows, nrhs)
    vin2 = vin.reshape(B.rows, nrhs)
    keep = of.Keep()
    for s in range(B.nsys):
        h = sv.oracle_amg(keep, B.system_setup(s).derive(prec))
        a, e = B.offsets[s], B.offsets[s + 1]
        for q in range(nrhs):
            ref = _oracle_vcycle(h, vin2[a:e, q], prec).astype(np.float64)
            got = out[a:e, q].astype(np.float64)
            assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref), (s, q)
    return vin, out


@pytest.mark.parametrize("nrhs", [1, 2, 4])
@pytest.mark.parametrize("prec", [sagb.F64, sagb.F32])
def test_batched_fp_vcycle(ctx, prec, nrhs):
    systems, _ = _systems(SYSTEMS)
    B = sagb.Batch(ctx, systems, nrhs)
    F = sagb.BatchFp(ctx, B, prec)
    tol = FP64_TOL if prec == sagb.F64 else FP32_TOL
    vin, out = _check_vcycle(B, F, prec, nrhs, 7 + nrhs, tol)
    # the autotuner changes lanes per row and the sweep form; results stay
    # within the same tolerance of the oracle
    F.autotune(2)
    _check_vcycle(B, F, prec, nrhs, 7 + nrhs, tol)
    F.close()
    B.close()


def test_batched_fp64_vcycle_poisson128(ctx):
    """The FP64 sibling of the headline engine on 3D Poisson 128^3 (batched
    defaults, autotuned) against the oracle's FP64 colour-ordered V-cycle."""
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, 128)
    _, b = A.rhs(1)
    A.lmax1_scaling(b)
    B = sagb.Batch(ctx, [A.arrays()], 1)
    F = sagb.BatchFp(ctx, B, sagb.F64)
    F.autotune(2)
    keep = of.Keep()
    h = sv.oracle_amg(keep, B.system_setup(0).derive(sagb.F64))
    got = F.precondition(b)
    ref = _oracle_vcycle(h, b, sagb.F64)
    assert np.linalg.norm(got - ref) <= FP64_TOL * np.linalg.norm(ref)
    F.close()
    B.close()


@pytest.mark.parametrize("prec", [sagb.F64, sagb.F32])
def test_batched_fp_fused_one_colour_sweeps(ctx, prec):
    """With one colour below the finest level (caps [8, 1]) the FP engine fuses
    those levels' sweeps into the neighbouring SpMVs (sa_batch_fp_fused_sweeps):
    the V-cycle stays within the oracle's tolerance and is bit-identical to the
    unfused one (the step (in - 0) * dinv is the same IEEE operation in the
    SpMV's epilogue as in the colour kernel)."""
    nrhs = 2
    systems, _ = _systems(SYSTEMS)
    B = sagb.Batch(ctx, systems, nrhs)
    B.set_colour_caps([8, 1])
    F = sagb.BatchFp(ctx, B, prec)
    nf = F.fused_sweeps()
    assert nf > 0
    tol = FP64_TOL if prec == sagb.F64 else FP32_TOL
    vin, out_on = _check_vcycle(B, F, prec, nrhs, 31, tol)
    assert F.fused_sweeps(0) == 0
    np.testing.assert_array_equal(F.precondition(vin), out_on.ravel())
    assert F.fused_sweeps(1) == nf
    F.close()
    B.close()


@pytest.mark.parametrize("prec", [sagb.F64, sagb.F32])
def test_batched_fp_solve(ctx, prec):
    """Restarted(FGMRES<T>) per pair against the oracle's solve on each
    system's own hierarchy, both stopping on the inner solver's estimate as
    the reference does: iteration counts within one (FP64) or three (FP32,
    whose float dot products round differently in any other summation
    order).  With the explicit-residual stop every pair reaches 1e-10."""
    systems, bs = _systems(SYSTEMS[:4])
    nrhs = 2
    B = sagb.Batch(ctx, systems, nrhs)
    F = sagb.BatchFp(ctx, B, prec)
    cols = []
    for s, b in enumerate(bs):
        cols.append(np.stack([b, np.roll(b, 3)], 1))
    bb = np.concatenate(cols, 0).ravel()
    nb = np.array([np.linalg.norm(c[:, q]) for c in cols for q in range(nrhs)])
    x = np.zeros(B.rows * nrhs)
    it_e, cv = F.solve(sagb.solver_params(m=20, explicit_stop=1), bb, nb, x)
    assert cv.all(), (it_e, cv)
    X = x.reshape(B.rows, nrhs).copy()
    x = np.zeros(B.rows * nrhs)
    it, cv = F.solve(sagb.solver_params(m=20), bb, nb, x)
    assert cv.all(), (it, cv)
    keep = of.Keep()
    for s, (r, c, v) in enumerate(systems):
        a, e = B.offsets[s], B.offsets[s + 1]
        setup = B.system_setup(s).derive(prec)
        h = sv.oracle_amg(keep, setup)
        dA = of.csr_f(keep, r, c, v, np.float64)
        for q in range(nrhs):
            bq = np.ascontiguousarray(cols[s][:, q])
            rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
            Ax = np.bincount(rows, weights=v * X[a:e, q][c], minlength=len(r) - 1)
            assert np.linalg.norm(bq - Ax) <= 1e-10 * np.linalg.norm(bq), (s, q)
            xo = np.zeros(len(bq))
            if prec == sagb.F64:
                it_o = of.lib().or_ir_solve_f64(C.byref(dA), C.byref(h), 20, 1e-10, of.ptr(bq, of.f64p),
                                                float(np.linalg.norm(bq)), of.ptr(xo, of.f64p), 50, 0)
            else:
                fA = of.csr_f(keep, r, c, v, np.float32)
                it_o = of.lib().or_ir_solve_f32(C.byref(dA), C.byref(fA), C.byref(h), 20, 1e-10,
                                                of.ptr(bq, of.f64p), float(np.linalg.norm(bq)),
                                                of.ptr(xo, of.f64p), 50, 0)
            assert abs(int(it[s * nrhs + q]) - it_o) <= (1 if prec == sagb.F64 else 3), (s, q, it[s * nrhs + q], it_o)
    F.close()
    B.close()


@pytest.mark.parametrize("prec", [sagb.F64, sagb.F32])
def test_batched_fp_cycle_graph(ctx, prec):
    """A restart cycle as one graph gated on the device gives the solve of
    the step-by-step form bit for bit (the same kernels in the same order)."""
    systems, bs = _systems(SYSTEMS[:3])
    B = sagb.Batch(ctx, systems, 1)
    F = sagb.BatchFp(ctx, B, prec)
    bb = np.concatenate(bs)
    nb = np.array([np.linalg.norm(b) for b in bs])
    p = sagb.solver_params(m=20, explicit_stop=1)
    x1 = np.zeros(B.rows)
    it1, cv1 = F.solve(p, bb, nb, x1)
    assert cv1.all() and F.cycle_graphs() > 0
    ctx.set_option(sagb.OPT_CYCLE_GRAPH, 0)
    try:
        x2 = np.zeros(B.rows)
        it2, cv2 = F.solve(p, bb, nb, x2)
        assert F.cycle_graphs() == 0
    finally:
        ctx.set_option(sagb.OPT_CYCLE_GRAPH, 1)
    np.testing.assert_array_equal(it1, it2)
    np.testing.assert_array_equal(x1, x2)
    F.close()
    B.close()
