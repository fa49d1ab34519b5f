"""GPU parity: the sm_103a kernels against the reference's own outputs
(tests/golden, dumped from the reference classes) and against the C oracle.

Integer kernels must be bit-exact.  FP64 kernels are bit-exact in the
sequential-order mode (SA_OPT_FP_EXACT) and within 1e-12 relative otherwise.
Whole solves are compared by iteration count and explicit residual (the FP64
norm of the refinement residual is a parallel reduction on the GPU, so its last
bits differ from the sequential CPU sum, and the integer iterates follow)."""
import ctypes as C

import numpy as np
import pytest

import oracle_ffi as of
import sagb
import setup_views as sv

pytestmark = pytest.mark.gpu

INT_CASES = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14", "p3d16bj", "p3d16js", "p2d64js"]
FP_TOL = 1e-12


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    yield c
    c.close()


def _params(case):
    """SOR (the default), BlockSOR-40 ("bj") or JacobiSORflex ("js")."""
    return sagb.amg_params(smoother_blocks=40 if case.endswith("bj") else 0, multicolor=2 if case.endswith("js") else 0)


def _amg(ctx, g, case, prec=sagb.INT):
    return sagb.Amg(ctx, prec, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], _params(case))


def seq_norm(x):
    return of.lib().or_nrm2_f64(of.ptr(np.ascontiguousarray(x), of.f64p), len(x))


def explicit_res(g, x):
    r, c, v = g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"]
    rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
    Ax = np.bincount(rows, weights=v * x[c], minlength=len(r) - 1)
    b = g["b_scaled"]
    return np.linalg.norm(b - Ax) / np.linalg.norm(b)


@pytest.mark.parametrize("case", INT_CASES)
def test_int_kernels_bit_exact(ctx, case):
    g = of.load_golden(case)
    M = _amg(ctx, g, case)
    D = int(g["depth"][0])
    assert M.depth == D
    np.testing.assert_array_equal(M.level_spmv(sagb.OP_A0, 0, g["t_A0_in"]), g["t_A0_out"])
    for i in range(D):
        np.testing.assert_array_equal(M.level_spmv(sagb.OP_P, i, g[f"t_L{i}_P_in"]), g[f"t_L{i}_P_out"])
        np.testing.assert_array_equal(M.level_spmv(sagb.OP_R, i, g[f"t_L{i}_R_in"]), g[f"t_L{i}_R_out"])
        if i < D - 1:
            np.testing.assert_array_equal(M.level_spmv(sagb.OP_CA, i, g[f"t_L{i}_CA_in"]), g[f"t_L{i}_CA_out"])
    for l in range(D):
        np.testing.assert_array_equal(M.level_spmv(sagb.OP_U, l, g[f"t_S{l}_U_in"]), g[f"t_S{l}_U_out"])
        np.testing.assert_array_equal(M.sweep(l, g[f"t_S{l}_LD_in"]), g[f"t_S{l}_LD_out"], err_msg=f"sweep {l}")
        out = M.smooth(l, g[f"t_S{l}_LD_in"], inited=False)
        np.testing.assert_array_equal(out, g[f"t_S{l}_pre_out"])
        out = M.smooth(l, g[f"t_S{l}_U_in"], out=out, inited=True)
        np.testing.assert_array_equal(out, g[f"t_S{l}_post_out"])
    np.testing.assert_array_equal(M.coarse_solve(g["t_LU_in"]), g["t_LU_out"])
    np.testing.assert_array_equal(M.precondition(g["t_V_in"]), g["t_V_out"])
    # the same V-cycle twice: the sweep schedule state resets itself
    np.testing.assert_array_equal(M.precondition(g["t_V_in"]), g["t_V_out"])
    M.close()


def _solver(ctx, g, case, prec, bits=None, fallback=1):
    keep = []
    dA = sagb.Matrix(ctx, sagb.MAT_F64, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"])
    if prec == sagb.INT:
        A = sagb.Matrix(ctx, sagb.MAT_FIXED, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], bit=30)
    elif prec == sagb.F64:
        A = dA
    else:
        A = sagb.Matrix(ctx, sagb.MAT_F32, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"])
    M = _amg(ctx, g, case, prec)
    m = int(g["cfg"][1])
    p = sagb.solver_params(m=m, frac_bits=int(g["bit"][0]) if bits is None else bits, overflow_fallback=fallback)
    S = sagb.Solver(ctx, prec, dA, A, M, p)
    keep += [dA, A, M]
    return S, keep


@pytest.mark.parametrize("case", ["p2d64", "p3d16", "cd3d16"])
def test_int_fgmres_cycle_bit_exact(ctx, case):
    """One FGMRESflex::Solve call with the reference's e0 injected: V, Z, H,
    c, s, e, y and x identical to the reference's."""
    g = of.load_golden(case)
    S, keep = _solver(ctx, g, case, sagb.INT)
    N, m = len(g["b_scaled"]), S.m
    r = g["b_scaled"].copy()
    x = np.zeros(N)
    V = np.zeros(N * (m + 1), np.int32)
    Z = np.zeros(N * (m + 1), np.int32)
    H = np.zeros((m + 1) * m, np.int64)
    c, s, e = np.zeros(m, np.int64), np.zeros(m, np.int64), np.zeros(m + 1, np.int64)
    y = np.zeros(m)
    it, conv = S.cycle(r, float(g["nrm_b"][0]), x, e0=seq_norm(r), dumps=[V, Z, H, c, s, e, y])
    assert it == int(g["cyc_iter"][0]) and conv == int(g["cyc_conv"][0])
    np.testing.assert_array_equal(V[:(it + 1) * N], g["cyc_V"][:(it + 1) * N])
    np.testing.assert_array_equal(Z[:it * N], g["cyc_Z"][:it * N])
    mask = np.zeros((m, m + 1), bool)
    for j in range(it):
        mask[j, : j + 2] = True
    np.testing.assert_array_equal(H[mask.ravel()], g["cyc_H"][mask.ravel()])
    np.testing.assert_array_equal(c[:it], g["cyc_c"][:it])
    np.testing.assert_array_equal(s[:it], g["cyc_s"][:it])
    np.testing.assert_array_equal(e[:it + 1], g["cyc_e"][:it + 1])
    np.testing.assert_array_equal(y[:it], g["cyc_y"][:it])
    np.testing.assert_array_equal(x, g["cyc_x"])
    S.close()


@pytest.mark.parametrize("case", ["p2d64", "p3d16", "cd3d16", "vc3d16", "s27n14", "p3d16bj", "p3d16js", "p2d64js"])
def test_int_full_solve(ctx, case):
    g = of.load_golden(case)
    S, keep = _solver(ctx, g, case, sagb.INT)
    x = np.zeros(len(g["b_scaled"]))
    it, conv = S.solve(g["b_scaled"], float(g["nrm_b"][0]), x)
    assert conv == 1
    assert abs(it - int(g["int_iter"][0])) <= 2, (it, int(g["int_iter"][0]))
    assert explicit_res(g, x) <= 1e-10
    S.close()


def test_int_overflow_detected_and_recovered(ctx):
    """The reference's int solve overflows int32 on this system with its rule
    bit (F=29) and then divides by zero; the GPU solver flags the overflow,
    drops to F-1 and converges."""
    g = of.load_golden("an2d64")
    S, keep = _solver(ctx, g, "an2d64", sagb.INT, bits=29, fallback=1)
    x = np.zeros(len(g["b_scaled"]))
    it, conv = S.solve(g["b_scaled"], float(g["nrm_b"][0]), x)
    hist, flags = S.history()
    assert flags & (sagb.FLAG_OVERFLOW | sagb.FLAG_NORM_OVERFLOW | sagb.FLAG_DIVZERO | sagb.FLAG_PRECOND_OVERFLOW)
    bits = C.c_int()
    sagb.check(sagb.lib().sa_solver_bits(S.h, C.byref(bits)))
    assert bits.value < 29
    assert conv == 1 and explicit_res(g, x) <= 1e-10
    S.close()


@pytest.mark.parametrize("case", ["p2d64", "p3d16"])
def test_fp64_vcycle(ctx, case):
    g = of.load_golden(case)
    ctx.set_option(sagb.OPT_FP_EXACT, 1)
    try:
        M = _amg(ctx, g, case, sagb.F64)
        np.testing.assert_array_equal(M.precondition(g["d_t_V_in"]), g["d_t_V_out"])
        np.testing.assert_array_equal(M.sweep(0, g["d_t_V_in"]), g["d_t_S0_LD_out"])
        np.testing.assert_array_equal(M.coarse_solve(g["d_t_LU_in"]), g["d_t_LU_out"])
        M.close()
    finally:
        ctx.set_option(sagb.OPT_FP_EXACT, 0)
    M = _amg(ctx, g, case, sagb.F64)
    out = M.precondition(g["d_t_V_in"])
    ref = g["d_t_V_out"]
    assert np.linalg.norm(out - ref) <= FP_TOL * np.linalg.norm(ref)
    M.close()


@pytest.mark.parametrize("case", ["p2d64", "p3d16", "cd3d16", "vc3d16", "s27n14"])
def test_fp64_full_solve(ctx, case):
    g = of.load_golden(case)
    S, keep = _solver(ctx, g, case, sagb.F64)
    x = np.zeros(len(g["b_scaled"]))
    it, conv = S.solve(g["b_scaled"], float(g["nrm_b"][0]), x)
    assert conv == 1 and abs(it - int(g["fp64_iter"][0])) <= 1
    assert explicit_res(g, x) <= 1e-10
    # the FP64 solution agrees with the reference's FP64 solution
    ref = g["fp64_x"]
    assert np.linalg.norm(x - ref) <= 1e-6 * np.linalg.norm(ref)
    S.close()


@pytest.mark.parametrize("case", ["p3d16", "cd3d16"])
def test_fp32_full_solve(ctx, case):
    g = of.load_golden(case)
    S, keep = _solver(ctx, g, case, sagb.F32)
    x = np.zeros(len(g["b_scaled"]))
    it, conv = S.solve(g["b_scaled"], float(g["nrm_b"][0]), x)
    assert conv == 1 and abs(it - int(g["fp32_iter"][0])) <= 3
    assert explicit_res(g, x) <= 1e-10
    S.close()


@pytest.mark.parametrize("n", [48])
def test_int_vcycle_vs_oracle_3d(ctx, n):
    """A deeper hierarchy (3D 7-point n^3): GPU V-cycle == oracle V-cycle."""
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, n)
    xs, b = A.rhs(1)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    setup = sagb.Setup(sagb.INT, r, c, v)
    M = sagb.Amg(ctx, sagb.INT, setup=setup)
    keep = of.Keep()
    h = sv.oracle_amg(keep, setup)
    rng = np.random.default_rng(5)
    vin = rng.integers(-(1 << 29), 1 << 29, size=len(r) - 1).astype(np.int32)
    ref = np.zeros_like(vin)
    of.lib().or_vcycle_i32(C.byref(h), of.ptr(vin, of.i32p), of.ptr(ref, of.i32p))
    np.testing.assert_array_equal(M.precondition(vin), ref)
    M.close()


FP32_CASES = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14"]


@pytest.mark.parametrize("case", FP32_CASES)
def test_fp32_vcycle(ctx, case):
    """dfAMG<CSR<float>, SOR<ldtri::CSR<float>, ...>, float>::Precondition
    (INTAMG.hpp:13-134 with T = float) on the reference's own float hierarchy
    input: bit for bit in the sequential-order mode, within float rounding
    otherwise."""
    g = of.load_golden(case)
    ctx.set_option(sagb.OPT_FP_EXACT, 1)
    try:
        M = _amg(ctx, g, case, sagb.F32)
        np.testing.assert_array_equal(M.precondition(g["f_t_V_in"]), g["f_t_V_out"])
        if "f_t_S0_LD_out" in g:
            np.testing.assert_array_equal(M.sweep(0, g["f_t_V_in"]), g["f_t_S0_LD_out"])
        if "f_t_LU_in" in g:
            np.testing.assert_array_equal(M.coarse_solve(g["f_t_LU_in"]), g["f_t_LU_out"])
        M.close()
    finally:
        ctx.set_option(sagb.OPT_FP_EXACT, 0)
    M = _amg(ctx, g, case, sagb.F32)
    out = M.precondition(g["f_t_V_in"]).astype(np.float64)
    ref = g["f_t_V_out"].astype(np.float64)
    assert np.linalg.norm(out - ref) <= 1e-5 * np.linalg.norm(ref)
    M.close()


RULE_CASES = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14", "p3d16bj"]


@pytest.mark.parametrize("case", RULE_CASES)
def test_rule_bits(ctx, case):
    """The reference's bit rule (Work/main.cpp:153-161): one FP64 V-cycle of
    the scaled right-hand side, F from max|c| / ||b||.  The V-cycle output c is
    the reference's bit for bit in the sequential-order mode and within 1e-12
    otherwise; the ratio and the bit are the reference's."""
    g = of.load_golden(case)
    b, nrm_b = g["b_scaled"], float(g["nrm_b"][0])
    ref_c = g["c_bitrule"]
    ref_q = np.abs(ref_c).max() / nrm_b
    for exact in (1, 0):
        ctx.set_option(sagb.OPT_FP_EXACT, exact)
        try:
            M = _amg(ctx, g, case, sagb.F64)
            c_gpu = M.precondition(b)
            if exact:
                np.testing.assert_array_equal(c_gpu, ref_c)
            else:
                assert np.linalg.norm(c_gpu - ref_c) <= FP_TOL * np.linalg.norm(ref_c)
            q = sagb.rule_ratio(ctx, M, b, nrm_b)
            assert abs(q - ref_q) <= 1e-12 * ref_q
            assert sagb.rule_bits(ctx, M, b, nrm_b) == int(g["bit"][0])
            M.close()
        finally:
            ctx.set_option(sagb.OPT_FP_EXACT, 0)


@pytest.mark.parametrize("case,prec", [("p2d64", sagb.F64), ("p3d16", sagb.F64), ("cd3d16", sagb.F64),
                                       ("vc3d16", sagb.F64), ("s27n14", sagb.F64), ("p3d16", sagb.F32),
                                       ("cd3d16", sagb.F32)])
def test_fp_full_solve_sequential_order(ctx, case, prec):
    """Restarted(FGMRES<double|float>) with dfAMG in the sequential-order mode
    (every reduction in the reference's index order, no fused multiply-add):
    the iteration count and the solution are the reference's, within 1e-12
    relative (FP64) or float rounding carried through FP64 refinement (FP32)."""
    g = of.load_golden(case)
    key = "fp64" if prec == sagb.F64 else "fp32"
    ctx.set_option(sagb.OPT_FP_EXACT, 1)
    try:
        S, keep = _solver(ctx, g, case, prec)
        x = np.zeros(len(g["b_scaled"]))
        it, conv = S.solve(g["b_scaled"], float(g["nrm_b"][0]), x)
        S.close()
    finally:
        ctx.set_option(sagb.OPT_FP_EXACT, 0)
    assert conv == 1 and it == int(g[key + "_iter"][0]), (it, int(g[key + "_iter"][0]))
    ref = g[key + "_x"]
    err = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    assert err <= (FP_TOL if prec == sagb.F64 else 1e-6), err
