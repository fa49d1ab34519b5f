"""Pins the C oracle to the reference: every check compares the oracle with
arrays the reference's own classes produced (tests/golden, made by
oracle/ref_harness.cpp).  Integer results must be identical; FP64/FP32 results
too, because both sides run the same IEEE operations in the same order."""
import ctypes as C

import numpy as np
import pytest

import oracle_ffi as of

# "js": JacobiSORflex, whose LD holds only couplings to earlier chunks, so the
# natural-order sweep of the oracle is its chunk-ordered sweep
CASES_INT = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14", "p3d16bj", "p3d16js", "p2d64js"]


@pytest.fixture(scope="module")
def L():
    return of.lib()


def test_blas_int(L):
    g = of.load_golden("blas")
    for bit in (20, 25, 30):
        p = f"blas_b{bit}"
        x, y = g[p + "_x"].copy(), g[p + "_y"].copy()
        n = len(x)
        dot, nrm, a = (int(v) for v in g[p + "_scal"])
        assert L.or_dot_i32(of.ptr(x, of.i32p), of.ptr(y, of.i32p), n, bit) == dot
        assert L.or_nrm2_i32(of.ptr(x, of.i32p), n) == nrm
        y2 = y.copy()
        L.or_axpy_i32(a, of.ptr(x, of.i32p), of.ptr(y2, of.i32p), n, bit)
        np.testing.assert_array_equal(y2, g[p + "_axpy"])
        x2 = x.copy()
        L.or_scal_i32(a, of.ptr(x2, of.i32p), n, bit)
        np.testing.assert_array_equal(x2, g[p + "_scalv"])
        xd = g[p + "_xd_in"].copy()
        L.or_axpy_d(float(g[p + "_ad"][0]), of.ptr(x, of.i32p), of.ptr(xd, of.f64p), n, bit)
        np.testing.assert_array_equal(xd, g[p + "_axpyd"])
        for i in range(len(g[p + "_ga"])):
            c, s = C.c_int64(), C.c_int64()
            r = L.or_ggen_i32(int(g[p + "_ga"][i]), int(g[p + "_gb"][i]), C.byref(c), C.byref(s), bit)
            assert (r, c.value, s.value) == (int(g[p + "_gr"][i]), int(g[p + "_gc"][i]), int(g[p + "_gs"][i]))
            a_, b_ = C.c_int64(int(g[p + "_ra"][i])), C.c_int64(int(g[p + "_rb"][i]))
            L.or_grot_i32(c.value, s.value, C.byref(a_), C.byref(b_), bit)
            assert (a_.value, b_.value) == (int(g[p + "_ra_out"][i]), int(g[p + "_rb_out"][i]))
        for q, rr in zip(g[p + "_lq"], g[p + "_lr"]):
            assert L.or_lsqrt(int(q)) == int(rr)


def _spmv_check(L, keep, g, pfx, tin, tout):
    A = of.g_csr_i32(keep, g, pfx)
    xin = g[tin].copy()
    out = np.zeros(A.n, dtype=np.int32)
    L.or_spmv_i32(C.byref(A), of.ptr(xin, of.i32p), of.ptr(out, of.i32p))
    np.testing.assert_array_equal(out, g[tout])


@pytest.mark.parametrize("case", CASES_INT)
def test_int_kernels_and_vcycle(L, case):
    g = of.load_golden(case)
    keep = of.Keep()
    bj = case.endswith("bj")
    h = of.golden_amg_i32(keep, g, bj=bj)
    D = h.depth
    _spmv_check(L, keep, g, "A0", "t_A0_in", "t_A0_out")
    for i in range(D):
        _spmv_check(L, keep, g, f"L{i}_P", f"t_L{i}_P_in", f"t_L{i}_P_out")
        _spmv_check(L, keep, g, f"L{i}_R", f"t_L{i}_R_in", f"t_L{i}_R_out")
        if i < D - 1:
            _spmv_check(L, keep, g, f"L{i}_CA", f"t_L{i}_CA_in", f"t_L{i}_CA_out")
    for l in range(D):
        _spmv_check(L, keep, g, f"S{l}_U", f"t_S{l}_U_in", f"t_S{l}_U_out")
        LD = h.LD[l]
        xin = g[f"t_S{l}_LD_in"].copy()
        out = np.zeros(LD.n, dtype=np.int32)
        bjp = h.bj[l] if bj else None
        L.or_ldtri_i32(C.byref(LD), bjp, h.nbj, of.ptr(xin, of.i32p), of.ptr(out, of.i32p))
        np.testing.assert_array_equal(out, g[f"t_S{l}_LD_out"])
        out2 = np.zeros(LD.n, dtype=np.int32)
        L.or_smooth_i32(C.byref(h), l, of.ptr(xin, of.i32p), of.ptr(out2, of.i32p), 0)
        np.testing.assert_array_equal(out2, g[f"t_S{l}_pre_out"])
        uin = g[f"t_S{l}_U_in"].copy()
        L.or_smooth_i32(C.byref(h), l, of.ptr(uin, of.i32p), of.ptr(out2, of.i32p), 1)
        np.testing.assert_array_equal(out2, g[f"t_S{l}_post_out"])
    lin = g["t_LU_in"].copy()
    lout = np.zeros_like(lin)
    L.or_lu_i32(C.byref(h), of.ptr(lin, of.i32p), of.ptr(lout, of.i32p))
    np.testing.assert_array_equal(lout, g["t_LU_out"])
    vin = g["t_V_in"].copy()
    vout = np.zeros_like(vin)
    L.or_vcycle_i32(C.byref(h), of.ptr(vin, of.i32p), of.ptr(vout, of.i32p))
    np.testing.assert_array_equal(vout, g["t_V_out"])


@pytest.mark.parametrize("case", ["p2d64", "p3d16", "cd3d16"])
def test_int_fgmres_cycle(L, case):
    """One FGMRESflex::Solve call from r = b, x = 0: all state must match."""
    g = of.load_golden(case)
    keep = of.Keep()
    h = of.golden_amg_i32(keep, g)
    A = h.A0
    N, m = A.n, int(g["cfg"][1])
    bit = int(g["bit"][0])
    r = g["b_scaled"].copy()
    x = np.zeros(N)
    V = np.zeros(N * (m + 1), np.int32)
    Z = np.zeros(N * (m + 1), np.int32)
    H = np.zeros((m + 1) * m, np.int64)
    c, s, e = np.zeros(m, np.int64), np.zeros(m, np.int64), np.zeros(m + 1, np.int64)
    y = np.zeros(m)
    conv = C.c_int()
    it = L.or_fgmres_i32_cycle(C.byref(A), C.byref(h), m, 1e-10, bit, of.ptr(r, of.f64p), float(g["nrm_b"][0]),
                               of.ptr(x, of.f64p), of.ptr(V, of.i32p), of.ptr(Z, of.i32p), of.ptr(H, of.i64p),
                               of.ptr(c, of.i64p), of.ptr(s, of.i64p), of.ptr(e, of.i64p), of.ptr(y, of.f64p),
                               None, C.byref(conv), 0)
    assert it == int(g["cyc_iter"][0]) and conv.value == int(g["cyc_conv"][0])
    # only the columns the cycle wrote (the reference's buffers start uninitialised)
    np.testing.assert_array_equal(V[:(it + 1) * N], g["cyc_V"][:(it + 1) * N])
    np.testing.assert_array_equal(Z[:it * N], g["cyc_Z"][:it * N])
    mask = np.zeros((m, m + 1), bool)
    for j in range(it):
        mask[j, : j + 2] = True
    mask = mask.ravel()
    np.testing.assert_array_equal(H[mask], g["cyc_H"][mask])
    np.testing.assert_array_equal(c[:it], g["cyc_c"][:it])
    np.testing.assert_array_equal(s[:it], g["cyc_s"][:it])
    np.testing.assert_array_equal(e[:it + 1], g["cyc_e"][:it + 1])
    np.testing.assert_array_equal(y[:it], g["cyc_y"][:it])
    np.testing.assert_array_equal(x, g["cyc_x"])


@pytest.mark.parametrize("case", ["p2d64", "p3d16", "cd3d16", "vc3d16", "s27n14", "p3d16bj", "p3d16js", "p2d64js"])
def test_int_full_solve(L, case):
    g = of.load_golden(case)
    keep = of.Keep()
    h = of.golden_amg_i32(keep, g, bj=case.endswith("bj"))
    dA = of.csr_f(keep, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], np.float64)
    m = int(g["cfg"][1])
    b = g["b_scaled"].copy()
    x = np.zeros(h.A0.n)
    it = L.or_ir_solve_i32(C.byref(dA), C.byref(h.A0), C.byref(h), m, 1e-10, int(g["bit"][0]), of.ptr(b, of.f64p),
                           float(g["nrm_b"][0]), of.ptr(x, of.f64p), 1000 // m, 0)
    assert it == int(g["int_iter"][0])
    np.testing.assert_array_equal(x, g["int_x"])


@pytest.mark.parametrize("case", ["p2d64", "p3d16"])
def test_fp64_kernels(L, case):
    g = of.load_golden(case)
    keep = of.Keep()
    h = of.golden_amg_f(keep, g, "d_", np.float64)
    vin = g["d_t_V_in"].copy()
    vout = np.zeros_like(vin)
    L.or_vcycle_f64(C.byref(h), of.ptr(vin, of.f64p), of.ptr(vout, of.f64p))
    np.testing.assert_array_equal(vout, g["d_t_V_out"])
    o2 = np.zeros_like(vin)
    L.or_ldtri_f64(C.byref(h.LD[0]), None, 0, of.ptr(vin, of.f64p), of.ptr(o2, of.f64p))
    np.testing.assert_array_equal(o2, g["d_t_S0_LD_out"])


@pytest.mark.parametrize("case", ["p2d64", "p3d16"])
def test_fp64_full_solve(L, case):
    g = of.load_golden(case)
    keep = of.Keep()
    h = of.golden_amg_f(keep, g, "d_", np.float64)
    dA = h.A0
    m = int(g["cfg"][1])
    b = g["b_scaled"].copy()
    x = np.zeros(dA.n)
    it = L.or_ir_solve_f64(C.byref(dA), C.byref(h), m, 1e-10, of.ptr(b, of.f64p), float(g["nrm_b"][0]),
                           of.ptr(x, of.f64p), 1000 // m, 0)
    assert it == int(g["fp64_iter"][0])
    np.testing.assert_array_equal(x, g["fp64_x"])


def test_fp32_full_solve(L):
    g = of.load_golden("p3d16")
    keep = of.Keep()
    hf = of.golden_amg_f(keep, g, "f_", np.float32)
    dA = of.csr_f(keep, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], np.float64)
    m = int(g["cfg"][1])
    b = g["b_scaled"].copy()
    x = np.zeros(dA.n)
    it = L.or_ir_solve_f32(C.byref(dA), C.byref(hf.A0), C.byref(hf), m, 1e-10, of.ptr(b, of.f64p),
                           float(g["nrm_b"][0]), of.ptr(x, of.f64p), 1000 // m, 0)
    assert it == int(g["fp32_iter"][0])
    np.testing.assert_array_equal(x, g["fp32_x"])
