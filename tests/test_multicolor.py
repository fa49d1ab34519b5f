"""The multicolour smoother variant on the host: colouring, split and oracle.

The reference renumbers a matrix into multicolour order and sweeps it with
ldtri::MCCSR (Library/matrix/trispmat.hpp:597-640) after a greedy colouring
(Library/helper/helper_graph.hpp:191-219).  This library keeps the natural
numbering and splits A in colour order instead: LD holds the couplings to
earlier colours and diag/omega (last in the row), U the (1-1/omega) diagonal
and the couplings to the same or later colours.  A forward sweep visiting the
rows colour by colour then computes exactly the renumbered Gauss-Seidel sweep,
and rows of one colour are independent, so the sweep has one level per colour.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_ffi as of
import sagb
import setup_views as sv


def _poisson(n):
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, n)
    xs, b = A.rhs(1)
    A.lmax1_scaling(b)
    return A, b


def _dense(r, c, v, n):
    D = np.zeros((n, n))
    for i in range(n):
        D[i, c[r[i]:r[i + 1]]] += v[r[i]:r[i + 1]]
    return D


@pytest.fixture(scope="module")
def mc_setups():
    A, b = _poisson(12)
    r, c, v = A.arrays()
    s64 = sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=1))
    si = s64.derive(sagb.INT)
    return (r, c, v), b, s64, si


def test_colouring_is_proper(mc_setups):
    _, _, s64, si = mc_setups
    for lv in range(s64.depth):
        col = s64.view(sagb.OP_COLOR, lv)
        r, c, v, *_ = s64.view(sagb.OP_A0 if lv == 0 else sagb.OP_CA, max(lv - 1, 0))
        rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
        off = rows != c
        assert (col[rows[off]] != col[c[off]]).all()
        assert col.min() == 0 and set(np.unique(col)) == set(range(col.max() + 1))
        # the integer hierarchy colours the same patterns
        np.testing.assert_array_equal(si.view(sagb.OP_COLOR, lv), col)
    # a 7-point stencil is 2-colourable, and the greedy colouring finds that
    assert s64.view(sagb.OP_COLOR, 0).max() == 1


def test_split_reconstructs_operator(mc_setups):
    _, _, s64, _ = mc_setups
    for lv in range(s64.depth):
        col = s64.view(sagb.OP_COLOR, lv)
        ar, ac, av, *_ = s64.view(sagb.OP_A0 if lv == 0 else sagb.OP_CA, max(lv - 1, 0))
        lr, lc, lvv, *_ = s64.view(sagb.OP_LD, lv)
        ur, uc, uv, *_ = s64.view(sagb.OP_U, lv)
        n = len(ar) - 1
        for i in range(n):
            row_l = lc[lr[i]:lr[i + 1]]
            assert row_l[-1] == i                                  # D^-1 last
            assert (col[row_l[:-1]] < col[i]).all()                # earlier colours only
            assert (col[uc[ur[i]:ur[i + 1]]][1:] >= col[i]).all()  # U: diag first, then the rest
        Ad = _dense(ar, ac, av, n)
        Ld = _dense(lr, lc, lvv, n)
        Ud = _dense(ur, uc, uv, n)
        diag = np.diag(Ad).copy()
        np.testing.assert_allclose(np.diag(Ld), 1.0 / diag, rtol=0, atol=0)
        Ld_off = Ld - np.diag(np.diag(Ld))
        np.testing.assert_array_equal(Ld_off + Ud - np.diag(np.diag(Ud)), Ad - np.diag(diag))


def test_bad_params_rejected():
    A, _ = _poisson(6)
    r, c, v = A.arrays()
    with pytest.raises(sagb.SagbError):
        sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=1, smoother_blocks=4))
    with pytest.raises(sagb.SagbError):
        sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=3))  # 2 is JacobiSORflex
    with pytest.raises(sagb.SagbError):
        sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=2, smoother_blocks=4))
    s = sagb.Setup(sagb.F64, r, c, v)
    with pytest.raises(sagb.SagbError):
        s.view(sagb.OP_COLOR, 0)   # natural-order setup has no colours


def test_oracle_colour_sweep_is_renumbered_gauss_seidel(mc_setups):
    """The ordered oracle sweep == forward GS on the colour-renumbered matrix."""
    (r, c, v), _, s64, _ = mc_setups
    col = s64.view(sagb.OP_COLOR, 0)
    n = len(r) - 1
    perm = of.colour_order(col)
    Ad = _dense(r, c, v, n)
    Ap = Ad[np.ix_(perm, perm)]
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n)
    # GS on the renumbered system: (D + L_p) y = x_p
    yp = np.linalg.solve(np.tril(Ap), x[perm])
    keep = of.Keep()
    lr, lc, lv, *_ = s64.view(sagb.OP_LD, 0)
    LD = of.csr_f(keep, lr, lc, lv, np.float64)
    out = np.zeros(n)
    of.lib().or_ldtri_order_f64(C.byref(LD), of.ptr(perm, of.i32p), of.ptr(x, of.f64p), of.ptr(out, of.f64p))
    np.testing.assert_allclose(out[perm], yp, rtol=1e-12, atol=1e-12)
    # within a colour the order does not matter: reversing each colour's rows
    # gives the same bits
    perm2 = np.concatenate([perm[col[perm] == k][::-1] for k in range(col.max() + 1)]).astype(np.int32)
    out2 = np.zeros(n)
    of.lib().or_ldtri_order_f64(C.byref(LD), of.ptr(perm2, of.i32p), of.ptr(x, of.f64p), of.ptr(out2, of.f64p))
    np.testing.assert_array_equal(out, out2)


def test_oracle_multicolour_solves(mc_setups):
    """AMG-preconditioned FGMRES with the multicolour smoother converges in the
    oracle, in FP64 and integer arithmetic, within a few iterations of the
    natural-order smoother."""
    (r, c, v), b, s64, si = mc_setups
    n = len(r) - 1
    keep = of.Keep()
    dA = of.csr_f(keep, r, c, v, np.float64)
    nrm_b = float(np.linalg.norm(b))
    s64n = sagb.Setup(sagb.F64, r, c, v)
    Ad = _dense(r, c, v, n)
    its = {}
    for name, st in (("mc", s64), ("nat", s64n)):
        h = sv.oracle_amg(keep, st)
        x = np.zeros(n)
        its[name] = of.lib().or_ir_solve_f64(C.byref(dA), C.byref(h), 30, 1e-10, of.ptr(b, of.f64p), nrm_b,
                                             of.ptr(x, of.f64p), 1000 // 30, 0)
        res = np.linalg.norm(b - Ad @ x) / nrm_b
        assert res <= 1e-9, (name, res)
        # integer solve, fraction bits by the rule of Work/main.cpp:153-161
        cb = np.zeros(n)
        of.lib().or_vcycle_f64(C.byref(h), of.ptr(b, of.f64p), of.ptr(cb, of.f64p))
        q = np.abs(cb).max() / nrm_b
        bit = 29 if q < 1 else 31 - (int(np.ceil(np.log2(int(q) + 1))) + 1)
        si_st = si if name == "mc" else s64n.derive(sagb.INT)
        hi = sv.oracle_amg(keep, si_st)
        iA = of.g_csr_i32(keep, sv._views(si_st), "A0")
        iA.bit = 30
        xi = np.zeros(n)
        it = of.lib().or_ir_solve_i32(C.byref(dA), C.byref(iA), C.byref(hi), 30, 1e-10, bit, of.ptr(b, of.f64p),
                                      nrm_b, of.ptr(xi, of.f64p), 1000 // 30, 0)
        assert np.linalg.norm(b - Ad @ xi) / nrm_b <= 1e-9
        its[name + "_int"] = it
    # on a 7-point stencil the colours are red/black; the Ruge-Stueben coarse
    # points are then one colour and the multicolour two-grid cycle is much
    # stronger than the natural-order one
    assert its["mc"] <= its["nat"] and its["mc_int"] <= its["nat_int"] + 3, its


def test_colour_caps_per_level():
    """max_colours caps the finest level's colours, coarse_colours the coarser
    levels' (rows beyond a cap join their least conflicting colour); the split
    still reconstructs each operator, and a negative cap is rejected."""
    A = sagb.HostCsr.generate(sagb.GEN_STENCIL27, 14)
    xs, b = A.rhs(1)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    s = sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=1, max_colours=8, coarse_colours=2, coarse_size=100))
    full = sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=1, coarse_size=100))
    assert s.depth >= 3
    assert s.view(sagb.OP_COLOR, 0).max() + 1 <= 8
    np.testing.assert_array_equal(s.view(sagb.OP_COLOR, 0), full.view(sagb.OP_COLOR, 0))  # 27-point: 8 suffice
    for lv in range(1, s.depth):
        col = s.view(sagb.OP_COLOR, lv)
        assert col.max() + 1 <= 2
        assert full.view(sagb.OP_COLOR, lv).max() + 1 > 2  # the cap binds below the finest level
        ar, ac, av, *_ = s.view(sagb.OP_CA, lv - 1)
        lr, lc, lvv, *_ = s.view(sagb.OP_LD, lv)
        ur, uc, uv, *_ = s.view(sagb.OP_U, lv)
        n = len(ar) - 1
        Ad, Ld, Ud = _dense(ar, ac, av, n), _dense(lr, lc, lvv, n), _dense(ur, uc, uv, n)
        Ld_off = Ld - np.diag(np.diag(Ld))
        np.testing.assert_array_equal(Ld_off + Ud - np.diag(np.diag(Ud)), Ad - np.diag(np.diag(Ad)))
    with pytest.raises(sagb.SagbError):
        sagb.Setup(sagb.F64, r, c, v, sagb.amg_params(multicolor=1, coarse_colours=-1))
