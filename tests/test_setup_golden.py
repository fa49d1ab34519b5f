"""The product's host AMG setup against the reference's hierarchy.

The reference's intAMGflex / dfAMG objects (dumped by oracle/ref_harness.cpp)
hold the integer and FP arrays the solve phase runs on; the product's setup
(sa_setup_* in the C ABI, no GPU involved) must produce the same arrays bit for
bit, because the integer operators are derived from FP64 values by truncation."""
import numpy as np
import pytest

import oracle_ffi as of
import sagb

CASES = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14", "p3d16bj", "p3d16js", "p2d64js"]


def _params(case):
    """SOR (the default), BlockSOR-40 ("bj") or JacobiSORflex ("js")."""
    return sagb.amg_params(smoother_blocks=40 if case.endswith("bj") else 0, multicolor=2 if case.endswith("js") else 0)


def _cmp(got, g, pfx, with_bits=True):
    r, c, v, bit, dbit, m = got
    meta = g[pfx + "_meta"]
    np.testing.assert_array_equal(r, g[pfx + "_rptr"], err_msg=pfx + " rptr")
    np.testing.assert_array_equal(c, g[pfx + "_cind"], err_msg=pfx + " cind")
    np.testing.assert_array_equal(v, g[pfx + "_val"], err_msg=pfx + " val")
    assert m == meta[1]
    if with_bits:
        assert (bit, dbit) == (meta[2], meta[3]), pfx


@pytest.mark.parametrize("case", CASES)
def test_lmax1_scaling(case):
    g = of.load_golden(case)
    A = sagb.HostCsr.from_arrays(g["in_rptr"], g["in_cind"], g["in_val"])
    b = g["in_b"].copy()
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    np.testing.assert_array_equal(r, g["Ascaled_rptr"])
    np.testing.assert_array_equal(c, g["Ascaled_cind"])
    np.testing.assert_array_equal(v, g["Ascaled_val"])
    np.testing.assert_array_equal(b, g["b_scaled"])


@pytest.mark.parametrize("case", CASES)
def test_int_hierarchy(case):
    g = of.load_golden(case)
    s = sagb.Setup(sagb.INT, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], _params(case))
    D = int(g["depth"][0])
    assert s.depth == D
    _cmp(s.view(sagb.OP_A0), g, "A0", with_bits=False)
    for i in range(D):
        if i < D - 1:
            _cmp(s.view(sagb.OP_CA, i), g, f"L{i}_CA")
        _cmp(s.view(sagb.OP_P, i), g, f"L{i}_P")
        _cmp(s.view(sagb.OP_R, i), g, f"L{i}_R")
        _cmp(s.view(sagb.OP_LD, i), g, f"S{i}_LD")
        _cmp(s.view(sagb.OP_U, i), g, f"S{i}_U", with_bits=False)
        if case.endswith("bj"):
            np.testing.assert_array_equal(s.view(sagb.OP_BJ, i), g[f"S{i}_bjsize"])
        if case.endswith("js"):
            # the sweep's colours are the reference's chunks (MCCSRflex c_size)
            cs = g[f"S{i}_csize"]
            np.testing.assert_array_equal(s.view(sagb.OP_COLOR, i), np.repeat(np.arange(len(cs) - 1), np.diff(cs)))
    _cmp(s.view(sagb.OP_LUL), g, "LU_L", with_bits=False)
    _cmp(s.view(sagb.OP_LUU), g, "LU_U")


@pytest.mark.parametrize("case,prec,pfx", [("p2d64", sagb.F64, "d_"), ("p3d16", sagb.F64, "d_"),
                                           ("p3d16", sagb.F32, "f_")])
def test_fp_hierarchy(case, prec, pfx):
    g = of.load_golden(case)
    s = sagb.Setup(prec, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], _params(case))
    D = int(g[pfx + "depth"][0])
    assert s.depth == D
    for i in range(D):
        if i < D - 1:
            _cmp(s.view(sagb.OP_CA, i), g, f"{pfx}L{i}_CA", with_bits=False)
        _cmp(s.view(sagb.OP_P, i), g, f"{pfx}L{i}_P", with_bits=False)
        _cmp(s.view(sagb.OP_R, i), g, f"{pfx}L{i}_R", with_bits=False)
        _cmp(s.view(sagb.OP_LD, i), g, f"{pfx}S{i}_LD", with_bits=False)
        _cmp(s.view(sagb.OP_U, i), g, f"{pfx}S{i}_U", with_bits=False)
    _cmp(s.view(sagb.OP_LUL), g, pfx + "LU_L", with_bits=False)
    _cmp(s.view(sagb.OP_LUU), g, pfx + "LU_U", with_bits=False)
