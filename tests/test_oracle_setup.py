"""The oracle's own AMG setup (oracle/oracle_setup.c) against the reference.

For every golden fixture the oracle builds the hierarchy from the same scaled
matrix the reference's driver built it from, and every array must equal the
reference's own (dumped by oracle/ref_harness.cpp): the integer operators of
intAMGflex (A0, coarse operators, interpolations, restrictions, the SOR split
of every level and the coarsest LU factors, with their fractional bits) and the
FP64 operators of dfAMG.  This pins the setup half of the oracle, which lets the
CPU baseline build its hierarchy without the product."""
import numpy as np
import pytest

import oracle_ffi as of

CASES = ["p2d64", "p3d16", "cd3d16", "vc3d16", "an2d64", "s27n14", "p3d16bj", "p3d16js", "p2d64js"]


def _same_i32(g, pfx, c):
    r, ci, v = of.csr_arrays(c)
    np.testing.assert_array_equal(r, g[pfx + "_rptr"], err_msg=pfx)
    np.testing.assert_array_equal(ci, g[pfx + "_cind"], err_msg=pfx)
    np.testing.assert_array_equal(v, g[pfx + "_val"], err_msg=pfx)
    meta = g[pfx + "_meta"]
    assert c.n == meta[0] and c.m == meta[1], pfx
    assert c.bit == meta[2] and c.dbit == meta[3], (pfx, c.bit, c.dbit, meta)


def _same_f64(g, pfx, c):
    r, ci, v = of.csr_arrays(c)
    np.testing.assert_array_equal(r, g[pfx + "_rptr"], err_msg=pfx)
    np.testing.assert_array_equal(ci, g[pfx + "_cind"], err_msg=pfx)
    np.testing.assert_array_equal(v, g[pfx + "_val"], err_msg=pfx)


@pytest.mark.parametrize("case", CASES)
def test_oracle_setup_equals_reference_hierarchy(case):
    g = of.load_golden(case)
    s = of.OracleSetup(g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"])
    D = int(g["depth"][0])
    assert s.depth == D
    h = s.h_i32
    # A0 = CSR<Fixed<30>> (its stored meta records 30 as the fixture's bit)
    r, ci, v = of.csr_arrays(h.A0)
    np.testing.assert_array_equal(v, g["A0_val"])
    for i in range(D):
        if i < D - 1:
            _same_i32(g, f"L{i}_CA", h.CA[i])
        _same_i32(g, f"L{i}_P", h.P[i])
        _same_i32(g, f"L{i}_R", h.R[i])
        # the oracle setup builds the SOR split (the BlockSOR and JacobiSOR splits are the product's)
        if not case.endswith(("bj", "js")):
            _same_i32(g, f"S{i}_LD", h.LD[i])
            _same_i32(g, f"S{i}_U", h.U[i])
    _same_i32(g, "LU_L", h.LUL)
    _same_i32(g, "LU_U", h.LUU)
    if "d_depth" in g and not case.endswith(("bj", "js")):
        d = s.h_f64
        for i in range(D):
            if i < D - 1:
                _same_f64(g, f"d_L{i}_CA", d.CA[i])
            _same_f64(g, f"d_L{i}_P", d.P[i])
            _same_f64(g, f"d_L{i}_R", d.R[i])
            _same_f64(g, f"d_S{i}_LD", d.LD[i])
            _same_f64(g, f"d_S{i}_U", d.U[i])
        _same_f64(g, "d_LU_L", d.LUL)
        _same_f64(g, "d_LU_U", d.LUU)
    s.close()
