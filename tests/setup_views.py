"""Oracle hierarchy structs built from the product's host setup arrays.

The product's setup (sagb.Setup) is pinned to the reference's own hierarchy by
test_setup_golden; these helpers hand the same arrays to the C oracle so that a
GPU V-cycle can be checked against the oracle on matrices that have no fixture
(generated 3D problems, the multicolour smoother)."""
import numpy as np

import oracle_ffi as of
import sagb


def _views(setup):
    g = {"depth": np.array([setup.depth])}
    D = setup.depth

    def put(pfx, op, level=0):
        r, c, v, bit, dbit, m = setup.view(op, level)
        g[pfx + "_rptr"], g[pfx + "_cind"], g[pfx + "_val"] = r, c, v
        g[pfx + "_meta"] = np.array([len(r) - 1, m, bit, dbit])

    put("A0", sagb.OP_A0)
    for i in range(D):
        if i < D - 1:
            put(f"L{i}_CA", sagb.OP_CA, i)
        put(f"L{i}_P", sagb.OP_P, i)
        put(f"L{i}_R", sagb.OP_R, i)
        put(f"S{i}_LD", sagb.OP_LD, i)
        put(f"S{i}_U", sagb.OP_U, i)
    put("LU_L", sagb.OP_LUL)
    put("LU_U", sagb.OP_LUU)
    return g


def colours(setup):
    """Per-level colour arrays of a multicolour setup (None for natural order)."""
    out = []
    for lv in range(setup.depth):
        try:
            out.append(setup.view(sagb.OP_COLOR, lv))
        except sagb.SagbError:
            out.append(None)
    return out


def oracle_amg(keep, setup):
    """An oracle hierarchy over the setup's arrays, with the multicolour sweep
    order attached when the setup has colours."""
    g = _views(setup)
    if setup.precision == sagb.INT:
        g["A0_meta"][2] = 30
        h = of.golden_amg_i32(keep, g)
    else:
        dt = np.float64 if setup.precision == sagb.F64 else np.float32
        g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"] = g["A0_rptr"], g["A0_cind"], g["A0_val"]
        h = of.golden_amg_f(keep, g, "", dt)
    cols = colours(setup)
    if any(c is not None for c in cols):
        of.set_orders(keep, h, [None if c is None else of.colour_order(c) for c in cols])
    return h
