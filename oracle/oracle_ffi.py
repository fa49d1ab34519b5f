"""ctypes bindings for the C oracle (oracle/oracle.h) and golden-fixture loaders.

Test infrastructure: the oracle is the checker, never the product.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # repository root
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liboracle.so")
GOLDEN = os.path.join(ROOT, "tests", "golden")

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)


class CsrI32(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("rptr", i32p), ("cind", i32p), ("val", i32p),
                ("bit", C.c_int), ("dbit", C.c_int)]


class CsrF64(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("rptr", i32p), ("cind", i32p), ("val", f64p)]


class CsrF32(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("rptr", i32p), ("cind", i32p), ("val", f32p)]


def _amg_struct(csr_t):
    class Amg(C.Structure):
        _fields_ = [("depth", C.c_int), ("A0", csr_t), ("CA", C.POINTER(csr_t)), ("P", C.POINTER(csr_t)),
                    ("R", C.POINTER(csr_t)), ("LD", C.POINTER(csr_t)), ("U", C.POINTER(csr_t)),
                    ("bj", C.POINTER(i32p)), ("nbj", C.c_int), ("smooth_iter", C.c_int),
                    ("LUL", csr_t), ("LUU", csr_t), ("order", C.POINTER(i32p))]
    return Amg


AmgI32 = _amg_struct(CsrI32)
AmgF64 = _amg_struct(CsrF64)
AmgF32 = _amg_struct(CsrF32)

_lib = None


def build_oracle():
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR, "port"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = C.CDLL(ORACLE_SO)
        ci, cf, cs = C.POINTER(CsrI32), C.POINTER(CsrF64), C.POINTER(CsrF32)
        ai, af, as_ = C.POINTER(AmgI32), C.POINTER(AmgF64), C.POINTER(AmgF32)
        sig = {
            "or_set_threads": (None, [C.c_int]),
            "or_spmv_i32": (C.c_int, [ci, i32p, i32p]),
            "or_ldtri_i32": (C.c_int, [ci, i32p, C.c_int, i32p, i32p]),
            "or_ldtri_order_i32": (C.c_int, [ci, i32p, i32p, i32p]),
            "or_ltri_i32": (C.c_int, [ci, i32p, i32p]),
            "or_dutri_i32": (C.c_int, [ci, i32p, i32p]),
            "or_lsqrt": (C.c_int64, [C.c_int64]),
            "or_dot_i32": (C.c_int64, [i32p, i32p, C.c_int, C.c_int]),
            "or_nrm2_i32": (C.c_int64, [i32p, C.c_int]),
            "or_axpy_i32": (None, [C.c_int64, i32p, i32p, C.c_int, C.c_int]),
            "or_scal_i32": (None, [C.c_int64, i32p, C.c_int, C.c_int]),
            "or_axpy_d": (None, [C.c_double, i32p, f64p, C.c_int, C.c_int]),
            "or_ggen_i32": (C.c_int64, [C.c_int64, C.c_int64, i64p, i64p, C.c_int]),
            "or_grot_i32": (None, [C.c_int64, C.c_int64, i64p, i64p, C.c_int]),
            "or_smooth_i32": (None, [ai, C.c_int, i32p, i32p, C.c_int]),
            "or_lu_i32": (None, [ai, i32p, i32p]),
            "or_vcycle_i32": (None, [ai, i32p, i32p]),
            "or_fgmres_i32_cycle": (C.c_int, [ci, ai, C.c_int, C.c_double, C.c_int, f64p, C.c_double, f64p,
                                              i32p, i32p, i64p, i64p, i64p, i64p, f64p, f64p,
                                              C.POINTER(C.c_int), C.c_int]),
            "or_ir_solve_i32": (C.c_int, [cf, ci, ai, C.c_int, C.c_double, C.c_int, f64p, C.c_double, f64p,
                                          C.c_int, C.c_int]),
            "or_spmv_f64": (C.c_int, [cf, f64p, f64p]),
            "or_ldtri_f64": (C.c_int, [cf, i32p, C.c_int, f64p, f64p]),
            "or_ldtri_order_f64": (C.c_int, [cf, i32p, f64p, f64p]),
            "or_ltri_f64": (C.c_int, [cf, f64p, f64p]),
            "or_dutri_f64": (C.c_int, [cf, f64p, f64p]),
            "or_vcycle_f64": (None, [af, f64p, f64p]),
            "or_ir_solve_f64": (C.c_int, [cf, af, C.c_int, C.c_double, f64p, C.c_double, f64p, C.c_int, C.c_int]),
            "or_spmv_f32": (C.c_int, [cs, f32p, f32p]),
            "or_ldtri_f32": (C.c_int, [cs, i32p, C.c_int, f32p, f32p]),
            "or_ldtri_order_f32": (C.c_int, [cs, i32p, f32p, f32p]),
            "or_vcycle_f32": (None, [as_, f32p, f32p]),
            "or_ir_solve_f32": (C.c_int, [cf, cs, as_, C.c_int, C.c_double, f64p, C.c_double, f64p, C.c_int,
                                          C.c_int]),
            "or_nrm2_f64": (C.c_double, [f64p, C.c_int]),
            "or_set_cycle_bits": (None, [C.c_int]),
            "or_ir_solve_i32x": (C.c_int, [cf, ci, ai, C.c_int, C.c_double, C.c_int, f64p, C.c_double, f64p,
                                           C.c_int, C.c_int, f64p]),
            "or_setup_create": (C.c_void_p, [C.c_int, i32p, i32p, f64p, C.c_double, C.c_int, C.c_int,
                                             C.c_double, C.POINTER(C.c_int)]),
            "or_setup_destroy": (None, [C.c_void_p]),
            "or_setup_depth": (C.c_int, [C.c_void_p]),
            "or_setup_warnings": (C.c_long, [C.c_void_p]),
            "or_setup_amg_i32": (None, [C.c_void_p, ai]),
            "or_setup_amg_f64": (None, [C.c_void_p, af]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def ptr(a, t):
    return a.ctypes.data_as(t)


class Keep:
    """Holds numpy arrays alive while ctypes structs point into them."""

    def __init__(self):
        self.refs = []

    def arr(self, a, dtype):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a


def csr_i32(keep, rptr, cind, val, bit, dbit=0, m=None):
    r, c, v = keep.arr(rptr, np.int32), keep.arr(cind, np.int32), keep.arr(val, np.int32)
    n = len(r) - 1
    return CsrI32(n, n if m is None else m, ptr(r, i32p), ptr(c, i32p), ptr(v, i32p), int(bit), int(dbit))


def csr_f(keep, rptr, cind, val, dtype, m=None):
    r, c, v = keep.arr(rptr, np.int32), keep.arr(cind, np.int32), keep.arr(val, dtype)
    n = len(r) - 1
    if dtype == np.float64:
        return CsrF64(n, n if m is None else m, ptr(r, i32p), ptr(c, i32p), ptr(v, f64p))
    return CsrF32(n, n if m is None else m, ptr(r, i32p), ptr(c, i32p), ptr(v, f32p))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def g_csr_i32(keep, g, pfx):
    meta = g[pfx + "_meta"]
    return csr_i32(keep, g[pfx + "_rptr"], g[pfx + "_cind"], g[pfx + "_val"], meta[2], meta[3], m=int(meta[1]))


def g_csr_f(keep, g, pfx, dtype):
    meta = g[pfx + "_meta"]
    return csr_f(keep, g[pfx + "_rptr"], g[pfx + "_cind"], g[pfx + "_val"], dtype, m=int(meta[1]))


def golden_amg_i32(keep, g, bj=False):
    """Build an AmgI32 struct from the reference hierarchy stored in a fixture."""
    D = int(g["depth"][0])
    CA = (CsrI32 * max(D - 1, 1))(*[g_csr_i32(keep, g, f"L{i}_CA") for i in range(D - 1)])
    P = (CsrI32 * D)(*[g_csr_i32(keep, g, f"L{i}_P") for i in range(D)])
    R = (CsrI32 * D)(*[g_csr_i32(keep, g, f"L{i}_R") for i in range(D)])
    LD = (CsrI32 * D)(*[g_csr_i32(keep, g, f"S{l}_LD") for l in range(D)])
    U = (CsrI32 * D)(*[g_csr_i32(keep, g, f"S{l}_U") for l in range(D)])
    keep.refs += [CA, P, R, LD, U]
    h = AmgI32()
    h.depth = D
    h.A0 = g_csr_i32(keep, g, "A0")
    h.CA, h.P, h.R, h.LD, h.U = CA, P, R, LD, U
    if bj:
        arrs = [keep.arr(g[f"S{l}_bjsize"], np.int32) for l in range(D)]
        bjp = (i32p * D)(*[ptr(a, i32p) for a in arrs])
        keep.refs.append(bjp)
        h.bj = bjp
        h.nbj = len(arrs[0]) - 1
    h.smooth_iter = 1
    h.LUL = g_csr_i32(keep, g, "LU_L")
    h.LUU = g_csr_i32(keep, g, "LU_U")
    return h


def colour_order(colour):
    """Rows colour by colour, increasing inside a colour (the MC renumbering)."""
    return np.argsort(np.asarray(colour), kind="stable").astype(np.int32)


def set_orders(keep, h, orders):
    """Attach per-level sweep orders (arrays or None) to an oracle hierarchy."""
    arrs = [None if o is None else keep.arr(o, np.int32) for o in orders]
    op = (i32p * len(arrs))(*[ptr(a, i32p) if a is not None else i32p() for a in arrs])
    keep.refs.append(op)
    h.order = op
    return h


def golden_amg_f(keep, g, pfx, dtype):
    D = int(g[pfx + "depth"][0])
    st = CsrF64 if dtype == np.float64 else CsrF32
    A = AmgF64 if dtype == np.float64 else AmgF32
    CA = (st * max(D - 1, 1))(*[g_csr_f(keep, g, f"{pfx}L{i}_CA", dtype) for i in range(D - 1)])
    P = (st * D)(*[g_csr_f(keep, g, f"{pfx}L{i}_P", dtype) for i in range(D)])
    R = (st * D)(*[g_csr_f(keep, g, f"{pfx}L{i}_R", dtype) for i in range(D)])
    LD = (st * D)(*[g_csr_f(keep, g, f"{pfx}S{l}_LD", dtype) for l in range(D)])
    U = (st * D)(*[g_csr_f(keep, g, f"{pfx}S{l}_U", dtype) for l in range(D)])
    keep.refs += [CA, P, R, LD, U]
    h = A()
    h.depth = D
    h.A0 = csr_f(keep, g["Ascaled_rptr"], g["Ascaled_cind"], g["Ascaled_val"], dtype)
    h.CA, h.P, h.R, h.LD, h.U = CA, P, R, LD, U
    h.smooth_iter = 1
    h.LUL = g_csr_f(keep, g, pfx + "LU_L", dtype)
    h.LUU = g_csr_f(keep, g, pfx + "LU_U", dtype)
    return h


class OracleSetup:
    """The oracle's own AMG setup (oracle_setup.c) of an LMax1-scaled matrix:
    .h_i32 / .h_f64 are the intAMGflex / dfAMG hierarchy structs."""

    def __init__(self, rptr, cind, val, theta=0.8, max_levels=20, coarse_limit=2000, omega=1.0):
        self._keep = Keep()
        r = self._keep.arr(rptr, np.int32)
        c = self._keep.arr(cind, np.int32)
        v = self._keep.arr(val, np.float64)
        st = C.c_int()
        self.h = lib().or_setup_create(len(r) - 1, ptr(r, i32p), ptr(c, i32p), ptr(v, f64p), theta, max_levels,
                                       coarse_limit, omega, C.byref(st))
        if not self.h:
            raise RuntimeError(f"oracle setup failed (status {st.value})")
        self.depth = lib().or_setup_depth(self.h)
        self.h_i32 = AmgI32()
        lib().or_setup_amg_i32(self.h, C.byref(self.h_i32))
        self.h_f64 = AmgF64()
        lib().or_setup_amg_f64(self.h, C.byref(self.h_f64))

    def close(self):
        if self.h:
            lib().or_setup_destroy(self.h)
            self.h = None

    __del__ = close


def csr_arrays(c):
    """(rptr, cind, val) numpy copies of an oracle CSR view."""
    n = c.n
    rptr = np.ctypeslib.as_array(c.rptr, shape=(n + 1,)).copy()
    nnz = int(rptr[-1])
    if nnz == 0:
        return rptr, np.zeros(0, np.int32), np.zeros(0)
    cind = np.ctypeslib.as_array(c.cind, shape=(nnz,)).copy()
    val = np.ctypeslib.as_array(c.val, shape=(nnz,)).copy()
    return rptr, cind, val
