"""ctypes bindings of the sagb C ABI (include/sagb.h).

This is the Python face of the same library a C or C++ caller links: every
call goes through the C ABI of _build/libsagb.so.  It raises if the library
is missing; nothing here computes on the CPU in place of the GPU.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsagb.so")

SA_OK, SA_ERR_ARG, SA_ERR_CUDA, SA_ERR_SETUP, SA_ERR_NUMERIC = 0, 1, 2, 3, 4
FLAG_OVERFLOW, FLAG_TIMEOUT, FLAG_DIVZERO, FLAG_NORM_OVERFLOW = 1, 2, 4, 8
FLAG_PRECOND_OVERFLOW = 16  # an int32 wrap inside the V-cycle (FGMRES continues)
INT, F64, F32 = 0, 1, 2
MAT_FIXED, MAT_FLEX, MAT_F64, MAT_F32 = 0, 1, 2, 3
OP_A0, OP_CA, OP_P, OP_R, OP_LD, OP_U, OP_LUL, OP_LUU, OP_BJ, OP_COLOR = range(10)
GEN_POISSON2D, GEN_POISSON3D, GEN_ANISO2D, GEN_STENCIL27, GEN_CONVDIFF3D, GEN_VARCOEF3D = range(6)
OPT_FP_EXACT, OPT_GRAPHS, OPT_PDL, OPT_GPU_SETUP, OPT_CYCLE_GRAPH = 0, 1, 2, 3, 4

VP = C.c_void_p
I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)
F32P = C.POINTER(C.c_float)


class CsrView(C.Structure):
    _fields_ = [("n", C.c_int), ("m", C.c_int), ("nnz", C.c_int64), ("rptr", I32P), ("cind", I32P),
                ("val", VP), ("bit", C.c_int), ("dbit", C.c_int)]


class AmgParams(C.Structure):
    _fields_ = [("max_levels", C.c_int), ("theta", C.c_double), ("smoother_blocks", C.c_int),
                ("omega", C.c_double), ("smooth_iter", C.c_int), ("multicolor", C.c_int),
                ("max_colours", C.c_int), ("coarse_size", C.c_int), ("coarse_colours", C.c_int)]


class SolverParams(C.Structure):
    _fields_ = [("m", C.c_int), ("eps", C.c_double), ("max_outer", C.c_int), ("frac_bits", C.c_int),
                ("verbose", C.c_int), ("overflow_fallback", C.c_int), ("explicit_stop", C.c_int),
                ("cycle_bits", C.c_int)]


# name -> (restype, argtypes); the list is the ABI, checked by the CPU tests
SIGNATURES = {
    "sa_version": (C.c_char_p, []),
    "sa_last_error": (C.c_char_p, []),
    "sa_ctx_create": (C.c_int, [C.c_int, C.POINTER(VP)]),
    "sa_ctx_destroy": (C.c_int, [VP]),
    "sa_ctx_set_option": (C.c_int, [VP, C.c_int, C.c_int]),
    "sa_ctx_flags": (C.c_int, [VP, C.POINTER(C.c_uint), C.c_int]),
    "sa_ctx_launches": (C.c_int, [VP, C.POINTER(C.c_longlong)]),
    "sa_ctx_sync": (C.c_int, [VP]),
    "sa_ctx_stream": (C.c_int, [VP, C.POINTER(VP)]),
    "sa_device_alloc": (C.c_int, [VP, C.c_uint64, C.POINTER(VP)]),
    "sa_device_free": (C.c_int, [VP, VP]),
    "sa_memcpy": (C.c_int, [VP, VP, VP, C.c_uint64]),
    "sa_host_alloc": (C.c_int, [C.c_uint64, C.POINTER(VP)]),
    "sa_host_free": (C.c_int, [VP]),
    "sa_event_create": (C.c_int, [C.POINTER(VP)]),
    "sa_event_record": (C.c_int, [VP, VP]),
    "sa_event_elapsed_ms": (C.c_int, [VP, VP, C.POINTER(C.c_float)]),
    "sa_event_destroy": (C.c_int, [VP]),
    "sa_hcsr_read_mm": (C.c_int, [C.c_char_p, C.POINTER(VP)]),
    "sa_hcsr_read_mm_cached": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(VP)]),
    "sa_hcsr_save": (C.c_int, [VP, C.c_char_p]),
    "sa_hcsr_load": (C.c_int, [C.c_char_p, C.POINTER(VP)]),
    "sa_hcsr_create": (C.c_int, [C.c_int, C.c_int, I32P, I32P, F64P, C.POINTER(VP)]),
    "sa_hcsr_view": (C.c_int, [VP, C.POINTER(CsrView)]),
    "sa_hcsr_lmax1_scaling": (C.c_int, [VP, F64P]),
    "sa_hcsr_rhs": (C.c_int, [VP, C.c_uint64, F64P, F64P]),
    "sa_hcsr_destroy": (C.c_int, [VP]),
    "sa_gen": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_uint64, C.POINTER(VP)]),
    "sa_mat_create": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_int, I32P, I32P, F64P, C.POINTER(VP)]),
    "sa_mat_create_i32": (C.c_int, [VP, C.c_int, C.c_int, I32P, I32P, I32P, C.c_int, C.POINTER(VP)]),
    "sa_mat_destroy": (C.c_int, [VP]),
    "sa_mat_info": (C.c_int, [VP, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64),
                              C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sa_spmv": (C.c_int, [VP, VP, VP, VP]),
    "sa_amg_params_default": (None, [C.POINTER(AmgParams)]),
    "sa_setup_create": (C.c_int, [C.c_int, C.POINTER(AmgParams), C.c_int, I32P, I32P, F64P, C.POINTER(VP)]),
    "sa_setup_create_gpu": (C.c_int, [VP, C.c_int, C.POINTER(AmgParams), C.c_int, I32P, I32P, F64P, C.POINTER(VP)]),
    "sa_setup_derive": (C.c_int, [VP, C.c_int, C.POINTER(VP)]),
    "sa_setup_destroy": (C.c_int, [VP]),
    "sa_setup_depth": (C.c_int, [VP]),
    "sa_setup_view": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(CsrView)]),
    "sa_amg_create": (C.c_int, [VP, C.c_int, C.POINTER(AmgParams), C.c_int, I32P, I32P, F64P, C.POINTER(VP)]),
    "sa_amg_create_from_setup": (C.c_int, [VP, VP, C.POINTER(VP)]),
    "sa_amg_destroy": (C.c_int, [VP]),
    "sa_amg_depth": (C.c_int, [VP]),
    "sa_amg_precision": (C.c_int, [VP]),
    "sa_amg_precondition": (C.c_int, [VP, VP, VP, VP]),
    "sa_amg_smooth": (C.c_int, [VP, VP, C.c_int, VP, VP, C.c_int]),
    "sa_amg_sweep": (C.c_int, [VP, VP, C.c_int, VP, VP]),
    "sa_amg_sweep_noalloc": (C.c_int, [VP, VP, C.c_int, VP, VP]),
    "sa_amg_coarse_solve": (C.c_int, [VP, VP, VP, VP]),
    "sa_amg_level_spmv": (C.c_int, [VP, VP, C.c_int, C.c_int, VP, VP]),
    "sa_amg_level_info": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sa_solver_params_default": (None, [C.POINTER(SolverParams)]),
    "sa_solver_create": (C.c_int, [VP, C.c_int, VP, VP, VP, C.POINTER(SolverParams), C.POINTER(VP)]),
    "sa_solver_destroy": (C.c_int, [VP]),
    "sa_solver_solve": (C.c_int, [VP, VP, C.c_double, VP, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sa_solver_cycle": (C.c_int, [VP, VP, C.c_double, VP, F64P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(VP)]),
    "sa_solver_set_bits": (C.c_int, [VP, C.c_int]),
    "sa_solver_bits": (C.c_int, [VP, C.POINTER(C.c_int)]),
    "sa_solver_history": (C.c_int, [VP, F64P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_uint)]),
    "sa_rule_bits": (C.c_int, [VP, VP, VP, C.c_double, C.POINTER(C.c_int)]),
    "sa_rule_ratio": (C.c_int, [VP, VP, VP, C.c_double, C.POINTER(C.c_double)]),
    "sa_setup_features": (C.c_int, [VP, C.c_double, F32P]),
    "sa_mlp_create": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(VP)]),
    "sa_mlp_destroy": (C.c_int, [VP]),
    "sa_mlp_nparams": (C.c_int, [VP, C.POINTER(C.c_int64)]),
    "sa_mlp_get_params": (C.c_int, [VP, F32P]),
    "sa_mlp_set_params": (C.c_int, [VP, F32P]),
    "sa_mlp_set_norm": (C.c_int, [VP, F32P, F32P]),
    "sa_mlp_predict": (C.c_int, [VP, VP, F32P, C.c_int, F32P]),
    "sa_mlp_gradient": (C.c_int, [VP, VP, F32P, F32P, F32P, C.c_int, F32P, C.POINTER(C.c_float)]),
    "sa_mlp_train": (C.c_int, [VP, VP, F32P, F32P, F32P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_uint64,
                               F32P]),
    "sa_mlp_select_bits": (C.c_int, [VP, VP, F32P, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_create": (C.c_int, [VP, C.c_int, I32P, C.POINTER(I32P), C.POINTER(I32P), C.POINTER(F64P), C.c_int,
                                  C.POINTER(AmgParams), C.c_int, C.POINTER(VP)]),
    "sa_batch_destroy": (C.c_int, [VP]),
    "sa_batch_info": (C.c_int, [VP, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_int64)]),
    "sa_batch_offsets": (C.c_int, [VP, C.POINTER(C.c_int64)]),
    "sa_batch_system_setup": (C.c_int, [VP, C.c_int, C.POINTER(VP)]),
    "sa_batch_precondition": (C.c_int, [VP, VP, VP, VP]),
    "sa_batch_autotune": (C.c_int, [VP, VP, C.c_int]),
    "sa_batch_set_colour_caps": (C.c_int, [VP, VP, C.c_int, I32P, C.c_int]),
    "sa_batch_colour_caps": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int), I32P]),
    "sa_batch_group": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_set_group": (C.c_int, [VP, C.c_int, C.c_int, C.c_int]),
    "sa_batch_sweep_form": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_compressed": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_fused_sweeps": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_ell": (C.c_int, [VP, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_tail": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_tail_selftest": (C.c_int, [VP, VP, C.c_int, C.c_double, C.POINTER(C.c_uint)]),
    "sa_batch_time_op": (C.c_int, [VP, VP, C.c_int, C.c_int, VP, VP, C.c_int, C.POINTER(C.c_float)]),
    "sa_batch_time_op_cold": (C.c_int, [VP, VP, C.c_int, C.c_int, VP, VP, C.c_int, C.POINTER(C.c_float)]),
    "sa_batch_rule_ratios": (C.c_int, [VP, VP, VP, VP, F64P]),
    "sa_batch_solve": (C.c_int, [VP, VP, C.POINTER(SolverParams), I32P, VP, VP, VP, I32P, I32P, I32P]),
    "sa_profiler_range": (C.c_int, [C.c_int]),
    "sa_batch_fp_create": (C.c_int, [VP, VP, C.c_int, C.c_int, C.POINTER(VP)]),
    "sa_batch_fp_destroy": (C.c_int, [VP]),
    "sa_batch_fp_precondition": (C.c_int, [VP, VP, VP, VP]),
    "sa_batch_fp_autotune": (C.c_int, [VP, VP, C.c_int]),
    "sa_batch_fp_time_vcycle": (C.c_int, [VP, VP, C.c_int, C.POINTER(C.c_float)]),
    "sa_batch_fp_fused_sweeps": (C.c_int, [VP, C.c_int, C.POINTER(C.c_int)]),
    "sa_batch_fp_solve": (C.c_int, [VP, VP, C.POINTER(SolverParams), VP, VP, VP, I32P, I32P]),
    "sa_batch_cycle_graphs": (C.c_int, [VP, VP, C.POINTER(C.c_int)]),
    "sa_batch_level_op": (C.c_int, [VP, VP, C.c_int, C.c_int, VP, VP]),
    "sa_batch_coarse_solve": (C.c_int, [VP, VP]),
    "sa_batch_level_info": (C.c_int, [VP, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
}

_lib = None


class SagbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sagb error {code}: {msg}")
        self.code = code


def lib():
    """Load libsagb.so (built by sc23-ad_gb300/build.py); raises if missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} not built; run sc23-ad_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code):
    if code != SA_OK:
        raise SagbError(code, lib().sa_last_error().decode())


def _ptr(a, t=VP):
    return a.ctypes.data_as(t) if isinstance(a, np.ndarray) else a


def ctype_of(precision):
    return {INT: np.int32, F64: np.float64, F32: np.float32}[precision]


def view_arrays(v, kind="f64"):
    """Copy a CsrView into numpy arrays (rptr, cind, val)."""
    n = v.n
    rptr = np.ctypeslib.as_array(v.rptr, shape=(n + 1,)).copy() if n >= 0 else None
    nnz = int(v.nnz)
    cind = np.ctypeslib.as_array(v.cind, shape=(nnz,)).copy() if nnz else np.zeros(0, np.int32)
    dt = {"f64": C.c_double, "i32": C.c_int32, "f32": C.c_float}[kind]
    if nnz:
        val = np.ctypeslib.as_array(C.cast(v.val, C.POINTER(dt)), shape=(nnz,)).copy()
    else:
        val = np.zeros(0, {"f64": np.float64, "i32": np.int32, "f32": np.float32}[kind])
    return rptr, cind, val


# ------------------------------------------------------------------ objects

class HostCsr:
    def __init__(self, handle):
        self.h = handle

    @staticmethod
    def generate(kind, nx, param=0.0, seed=0):
        h = VP()
        check(lib().sa_gen(kind, nx, param, seed, C.byref(h)))
        return HostCsr(h)

    @staticmethod
    def from_arrays(rptr, cind, val, m=None):
        rptr = np.ascontiguousarray(rptr, np.int32)
        cind = np.ascontiguousarray(cind, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        n = len(rptr) - 1
        h = VP()
        check(lib().sa_hcsr_create(n, n if m is None else m, _ptr(rptr, I32P), _ptr(cind, I32P),
                                   _ptr(val, F64P), C.byref(h)))
        return HostCsr(h)

    @staticmethod
    def read_mm(path, cache=None):
        """io::ReadMM; with cache, through a binary CSR file that is reused
        while it records this very Matrix Market file."""
        h = VP()
        if cache is None:
            check(lib().sa_hcsr_read_mm(path.encode(), C.byref(h)))
        else:
            check(lib().sa_hcsr_read_mm_cached(path.encode(), cache.encode(), C.byref(h)))
        return HostCsr(h)

    def save(self, path):
        check(lib().sa_hcsr_save(self.h, path.encode()))

    @staticmethod
    def load(path):
        h = VP()
        check(lib().sa_hcsr_load(path.encode(), C.byref(h)))
        return HostCsr(h)

    def arrays(self):
        v = CsrView()
        check(lib().sa_hcsr_view(self.h, C.byref(v)))
        return view_arrays(v, "f64")

    @property
    def n(self):
        v = CsrView()
        check(lib().sa_hcsr_view(self.h, C.byref(v)))
        return v.n

    def rhs(self, seed):
        n = self.n
        xs, b = np.zeros(n), np.zeros(n)
        check(lib().sa_hcsr_rhs(self.h, seed, _ptr(xs, F64P), _ptr(b, F64P)))
        return xs, b

    def lmax1_scaling(self, b):
        check(lib().sa_hcsr_lmax1_scaling(self.h, _ptr(b, F64P)))

    def close(self):
        if self.h:
            lib().sa_hcsr_destroy(self.h)
            self.h = None

    __del__ = close


def amg_params(max_levels=20, theta=0.8, smoother_blocks=0, omega=1.0, smooth_iter=1, multicolor=0, max_colours=0,
               coarse_size=0, coarse_colours=0):
    return AmgParams(max_levels, theta, smoother_blocks, omega, smooth_iter, multicolor, max_colours, coarse_size,
                     coarse_colours)


class Setup:
    """The AMG hierarchy (host arrays).  With a Context the Ruge-Stueben
    levels' strength split, transposes, interpolation and Galerkin products
    run on its GPU; the hierarchy is the same bit for bit."""

    def __init__(self, precision, rptr=None, cind=None, val=None, params=None, _handle=None, ctx=None):
        if _handle is not None:
            self.precision, self.h = precision, _handle
            return
        rptr = np.ascontiguousarray(rptr, np.int32)
        cind = np.ascontiguousarray(cind, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        p = params or amg_params()
        self.precision = precision
        self.h = VP()
        if ctx is None:
            check(lib().sa_setup_create(precision, C.byref(p), len(rptr) - 1, _ptr(rptr, I32P), _ptr(cind, I32P),
                                        _ptr(val, F64P), C.byref(self.h)))
        else:
            check(lib().sa_setup_create_gpu(ctx.h, precision, C.byref(p), len(rptr) - 1, _ptr(rptr, I32P),
                                            _ptr(cind, I32P), _ptr(val, F64P), C.byref(self.h)))

    def derive(self, precision):
        """The same coarsening in another precision."""
        h = VP()
        check(lib().sa_setup_derive(self.h, precision, C.byref(h)))
        return Setup(precision, _handle=h)

    @property
    def depth(self):
        return lib().sa_setup_depth(self.h)

    def view(self, op, level=0):
        v = CsrView()
        check(lib().sa_setup_view(self.h, op, level, C.byref(v)))
        if op == OP_BJ:
            return np.ctypeslib.as_array(v.rptr, shape=(v.n + 1,)).copy()
        if op == OP_COLOR:
            return np.ctypeslib.as_array(v.rptr, shape=(v.n,)).copy()
        kind = {INT: "i32", F64: "f64", F32: "f32"}[self.precision]
        r, c, val = view_arrays(v, kind)
        return r, c, val, v.bit, v.dbit, v.m

    def close(self):
        if self.h:
            lib().sa_setup_destroy(self.h)
            self.h = None

    __del__ = close


class Context:
    def __init__(self, device=0):
        self.h = VP()
        check(lib().sa_ctx_create(device, C.byref(self.h)))

    def set_option(self, opt, value):
        check(lib().sa_ctx_set_option(self.h, opt, int(value)))

    def flags(self, clear=False):
        f = C.c_uint()
        check(lib().sa_ctx_flags(self.h, C.byref(f), int(clear)))
        return f.value

    def launches(self):
        n = C.c_longlong()
        check(lib().sa_ctx_launches(self.h, C.byref(n)))
        return n.value

    def sync(self):
        check(lib().sa_ctx_sync(self.h))

    def stream(self):
        s = VP()
        check(lib().sa_ctx_stream(self.h, C.byref(s)))
        return s.value

    def close(self):
        if self.h:
            lib().sa_ctx_destroy(self.h)
            self.h = None


class DeviceArray:
    """Device buffer owned through the C ABI (no torch needed)."""

    def __init__(self, ctx, shape, dtype):
        self.ctx = ctx
        self.dtype = np.dtype(dtype)
        self.shape = (shape,) if np.isscalar(shape) else tuple(shape)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self.ptr = VP()
        check(lib().sa_device_alloc(ctx.h, max(self.nbytes, 16), C.byref(self.ptr)))

    @staticmethod
    def from_host(ctx, a):
        a = np.ascontiguousarray(a)
        d = DeviceArray(ctx, a.shape, a.dtype)
        d.upload(a)
        return d

    def upload(self, a):
        a = np.ascontiguousarray(a, self.dtype)
        check(lib().sa_memcpy(self.ctx.h, self.ptr, a.ctypes.data_as(VP), a.nbytes))

    def download(self, out=None):
        out = np.empty(self.shape, self.dtype) if out is None else out
        check(lib().sa_memcpy(self.ctx.h, out.ctypes.data_as(VP), self.ptr, self.nbytes))
        return out

    def close(self):
        if self.ptr:
            lib().sa_device_free(self.ctx.h, self.ptr)
            self.ptr = None

    __del__ = close


class PinnedArray:
    """Page-locked host buffer exposed as a numpy array (.a)."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        n = int(np.prod((shape,) if np.isscalar(shape) else shape))
        self.ptr = VP()
        check(lib().sa_host_alloc(max(n * dtype.itemsize, 16), C.byref(self.ptr)))
        buf = (C.c_char * (n * dtype.itemsize)).from_address(self.ptr.value)
        self.a = np.frombuffer(buf, dtype=dtype, count=n)

    def close(self):
        if self.ptr:
            self.a = None
            lib().sa_host_free(self.ptr)
            self.ptr = None

    __del__ = close


class Event:
    def __init__(self):
        self.h = VP()
        check(lib().sa_event_create(C.byref(self.h)))

    def record(self, ctx):
        check(lib().sa_event_record(ctx.h, self.h))

    def elapsed_ms(self, later):
        ms = C.c_float()
        check(lib().sa_event_elapsed_ms(self.h, later.h, C.byref(ms)))
        return ms.value

    def close(self):
        if self.h:
            lib().sa_event_destroy(self.h)
            self.h = None

    __del__ = close


def _arg(x):
    if isinstance(x, PinnedArray):
        return x.ptr
    if isinstance(x, DeviceArray):
        return x.ptr
    if isinstance(x, np.ndarray):
        return x.ctypes.data_as(VP)
    return x


class Matrix:
    def __init__(self, ctx, kind, rptr, cind, val, bit=30, m=None):
        rptr = np.ascontiguousarray(rptr, np.int32)
        cind = np.ascontiguousarray(cind, np.int32)
        n = len(rptr) - 1
        self.ctx = ctx
        self.h = VP()
        if kind == "i32":
            val = np.ascontiguousarray(val, np.int32)
            check(lib().sa_mat_create_i32(ctx.h, n, n if m is None else m, _ptr(rptr, I32P), _ptr(cind, I32P),
                                          _ptr(val, I32P), bit, C.byref(self.h)))
        else:
            val = np.ascontiguousarray(val, np.float64)
            check(lib().sa_mat_create(ctx.h, kind, bit, n, n if m is None else m, _ptr(rptr, I32P),
                                      _ptr(cind, I32P), _ptr(val, F64P), C.byref(self.h)))
        self.info()

    def info(self):
        n, m, nnz, bit, prec = C.c_int(), C.c_int(), C.c_int64(), C.c_int(), C.c_int()
        check(lib().sa_mat_info(self.h, C.byref(n), C.byref(m), C.byref(nnz), C.byref(bit), C.byref(prec)))
        self.n, self.m, self.nnz, self.bit, self.precision = n.value, m.value, nnz.value, bit.value, prec.value
        return self

    def spmv(self, x, y=None):
        if y is None:
            y = np.zeros(self.n, ctype_of(self.precision))
        check(lib().sa_spmv(self.ctx.h, self.h, _arg(x), _arg(y)))
        return y

    def close(self):
        if self.h:
            lib().sa_mat_destroy(self.h)
            self.h = None


class Amg:
    def __init__(self, ctx, precision, rptr=None, cind=None, val=None, params=None, setup=None):
        self.ctx = ctx
        self.precision = precision
        self.h = VP()
        if setup is not None:
            check(lib().sa_amg_create_from_setup(ctx.h, setup.h, C.byref(self.h)))
        else:
            rptr = np.ascontiguousarray(rptr, np.int32)
            cind = np.ascontiguousarray(cind, np.int32)
            val = np.ascontiguousarray(val, np.float64)
            p = params or amg_params()
            check(lib().sa_amg_create(ctx.h, precision, C.byref(p), len(rptr) - 1, _ptr(rptr, I32P),
                                      _ptr(cind, I32P), _ptr(val, F64P), C.byref(self.h)))
        self.depth = lib().sa_amg_depth(self.h)
        self.n = self.level_info(OP_A0)[0]

    def level_info(self, op, level=0):
        n, m, nnz, bit, nlev = C.c_int(), C.c_int(), C.c_int64(), C.c_int(), C.c_int()
        check(lib().sa_amg_level_info(self.h, op, level, C.byref(n), C.byref(m), C.byref(nnz), C.byref(bit),
                                      C.byref(nlev)))
        return n.value, m.value, nnz.value, bit.value, nlev.value

    def _out(self, n, out):
        return np.zeros(n, ctype_of(self.precision)) if out is None else out

    def precondition(self, x, out=None):
        out = self._out(self.n, out)
        check(lib().sa_amg_precondition(self.ctx.h, self.h, _arg(x), _arg(out)))
        return out

    def smooth(self, level, x, out=None, inited=False):
        out = self._out(self.level_info(OP_LD, level)[0], out)
        check(lib().sa_amg_smooth(self.ctx.h, self.h, level, _arg(x), _arg(out), int(inited)))
        return out

    def sweep(self, level, x, out=None):
        out = self._out(self.level_info(OP_LD, level)[0], out)
        check(lib().sa_amg_sweep(self.ctx.h, self.h, level, _arg(x), _arg(out)))
        return out

    def coarse_solve(self, x, out=None):
        out = self._out(self.level_info(OP_LUL)[0], out)
        check(lib().sa_amg_coarse_solve(self.ctx.h, self.h, _arg(x), _arg(out)))
        return out

    def level_spmv(self, op, level, x, out=None):
        out = self._out(self.level_info(op, level)[0], out)
        check(lib().sa_amg_level_spmv(self.ctx.h, self.h, op, level, _arg(x), _arg(out)))
        return out

    def close(self):
        if self.h:
            lib().sa_amg_destroy(self.h)
            self.h = None


def solver_params(m=30, eps=1e-10, max_outer=None, frac_bits=29, verbose=0, overflow_fallback=1, explicit_stop=0,
                  cycle_bits=0):
    return SolverParams(m, eps, 1000 // m if max_outer is None else max_outer, frac_bits, verbose, overflow_fallback,
                        explicit_stop, cycle_bits)


class Solver:
    def __init__(self, ctx, precision, dA, A, M, params=None):
        self.ctx = ctx
        self.h = VP()
        p = params or solver_params()
        self.m = p.m
        check(lib().sa_solver_create(ctx.h, precision, dA.h, A.h, M.h, C.byref(p), C.byref(self.h)))

    def solve(self, b, nrm_b, x):
        it, conv = C.c_int(), C.c_int()
        check(lib().sa_solver_solve(self.h, _arg(b), nrm_b, _arg(x), C.byref(it), C.byref(conv)))
        return it.value, conv.value

    def cycle(self, r, nrm_b, x, e0=None, dumps=None):
        it, conv = C.c_int(), C.c_int()
        e0p = C.byref(C.c_double(e0)) if e0 is not None else None
        dp = None
        if dumps is not None:
            dp = (VP * 7)(*[d.ctypes.data_as(VP) if d is not None else None for d in dumps])
        check(lib().sa_solver_cycle(self.h, _arg(r), nrm_b, _arg(x), e0p, C.byref(it), C.byref(conv), dp))
        return it.value, conv.value

    def set_bits(self, bits):
        check(lib().sa_solver_set_bits(self.h, bits))

    def history(self):
        n, f = C.c_int(), C.c_uint()
        check(lib().sa_solver_history(self.h, None, 0, C.byref(n), C.byref(f)))
        h = np.zeros(n.value)
        check(lib().sa_solver_history(self.h, _ptr(h, F64P), n.value, C.byref(n), C.byref(f)))
        return h, f.value

    def close(self):
        if self.h:
            lib().sa_solver_destroy(self.h)
            self.h = None


def rule_ratio(ctx, M64, b, nrm_b):
    """max|M b| / ||b|| of one FP64 V-cycle (the rule's input, Work/main.cpp:153-161)."""
    q = C.c_double()
    check(lib().sa_rule_ratio(ctx.h, M64.h, _arg(b), nrm_b, C.byref(q)))
    return q.value


NUM_FEATURES = 20


def setup_features(setup_int, ratio):
    f = np.zeros(NUM_FEATURES, np.float32)
    check(lib().sa_setup_features(setup_int.h, ratio, _ptr(f, F32P)))
    return f


class Mlp:
    """The bit selector's 3-layer FP32 MLP (trained and run by this library's kernels)."""

    def __init__(self, ctx, n_in, hidden, n_out, seed=0):
        self.ctx, self.n_in, self.n_out = ctx, n_in, n_out
        self.h = VP()
        check(lib().sa_mlp_create(ctx.h, n_in, hidden, n_out, seed, C.byref(self.h)))

    @property
    def nparams(self):
        n = C.c_int64()
        check(lib().sa_mlp_nparams(self.h, C.byref(n)))
        return n.value

    def params(self):
        p = np.zeros(self.nparams, np.float32)
        check(lib().sa_mlp_get_params(self.h, _ptr(p, F32P)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        check(lib().sa_mlp_set_params(self.h, _ptr(p, F32P)))

    def set_norm(self, mu, sd):
        mu = np.ascontiguousarray(mu, np.float32)
        sd = np.ascontiguousarray(sd, np.float32)
        check(lib().sa_mlp_set_norm(self.h, _ptr(mu, F32P), _ptr(sd, F32P)))

    def predict(self, X):
        X = np.ascontiguousarray(np.atleast_2d(X), np.float32)
        Y = np.zeros((X.shape[0], self.n_out), np.float32)
        check(lib().sa_mlp_predict(self.ctx.h, self.h, _ptr(X, F32P), X.shape[0], _ptr(Y, F32P)))
        return Y

    def gradient(self, X, T, M):
        X, T, M = (np.ascontiguousarray(a, np.float32) for a in (X, T, M))
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_float()
        check(lib().sa_mlp_gradient(self.ctx.h, self.h, _ptr(X, F32P), _ptr(T, F32P), _ptr(M, F32P), X.shape[0],
                                    _ptr(g, F32P), C.byref(loss)))
        return loss.value, g

    def train(self, X, T, M, epochs, batch, lr, seed=0):
        X, T, M = (np.ascontiguousarray(a, np.float32) for a in (X, T, M))
        hist = np.zeros(epochs, np.float32)
        check(lib().sa_mlp_train(self.ctx.h, self.h, _ptr(X, F32P), _ptr(T, F32P), _ptr(M, F32P), X.shape[0],
                                 epochs, batch, lr, seed, _ptr(hist, F32P)))
        return hist

    def select_bits(self, feat, f_lo):
        f = np.ascontiguousarray(feat, np.float32)
        b = C.c_int()
        check(lib().sa_mlp_select_bits(self.ctx.h, self.h, _ptr(f, F32P), f_lo, C.byref(b)))
        return b.value

    def close(self):
        if self.h:
            lib().sa_mlp_destroy(self.h)
            self.h = None

    __del__ = close


class Batch:
    """Many systems (already scaled), nrhs right-hand sides each, solved together.

    The default parameters cap the colours of the finest level at 8 (a proper
    colouring of 7- and 27-point stencils) and of every coarser level at 2:
    coarse operators need up to ~150 colours for a proper colouring, each
    colour is one dependent step of the sweep (~1.6 us), and the capped split
    (rows beyond the cap act Jacobi-like within their colour) keeps the
    iteration count within about one iteration on the synthetic test
    families while the V-cycle has 6 colour steps per coarse level instead
    of ~16.  They also coarsen down to 400 rows instead of the reference's
    2000, so the dense coarsest LU is ~11x faster (0.05 instead of 0.55 ms
    per V-cycle at 128^3) for two or three more cheap levels, with the same
    iteration counts.  (100 rows is ~5 % faster still, but the bit
    selector's features describe the hierarchy, and its network was trained
    on 400-row hierarchies.)"""

    DEFAULT_MAX_COLOURS = 8     # the finest level: a proper colouring of 7- and 27-point stencils
    DEFAULT_COARSE_COLOURS = 2  # the levels below: fewer dependent colour steps (see the batched engine's notes)
    DEFAULT_COARSE_SIZE = 400

    def __init__(self, ctx, systems, nrhs=1, params=None, threads=0):
        self.ctx = ctx
        S = len(systems)
        self._keep = [(np.ascontiguousarray(r, np.int32), np.ascontiguousarray(c, np.int32),
                       np.ascontiguousarray(v, np.float64)) for r, c, v in systems]
        n = np.array([len(r) - 1 for r, _, _ in self._keep], np.int32)
        rp = (I32P * S)(*[_ptr(r, I32P) for r, _, _ in self._keep])
        cp = (I32P * S)(*[_ptr(c, I32P) for _, c, _ in self._keep])
        vp = (F64P * S)(*[_ptr(v, F64P) for _, _, v in self._keep])
        p = params or amg_params(max_colours=self.DEFAULT_MAX_COLOURS, coarse_size=self.DEFAULT_COARSE_SIZE,
                                 coarse_colours=self.DEFAULT_COARSE_COLOURS)
        self.h = VP()
        check(lib().sa_batch_create(ctx.h, S, _ptr(n, I32P), rp, cp, vp, nrhs, C.byref(p), threads,
                                    C.byref(self.h)))
        self._keep = None
        ns, nr, d, rows = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        check(lib().sa_batch_info(self.h, C.byref(ns), C.byref(nr), C.byref(d), C.byref(rows)))
        self.nsys, self.nrhs, self.depth, self.rows = ns.value, nr.value, d.value, rows.value
        off = np.zeros(self.nsys + 1, np.int64)
        check(lib().sa_batch_offsets(self.h, _ptr(off, C.POINTER(C.c_int64))))
        self.offsets = off

    def system_setup(self, s):
        h = VP()
        check(lib().sa_batch_system_setup(self.h, s, C.byref(h)))
        return Setup(INT, _handle=h)

    def precondition(self, x, out=None):
        out = np.zeros(self.rows * self.nrhs, np.int32) if out is None else out
        check(lib().sa_batch_precondition(self.ctx.h, self.h, _arg(x), _arg(out)))
        return out

    def level_info(self, level, op):
        n, m, nnz, nc = C.c_int(), C.c_int(), C.c_int64(), C.c_int()
        check(lib().sa_batch_level_info(self.h, level, op, C.byref(n), C.byref(m), C.byref(nnz), C.byref(nc)))
        return n.value, m.value, nnz.value, nc.value

    def level_op(self, level, op, x, out=None):
        n, m, _, _ = self.level_info(level, op)
        if out is None:
            out = np.zeros(n * self.nrhs, np.int32)
        check(lib().sa_batch_level_op(self.ctx.h, self.h, level, op, _arg(x), _arg(out)))
        return out

    def coarse_solve(self):
        check(lib().sa_batch_coarse_solve(self.ctx.h, self.h))

    OP_LU, OP_VCYCLE = 5, 6

    def time_op(self, level, op, x=None, out=None, reps=10, cold=False):
        """Milliseconds per call of one level operator (0 A, 1 LD sweep, 2 U,
        3 P, 4 R), the coarsest LU (5) or the V-cycle (6), timed as the solver
        runs it; x and out are DeviceArrays.  cold: the L2 flushed before every
        call (the operator read from HBM)."""
        ms = C.c_float()
        fn = lib().sa_batch_time_op_cold if cold else lib().sa_batch_time_op
        check(fn(self.ctx.h, self.h, level, op, None if x is None else x.ptr, None if out is None else out.ptr, reps,
                 C.byref(ms)))
        return ms.value

    def autotune(self, reps=3):
        check(lib().sa_batch_autotune(self.ctx.h, self.h, reps))

    def set_colour_caps(self, caps, threads=0):
        """Rebuild the smoother splits with colour caps per level (the last
        for deeper levels; 0 = proper colouring); launch shapes reset."""
        a = np.ascontiguousarray(caps, np.int32)
        check(lib().sa_batch_set_colour_caps(self.ctx.h, self.h, len(a), _ptr(a, I32P), threads))
        self.depth = self._depth()

    def colour_caps(self):
        n = C.c_int()
        check(lib().sa_batch_colour_caps(self.h, 0, C.byref(n), None))
        a = np.zeros(max(n.value, 1), np.int32)
        check(lib().sa_batch_colour_caps(self.h, len(a), C.byref(n), _ptr(a, I32P)))
        return [int(v) for v in a[:n.value]]

    def _depth(self):
        ns, nr, d, rows = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        check(lib().sa_batch_info(self.h, C.byref(ns), C.byref(nr), C.byref(d), C.byref(rows)))
        return d.value

    def tune_colour_caps(self, params, bits, b, nrm_b, x, candidates, reps=2, tune_reps=2):
        """Pick the colour caps by measured time to solution: for each
        candidate cap list, rebuild the splits, autotune the launch shapes and
        time `reps` solves of (b, nrm_b) into x (device arrays; x is zeroed
        before each solve) with CUDA events; keep the fastest.  Returns the
        table [(caps, ms per solve, iterations per pair)] and leaves the
        batch on the winner, tuned."""
        table = []
        zeros = np.zeros(self.rows * self.nrhs)
        for caps in candidates:
            self.set_colour_caps(caps)
            self.autotune(tune_reps)
            x.upload(zeros)
            self.solve(params, bits, b, nrm_b, x)  # warm-up (graphs captured)
            e0, e1 = Event(), Event()
            best = None
            for _ in range(reps):
                x.upload(zeros)
                self.ctx.sync()
                e0.record(self.ctx)
                it, cv, _ = self.solve(params, bits, b, nrm_b, x)
                e1.record(self.ctx)
                self.ctx.sync()
                ms = e0.elapsed_ms(e1)
                best = ms if best is None else min(best, ms)
            table.append((list(caps), best if cv.all() else float("inf"), [int(i) for i in it]))
        win = min(table, key=lambda t: t[1])
        self.set_colour_caps(win[0])
        self.autotune(tune_reps)
        return table

    def group(self, level, op):
        g = C.c_int()
        check(lib().sa_batch_group(self.h, level, op, C.byref(g)))
        return g.value

    def set_group(self, level, op, group):
        check(lib().sa_batch_set_group(self.h, level, op, group))

    SWEEP_PER_COLOUR, SWEEP_CLUSTER, SWEEP_PACKED, SWEEP_PACKED_COLOUR = 0, 1, 2, 3

    def compressed(self, level, op, set=-1):
        """16-bit column offsets for the level's A (op 0) or U (op 2); set 1 /
        0 chooses them."""
        f = C.c_int()
        check(lib().sa_batch_compressed(self.h, level, op, set, C.byref(f)))
        return f.value

    def fused_sweeps(self, set=-1):
        """Sweeps of one-colour levels fused into the neighbouring SpMVs: set 1
        / 0 turns it on / off; returns the levels fused."""
        f = C.c_int()
        check(lib().sa_batch_fused_sweeps(self.h, set, C.byref(f)))
        return f.value

    def ell(self, level, op, set=-1):
        """The ELL copy of the level's A (op 0) or U (op 2); set 1 / 0 chooses
        it (level-0 A: also in the Arnoldi SpMV)."""
        f = C.c_int()
        check(lib().sa_batch_ell(self.h, level, op, set, C.byref(f)))
        return f.value

    def tail(self, set=-1):
        """The V-cycle's persistent coarse tail: set t >= 1 runs levels t ..
        depth-1 and the coarsest LU in one cooperative launch, 0 turns it off;
        returns the tail's first level (0: none)."""
        f = C.c_int()
        check(lib().sa_batch_tail(self.h, set, C.byref(f)))
        return f.value

    def tail_selftest(self, level, timeout_ms=100.0):
        """One persistent-tail launch whose first grid barrier cannot complete:
        returns the status bits it raised (FLAG_TIMEOUT when the bounded wait
        ran out and every CTA returned)."""
        st = C.c_uint()
        check(lib().sa_batch_tail_selftest(self.ctx.h, self.h, level, timeout_ms, C.byref(st)))
        return st.value

    def sweep_form(self, level, set=-1):
        """The colour sweep's launch form at one level (0 a launch per colour,
        1 a cluster launch, 2 a cluster launch over the packed LD, 3 a launch
        per colour over LD packed in colour order); set >= 0 chooses it."""
        f = C.c_int()
        check(lib().sa_batch_sweep_form(self.h, level, set, C.byref(f)))
        return f.value

    def cycle_graphs(self):
        """Restart cycles of the last solve that ran as one graph each."""
        n = C.c_int()
        check(lib().sa_batch_cycle_graphs(self.h, None, C.byref(n)))
        return n.value

    def rule_ratios(self, b, nrm_b):
        q = np.zeros(self.nsys * self.nrhs)
        check(lib().sa_batch_rule_ratios(self.ctx.h, self.h, _arg(b), _arg(np.ascontiguousarray(nrm_b, np.float64)),
                                         _ptr(q, F64P)))
        return q

    def solve(self, params, bits, b, nrm_b, x):
        P = self.nsys * self.nrhs
        bits = np.ascontiguousarray(bits, np.int32)
        it, cv, fb = np.zeros(P, np.int32), np.zeros(P, np.int32), np.zeros(P, np.int32)
        check(lib().sa_batch_solve(self.ctx.h, self.h, C.byref(params), _ptr(bits, I32P), _arg(b),
                                   _arg(np.ascontiguousarray(nrm_b, np.float64)), _arg(x), _ptr(it, I32P),
                                   _ptr(cv, I32P), _ptr(fb, I32P)))
        return it, cv, fb

    def close(self):
        if self.h:
            lib().sa_batch_destroy(self.h)
            self.h = None

    __del__ = close


class BatchFp:
    """FP64-AMG-FGMRES (F64) or FP32-mixed AMG-FGMRES (F32) of an integer
    batch's systems, on its coarsening, level order and colour caps, run by
    the same batched GPU design (one launch per operation over all systems,
    graph-captured Arnoldi steps)."""

    def __init__(self, ctx, batch, precision=F64, threads=0):
        self.ctx = ctx
        self.batch = batch  # the integer batch must outlive this handle
        self.precision = precision
        self.rows, self.nrhs, self.nsys, self.offsets = batch.rows, batch.nrhs, batch.nsys, batch.offsets
        self.h = VP()
        check(lib().sa_batch_fp_create(ctx.h, batch.h, precision, threads, C.byref(self.h)))

    def precondition(self, x, out=None):
        out = np.zeros(self.rows * self.nrhs, ctype_of(self.precision)) if out is None else out
        check(lib().sa_batch_fp_precondition(self.ctx.h, self.h, _arg(x), _arg(out)))
        return out

    def autotune(self, reps=3):
        check(lib().sa_batch_fp_autotune(self.ctx.h, self.h, reps))

    def time_vcycle(self, reps=10):
        ms = C.c_float()
        check(lib().sa_batch_fp_time_vcycle(self.ctx.h, self.h, reps, C.byref(ms)))
        return ms.value

    def fused_sweeps(self, set=-1):
        """Sweeps of one-colour levels fused into the neighbouring SpMVs: set 1
        / 0 turns it on / off; returns the levels fused."""
        f = C.c_int()
        check(lib().sa_batch_fp_fused_sweeps(self.h, set, C.byref(f)))
        return f.value

    def cycle_graphs(self):
        """Restart cycles of the last solve that ran as one graph each."""
        n = C.c_int()
        check(lib().sa_batch_cycle_graphs(None, self.h, C.byref(n)))
        return n.value

    def solve(self, params, b, nrm_b, x):
        P = self.nsys * self.nrhs
        it, cv = np.zeros(P, np.int32), np.zeros(P, np.int32)
        check(lib().sa_batch_fp_solve(self.ctx.h, self.h, C.byref(params), _arg(b),
                                      _arg(np.ascontiguousarray(nrm_b, np.float64)), _arg(x), _ptr(it, I32P),
                                      _ptr(cv, I32P)))
        return it, cv

    def close(self):
        if self.h:
            lib().sa_batch_fp_destroy(self.h)
            self.h = None

    __del__ = close


def rule_bits(ctx, M64, b, nrm_b):
    bits = C.c_int()
    check(lib().sa_rule_bits(ctx.h, M64.h, _arg(b), nrm_b, C.byref(bits)))
    return bits.value
