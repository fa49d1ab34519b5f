"""CPU checks: the C++ generators against the independent numpy ones, and the
C ABI library exports every function include/sagb.h declares (no GPU calls)."""
import os
import re
import sys

import numpy as np
import pytest

import sagb

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import gen_matrices as gm  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("kind,nx,param,seed,ref", [
    (sagb.GEN_POISSON2D, 17, 0.0, 0, lambda: gm.poisson2d(17)),
    (sagb.GEN_POISSON3D, 9, 0.0, 0, lambda: gm.poisson3d(9)),
    (sagb.GEN_ANISO2D, 13, 1e-3, 0, lambda: gm.aniso2d(13, 1e-3)),
    (sagb.GEN_STENCIL27, 7, 0.0, 11, lambda: gm.stencil27(7, 11)),
    (sagb.GEN_CONVDIFF3D, 8, 50.0, 0, lambda: gm.convdiff3d(8, 50.0)),
])
def test_generators_match_numpy(kind, nx, param, seed, ref):
    A = sagb.HostCsr.generate(kind, nx, param, seed)
    r, c, v = A.arrays()
    rr, cc, vv = ref()
    np.testing.assert_array_equal(r, rr)
    np.testing.assert_array_equal(c, cc)
    np.testing.assert_array_equal(v, vv)
    xs, b = A.rhs(12345)
    xs2, b2 = gm.rhs(rr, cc, vv, 12345)
    np.testing.assert_array_equal(xs, xs2)
    np.testing.assert_array_equal(b, b2)


def test_varcoef_close_to_numpy():
    # transcendental functions may differ in the last ulp between libm and numpy
    A = sagb.HostCsr.generate(sagb.GEN_VARCOEF3D, 6, 2.0, 7)
    r, c, v = A.arrays()
    rr, cc, vv = gm.varcoef3d(6, 2.0, 7)
    np.testing.assert_array_equal(r, rr)
    np.testing.assert_array_equal(c, cc)
    np.testing.assert_allclose(v, vv, rtol=1e-13)


def test_matrix_market_reader(tmp_path):
    rptr, cind, val = gm.poisson2d(9)
    p = tmp_path / "a.mtx"
    gm.write_mtx(str(p), rptr, cind, val)
    r, c, v = sagb.HostCsr.read_mm(str(p)).arrays()
    np.testing.assert_array_equal(r, rptr)
    np.testing.assert_array_equal(c, cind)
    np.testing.assert_array_equal(v, val)
    # symmetric storage (lower triangle) expands to the full matrix
    rows = np.repeat(np.arange(len(rptr) - 1), np.diff(rptr))
    low = cind <= rows
    with open(tmp_path / "s.mtx", "w") as f:
        f.write("%%MatrixMarket matrix coordinate real symmetric\n% comment\n")
        f.write(f"{len(rptr) - 1} {len(rptr) - 1} {int(low.sum())}\n")
        for a, b_, x in zip(rows[low], cind[low], val[low]):
            f.write(f"{a + 1} {b_ + 1} {x:.17g}\n")
    r, c, v = sagb.HostCsr.read_mm(str(tmp_path / "s.mtx")).arrays()
    np.testing.assert_array_equal(r, rptr)
    np.testing.assert_array_equal(c, cind)
    np.testing.assert_array_equal(v, val)


def test_bad_inputs_are_rejected_not_fatal(tmp_path):
    with pytest.raises(sagb.SagbError):
        sagb.HostCsr.read_mm(str(tmp_path / "missing.mtx"))
    (tmp_path / "bad.mtx").write_text("not a matrix\n")
    with pytest.raises(sagb.SagbError):
        sagb.HostCsr.read_mm(str(tmp_path / "bad.mtx"))
    with pytest.raises(sagb.SagbError):  # column index out of range
        sagb.HostCsr.from_arrays(np.array([0, 1]), np.array([5]), np.array([1.0]))
    with pytest.raises(sagb.SagbError):  # theta outside (0, 1]
        r, c, v = gm.poisson2d(5)
        sagb.Setup(sagb.INT, r, c, v, sagb.amg_params(theta=1.5))


def test_abi_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "sagb.h")).read()
    declared = set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sa_\w+)\s*\(", hdr, re.M))
    assert len(declared) > 40
    L = sagb.lib()
    for name in sorted(declared):
        assert hasattr(L, name), name
    assert declared == set(sagb.SIGNATURES), declared ^ set(sagb.SIGNATURES)


def test_no_gpu_context_fails_cleanly():
    # without a GPU the context call must return an error code, not abort
    import ctypes as C
    h = C.c_void_p()
    code = sagb.lib().sa_ctx_create(0, C.byref(h))
    if code == sagb.SA_OK:
        sagb.lib().sa_ctx_destroy(h)
        pytest.skip("a GPU is present")
    assert code == sagb.SA_ERR_CUDA
    assert sagb.lib().sa_last_error()


def _mm_text(n, rows, cols, vals, shape="general", split=False, extra=""):
    lines = [f"%%MatrixMarket matrix coordinate real {shape}", "% comment", f"{n} {n} {len(rows)}"]
    for k, (a, b_, x) in enumerate(zip(rows, cols, vals)):
        if split and k % 97 == 5:  # an entry broken over two lines (strtod skips the newline)
            lines.append(f"{a + 1} {b_ + 1}")
            lines.append(f"{float(x)!r}")
        else:
            lines.append(f"{a + 1} {b_ + 1} {float(x)!r}")
    return "\n".join(lines) + "\n" + extra


def test_mm_reader_parallel_parse_matches_reference_rules(tmp_path):
    """The parallel reader gives what a sequential strtol/strtod read gives:
    the same values (exact decimal round trip, signs, exponents, integers,
    zeros dropped), entries split across lines, extra lines after the
    declared count ignored, too few entries rejected."""
    rng = np.random.default_rng(4)
    n = 3000
    rows = rng.integers(0, n, size=60000)
    cols = rng.integers(0, n, size=60000)
    key = np.unique(rows.astype(np.int64) * n + cols)
    rows, cols = (key // n).astype(int), (key % n).astype(int)
    vals = rng.standard_normal(len(rows)) * 10.0 ** rng.integers(-12, 12, size=len(rows))
    vals[::50] = 0.0  # dropped on read
    vals[1::50] = np.round(vals[1::50])  # integral values written as e.g. 3.0
    keep = vals != 0
    rptr = np.zeros(n + 1, np.int32)
    np.add.at(rptr, rows[keep] + 1, 1)
    rptr = np.cumsum(rptr).astype(np.int32)
    order = np.lexsort((cols[keep], rows[keep]))
    for split, extra in ((False, ""), (True, ""), (False, "1 1 5.0\n2 2 6.0\n")):
        p = tmp_path / f"m{int(split)}{len(extra)}.mtx"
        p.write_text(_mm_text(n, rows, cols, vals, split=split, extra=extra))
        r, c, v = sagb.HostCsr.read_mm(str(p)).arrays()
        np.testing.assert_array_equal(r, rptr)
        np.testing.assert_array_equal(c, cols[keep][order])
        np.testing.assert_array_equal(v, vals[keep][order])
    p = tmp_path / "short.mtx"
    txt = _mm_text(n, rows, cols, vals).splitlines()
    p.write_text("\n".join(txt[:-10]) + "\n")
    with pytest.raises(sagb.SagbError):
        sagb.HostCsr.read_mm(str(p))


def test_binary_csr_cache(tmp_path):
    """The binary CSR file round-trips a matrix exactly; the cached reader
    writes it on the first read, reuses it while the Matrix Market file is
    unchanged, and re-reads the Matrix Market file once it changes."""
    import os
    rptr, cind, val = gm.poisson2d(40)
    A = sagb.HostCsr.from_arrays(rptr, cind, val)
    A.save(str(tmp_path / "a.csr"))
    r, c, v = sagb.HostCsr.load(str(tmp_path / "a.csr")).arrays()
    np.testing.assert_array_equal(r, rptr)
    np.testing.assert_array_equal(c, cind)
    np.testing.assert_array_equal(v, val)
    (tmp_path / "bad.csr").write_bytes(b"SACSR01\x00" + b"\x00" * 10)
    with pytest.raises(sagb.SagbError):
        sagb.HostCsr.load(str(tmp_path / "bad.csr"))
    mm, cache = tmp_path / "a.mtx", tmp_path / "a.mtx.csr"
    gm.write_mtx(str(mm), rptr, cind, val)
    r, c, v = sagb.HostCsr.read_mm(str(mm), cache=str(cache)).arrays()
    np.testing.assert_array_equal(v, val)
    assert cache.exists()
    stamp = os.stat(cache).st_mtime_ns
    r, c, v = sagb.HostCsr.read_mm(str(mm), cache=str(cache)).arrays()  # from the cache
    np.testing.assert_array_equal(v, val)
    assert os.stat(cache).st_mtime_ns == stamp
    # a changed source: scale the values, rewrite the file with a new modification time
    gm.write_mtx(str(mm), rptr, cind, 2 * val)
    os.utime(mm, ns=(stamp + 10**9, stamp + 10**9))
    r, c, v = sagb.HostCsr.read_mm(str(mm), cache=str(cache)).arrays()
    np.testing.assert_array_equal(v, 2 * val)
    r, c, v = sagb.HostCsr.load(str(cache)).arrays()
    np.testing.assert_array_equal(v, 2 * val)
