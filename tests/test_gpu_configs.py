"""GPU parity on the benchmark configurations themselves, not only on the small
reference fixtures.

The hierarchies here are the ones the benchmarks time: 3D 7-point Poisson 128^3
(2,097,152 rows; the plain drop-in with the reference's parameters and the
batched engine with its defaults), 3D convection-diffusion 128^3 with Peclet 50
(the bit selector's evaluation system) and a batch shaped like the 256-system
27-point workload (uneven cube sides 16..64, four right-hand sides).  At these
sizes the long coarse rows, the packed and cluster sweep forms, the cluster LU
and the 16-bit column offsets are the forms the autotuner picks, so every one
of them is checked here bit for bit against the C oracle's V-cycle
(intAMGflex::Precondition, Library/preconditioner/INTAMG.hpp:269-293, with the
natural or the colour-ordered SOR sweep) on the same hierarchy and input."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle_ffi as of
import sagb
import setup_views as sv

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    of.lib().or_set_threads(os.cpu_count() or 1)
    yield c
    c.close()


def _scaled(kind, n, prm=0.0, seed=1):
    A = sagb.HostCsr.generate(kind, n, prm)
    _, b = A.rhs(seed)
    A.lmax1_scaling(b)
    return A.arrays(), b


def _v0(b, bits=29):
    """The first Krylov vector the solver hands the V-cycle: (int)(b/||b|| 2^F)."""
    return np.trunc(b / np.linalg.norm(b) * float(1 << bits)).astype(np.int32)


def _oracle_vcycle(h, vin):
    x = np.ascontiguousarray(vin, np.int32)
    ref = np.zeros_like(x)
    of.lib().or_vcycle_i32(C.byref(h), of.ptr(x, of.i32p), of.ptr(ref, of.i32p))
    return ref


def _inputs(b, n, seed):
    rng = np.random.default_rng(seed)
    return [_v0(b), rng.integers(-(1 << 28), 1 << 28, size=n).astype(np.int32)]


def test_plain_vcycle_poisson128(ctx):
    """The plain drop-in (reference parameters, natural-order SOR, 2000-row
    coarsest level) on the headline system: 10 levels, coarse rows up to ~600
    entries, dependency depths of 382-1112 per sweep."""
    (r, c, v), b = _scaled(sagb.GEN_POISSON3D, 128)
    setup = sagb.Setup(sagb.INT, r, c, v)
    assert setup.depth >= 9
    M = sagb.Amg(ctx, sagb.INT, setup=setup)
    keep = of.Keep()
    h = sv.oracle_amg(keep, setup)
    for k, vin in enumerate(_inputs(b, len(b), 11)):
        ref = _oracle_vcycle(h, vin)
        np.testing.assert_array_equal(M.precondition(vin), ref, err_msg=f"input {k}")
        # twice in a row: the sweep schedules' epoch state carries over correctly
        np.testing.assert_array_equal(M.precondition(vin), ref, err_msg=f"input {k}, second call")
    M.close()


def _batch_forms_match(B, vin, ref, nrhs):
    """Every sweep form, lanes-per-row choice, column storage and the
    persistent tail give the oracle's V-cycle."""
    out = lambda: B.precondition(vin).reshape(B.rows, nrhs)  # noqa: E731
    forms_run = set()
    for form in (0, 1, 2, 3):
        for g in (1, 8, 32):
            n_set = 0
            for lv in range(B.depth):
                try:
                    B.sweep_form(lv, form)
                    n_set += 1
                except sagb.SagbError:
                    continue
                B.set_group(lv, 1, g)
            if n_set:
                forms_run.add(form)
            np.testing.assert_array_equal(out(), ref, err_msg=f"sweep form {form}, {g} lanes per row")
    assert forms_run == {0, 1, 2, 3}, forms_run
    for on in (1, 0):
        n_on = 0
        for lv in range(B.depth):
            for op in (0, 2):
                try:
                    B.compressed(lv, op, on)
                    B.set_group(lv, op, 4)
                    n_on += on
                except sagb.SagbError:
                    pass
        assert n_on > 0 or on == 0
        np.testing.assert_array_equal(out(), ref, err_msg=f"16-bit column offsets {on}")
    for on in (1, 0):
        for lv in range(B.depth):
            for op in (0, 2):
                try:
                    B.ell(lv, op, on)
                except sagb.SagbError:
                    pass
        np.testing.assert_array_equal(out(), ref, err_msg=f"ELL copies {on}")
    for t in (B.depth - 1, max(1, B.depth - 4)):
        assert B.tail(t) == t
        np.testing.assert_array_equal(out(), ref, err_msg=f"persistent tail from level {t}")
    B.tail(0)


def test_batched_vcycle_poisson128(ctx):
    """The headline engine: batched defaults (8 colours on the finest level,
    2 below, 400-row coarsest level), autotuned, then every form forced."""
    (r, c, v), b = _scaled(sagb.GEN_POISSON3D, 128)
    B = sagb.Batch(ctx, [(r, c, v)], 1)
    keep = of.Keep()
    h = sv.oracle_amg(keep, B.system_setup(0))
    ins = _inputs(b, len(b), 12)
    refs = [_oracle_vcycle(h, x) for x in ins]
    for x, ref in zip(ins, refs):
        np.testing.assert_array_equal(B.precondition(x), ref)
    B.autotune(2)
    for x, ref in zip(ins, refs):
        np.testing.assert_array_equal(B.precondition(x), ref, err_msg="after autotuning")
    assert B.ell(0, 0, 1) == 1  # the 7-point finest level has an ELL copy
    _batch_forms_match(B, ins[1], refs[1][:, None], 1)
    B.close()


def test_batched_vcycle_convdiff128(ctx):
    """Upwinded convection-diffusion 128^3, Peclet 50 (nonsymmetric): the
    V-cycle wraps int32 in its coarse levels at F = 29, and the wrapped values
    must still be the reference's."""
    (r, c, v), b = _scaled(sagb.GEN_CONVDIFF3D, 128, 50.0)
    B = sagb.Batch(ctx, [(r, c, v)], 1)
    B.autotune(2)
    keep = of.Keep()
    h = sv.oracle_amg(keep, B.system_setup(0))
    for k, x in enumerate(_inputs(b, len(b), 13)):
        np.testing.assert_array_equal(B.precondition(x), _oracle_vcycle(h, x), err_msg=f"input {k}")
    B.close()


def test_batched_vcycle_batch256_subset(ctx):
    """Eight systems of the 256-system workload's family (27-point SPD,
    diagonal 26 + U[0.1, 1], off-diagonals -1; sides 16..64 including both
    ends), four right-hand sides each, autotuned, every form forced."""
    sides = [16, 64, 23, 41, 57, 30, 48, 35]
    nrhs = 4
    systems = []
    for s, n in enumerate(sides):
        A = sagb.HostCsr.generate(sagb.GEN_STENCIL27, n, 0.0, seed=2024 + s)
        _, b = A.rhs(s + 1)
        A.lmax1_scaling(b)
        systems.append(A.arrays())
    B = sagb.Batch(ctx, systems, nrhs)
    rng = np.random.default_rng(14)
    vin = rng.integers(-(1 << 28), 1 << 28, size=B.rows * nrhs).astype(np.int32)
    vin2 = vin.reshape(B.rows, nrhs)
    ref = np.zeros_like(vin2)
    keep = of.Keep()
    for s in range(B.nsys):
        h = sv.oracle_amg(keep, B.system_setup(s))
        a, e = B.offsets[s], B.offsets[s + 1]
        for q in range(nrhs):
            ref[a:e, q] = _oracle_vcycle(h, vin2[a:e, q])
    np.testing.assert_array_equal(B.precondition(vin).reshape(B.rows, nrhs), ref)
    B.autotune(2)
    np.testing.assert_array_equal(B.precondition(vin).reshape(B.rows, nrhs), ref, err_msg="after autotuning")
    _batch_forms_match(B, vin, ref, nrhs)
    B.close()
