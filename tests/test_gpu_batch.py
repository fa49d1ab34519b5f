"""GPU parity of the batched solver: many systems of uneven size, several
right-hand sides each, one launch per operation.

Per system and right-hand side the batch must compute what the system's own
multicolour hierarchy computes: the batched V-cycle is compared bit for bit
with the C oracle's V-cycle on each system (colour-ordered sweeps), and with
the single-system GPU path; whole solves are compared by convergence, explicit
residual and iteration count with the single-system solver."""
import ctypes as C

import numpy as np
import pytest

import oracle_ffi as of
import sagb
import setup_views as sv

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sagb.Context(0)
    yield c
    c.close()


SYSTEMS = [(sagb.GEN_POISSON3D, 12, 0.0), (sagb.GEN_STENCIL27, 10, 0.0), (sagb.GEN_CONVDIFF3D, 14, 20.0),
           (sagb.GEN_POISSON2D, 40, 0.0), (sagb.GEN_POISSON3D, 17, 0.0), (sagb.GEN_VARCOEF3D, 13, 1.0)]


def _systems(specs, nrhs, seed=1):
    out, bs = [], []
    for k, (kind, n, prm) in enumerate(specs):
        A = sagb.HostCsr.generate(kind, n, prm, seed=k + 1)
        cols = []
        for r in range(nrhs):
            xs, b = A.rhs(seed + 100 * k + r)
            cols.append(b)
        B = np.stack(cols, 1)
        # LMax1Scaling scales A and one b; the other columns by the same row maxima
        r0, c0, v0 = A.arrays()
        rows = np.repeat(np.arange(len(r0) - 1), np.diff(r0))
        rmax = np.zeros(len(r0) - 1)
        np.maximum.at(rmax, rows, np.abs(v0))
        b0 = B[:, 0].copy()
        A.lmax1_scaling(b0)
        out.append(A.arrays())
        bs.append(B / rmax[:, None])
    return out, bs


def _interleave(batch, cols):
    v = np.zeros((batch.rows, batch.nrhs), cols[0].dtype)
    for s, c in enumerate(cols):
        v[batch.offsets[s]:batch.offsets[s + 1]] = c
    return v.ravel()


@pytest.mark.parametrize("nrhs", [1, 2, 4])
def test_batched_vcycle_bit_exact(ctx, nrhs):
    systems, _ = _systems(SYSTEMS, nrhs)
    B = sagb.Batch(ctx, systems, nrhs)
    assert B.nsys == len(SYSTEMS) and B.offsets[-1] == B.rows
    rng = np.random.default_rng(nrhs)
    vin = rng.integers(-(1 << 28), 1 << 28, size=B.rows * nrhs).astype(np.int32)
    out = B.precondition(vin).reshape(B.rows, nrhs)
    vin2 = vin.reshape(B.rows, nrhs)
    for s in range(B.nsys):
        setup = B.system_setup(s)
        keep = of.Keep()
        h = sv.oracle_amg(keep, setup)
        M = sagb.Amg(ctx, sagb.INT, setup=setup)
        a, b = B.offsets[s], B.offsets[s + 1]
        for r in range(nrhs):
            x = np.ascontiguousarray(vin2[a:b, r])
            ref = np.zeros_like(x)
            of.lib().or_vcycle_i32(C.byref(h), of.ptr(x, of.i32p), of.ptr(ref, of.i32p))
            np.testing.assert_array_equal(out[a:b, r], ref, err_msg=f"system {s} rhs {r}")
            np.testing.assert_array_equal(M.precondition(x), ref)
        M.close()
    # the autotuner changes launch shapes only, never results
    B.autotune(2)
    np.testing.assert_array_equal(B.precondition(vin).reshape(B.rows, nrhs), out)
    # nor does the sweep's launch form (per colour, cluster, packed cluster, packed per colour) or its
    # lanes per row
    for form in (0, 1, 2, 3):
        for g in (1, 4, 32):
            for lv in range(B.depth):
                try:
                    B.sweep_form(lv, form)
                except sagb.SagbError:
                    continue
                B.set_group(lv, 1, g)
            np.testing.assert_array_equal(B.precondition(vin).reshape(B.rows, nrhs), out, err_msg=f"form {form} G {g}")
    # nor does the persistent coarse tail (levels t .. depth-1 and the LU in one cooperative launch)
    for t in range(1, B.depth):
        assert B.tail(t) == t
        np.testing.assert_array_equal(B.precondition(vin).reshape(B.rows, nrhs), out, err_msg=f"tail from {t}")
    B.tail(0)
    # nor does the compressed column storage of A and U (16-bit offsets), on or off at every level
    for on in (1, 0):
        n_on = 0
        for lv in range(B.depth):
            for op in (0, 2):
                try:
                    B.compressed(lv, op, on)
                    B.set_group(lv, op, 2)  # a lane kernel (the stream form reads 32-bit columns)
                    n_on += on
                except sagb.SagbError:
                    pass
        assert n_on > 0 or on == 0
        np.testing.assert_array_equal(B.precondition(vin).reshape(B.rows, nrhs), out, err_msg=f"compressed {on}")
    B.close()


def test_packed_sweep_many_groups_and_long_rows(ctx):
    """The packed cluster sweep on a batch of many systems (one cluster per
    group of systems) whose coarse rows are longer than the entries a lane
    fetches ahead, compared with the one-launch-per-colour form."""
    specs = [(sagb.GEN_STENCIL27, 9 + (k % 5), 0.0) for k in range(40)]
    systems, _ = _systems(specs, 2)
    B = sagb.Batch(ctx, systems, 2)
    rng = np.random.default_rng(5)
    vin = rng.integers(-(1 << 28), 1 << 28, size=B.rows * 2).astype(np.int32)
    for lv in range(B.depth):
        B.sweep_form(lv, 0)
    ref = B.precondition(vin)
    for form in (2, 3):
        packed = 0
        for lv in range(B.depth):
            try:
                B.sweep_form(lv, form)
                packed += 1
            except sagb.SagbError:
                pass
            B.set_group(lv, 1, 1)  # one lane a row: rows longer than 4 entries take the tail loop
        assert packed >= 1
        np.testing.assert_array_equal(B.precondition(vin), ref, err_msg=f"form {form}")
    B.close()


def test_batched_solve_matches_single_system(ctx):
    nrhs = 2
    systems, bs = _systems(SYSTEMS, nrhs)
    B = sagb.Batch(ctx, systems, nrhs)
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(bs[s][:, r]) for s in range(B.nsys) for r in range(nrhs)])
    ratios = B.rule_ratios(b, nrm_b)
    bits = []
    for s in range(B.nsys):
        q = ratios[s * nrhs]
        bits.append(29 if q < 1 else 31 - (int(np.ceil(np.log2(int(q) + 1))) + 1))
    params = sagb.solver_params(m=20, explicit_stop=1)
    x = np.zeros(B.rows * nrhs)
    it, cv, fb = B.solve(params, bits, b, nrm_b, x)
    X = x.reshape(B.rows, nrhs)
    for s, (r, c, v) in enumerate(systems):
        rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
        a, e = B.offsets[s], B.offsets[s + 1]
        setup = B.system_setup(s)
        M = sagb.Amg(ctx, sagb.INT, setup=setup)
        dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
        iA = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
        S1 = sagb.Solver(ctx, sagb.INT, dA, iA, M, sagb.solver_params(m=20, frac_bits=bits[s], explicit_stop=1))
        for q in range(nrhs):
            p = s * nrhs + q
            xs = X[a:e, q]
            res = np.linalg.norm(bs[s][:, q] - np.bincount(rows, weights=v * xs[c], minlength=len(r) - 1))
            assert cv[p] == 1 and res / nrm_b[p] <= 1e-10, (s, q, it[p], res / nrm_b[p])
            x1 = np.zeros(len(r) - 1)
            it1, cv1 = S1.solve(np.ascontiguousarray(bs[s][:, q]), float(nrm_b[p]), x1)
            assert cv1 == 1 and abs(int(it[p]) - it1) <= 2, (s, q, it[p], it1)
        S1.close(); M.close()
    B.close()


def test_batched_overflow_falls_back_per_pair(ctx):
    """A pair whose fractional bits overflow the Arnoldi arithmetic is redone
    with fewer bits (wraps inside the V-cycle only cost convergence speed:
    FGMRES is flexible) while the other systems of the batch are not
    disturbed."""
    specs = [(sagb.GEN_POISSON3D, 12, 0.0), (sagb.GEN_ANISO2D, 64, 1e-3)]
    systems, bs = _systems(specs, 1)
    B = sagb.Batch(ctx, systems, 1)
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(x[:, 0]) for x in bs])
    params = sagb.solver_params(m=20, explicit_stop=1)
    x = np.zeros(B.rows)
    it, cv, fb = B.solve(params, [29, 30], b, nrm_b, x)
    assert cv.all(), (it, cv, fb)
    assert fb[0] == 29 and fb[1] <= 30
    B.close()


def test_copies_share_one_setup(ctx):
    """Copies of one matrix (the same arrays) share a setup; solved with
    different fractional bits, each copy matches the single-system solver."""
    systems, bs = _systems([(sagb.GEN_POISSON3D, 14, 0.0)], 1)
    r, c, v = systems[0]
    bits = [20, 25, 29]
    B = sagb.Batch(ctx, [(r, c, v)] * len(bits), 1)
    b = np.concatenate([bs[0][:, 0]] * len(bits))
    nrm = np.linalg.norm(bs[0][:, 0])
    x = np.zeros(B.rows)
    it, cv, fb = B.solve(sagb.solver_params(m=20, explicit_stop=1), bits, b, np.full(len(bits), nrm), x)
    setup = B.system_setup(0)
    M = sagb.Amg(ctx, sagb.INT, setup=setup)
    dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
    iA = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
    for k, f in enumerate(bits):
        S1 = sagb.Solver(ctx, sagb.INT, dA, iA, M, sagb.solver_params(m=20, frac_bits=f, explicit_stop=1))
        x1 = np.zeros(len(r) - 1)
        it1, cv1 = S1.solve(np.ascontiguousarray(bs[0][:, 0]), float(nrm), x1)
        assert cv[k] == cv1 and abs(int(it[k]) - it1) <= 2, (f, it[k], it1)
        S1.close()
    B.close()


def test_launch_options_do_not_change_results(ctx):
    """Graph replay of the V-cycle, programmatic dependent launch, the
    restart cycle as one graph gated on the device and the graph-timed
    operator clock change launch mechanics only: V-cycles and whole solves are
    identical bit for bit with each of them off."""
    nrhs = 2
    systems, bs = _systems(SYSTEMS, nrhs)
    B = sagb.Batch(ctx, systems, nrhs)
    rng = np.random.default_rng(9)
    vin = rng.integers(-(1 << 28), 1 << 28, size=B.rows * nrhs).astype(np.int32)
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(bs[s][:, r]) for s in range(B.nsys) for r in range(nrhs)])
    params = sagb.solver_params(m=20, explicit_stop=1)
    bits = [28] * B.nsys

    def run():
        out = B.precondition(vin)
        x = np.zeros(B.rows * nrhs)
        it, cv, fb = B.solve(params, bits, b, nrm_b, x)
        return out, x, it

    ref = run()
    # each restart cycle ran as one graph with its steps gated on the device;
    # the same solve step by step (a status read after every step) is identical
    assert B.cycle_graphs() > 0
    ctx.set_option(sagb.OPT_CYCLE_GRAPH, 0)
    try:
        got = run()
        assert B.cycle_graphs() == 0
        for k in range(3):
            np.testing.assert_array_equal(got[k], ref[k], err_msg="step by step")
    finally:
        ctx.set_option(sagb.OPT_CYCLE_GRAPH, 1)
    # a solve whose V-cycles run their coarse levels in the persistent tail
    for t in (1, B.depth - 1):
        B.tail(t)
        got = run()
        for k in range(3):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"tail from {t}")
    B.tail(0)
    # the Arnoldi SpMV and the V-cycle with compressed columns wherever they fit
    for lv in range(B.depth):
        for op in (0, 2):
            try:
                B.compressed(lv, op, 1)
                B.set_group(lv, op, 1)
            except sagb.SagbError:
                pass
    got = run()
    for k in range(3):
        np.testing.assert_array_equal(got[k], ref[k])
    try:
        for opt in (sagb.OPT_PDL, sagb.OPT_GRAPHS):
            ctx.set_option(opt, 0)
            got = run()
            np.testing.assert_array_equal(got[0], ref[0])
            np.testing.assert_array_equal(got[1], ref[1])
            np.testing.assert_array_equal(got[2], ref[2])
    finally:
        ctx.set_option(sagb.OPT_PDL, 1)
        ctx.set_option(sagb.OPT_GRAPHS, 1)
    x = sagb.DeviceArray.from_host(ctx, vin)
    y = sagb.DeviceArray(ctx, B.rows * nrhs, np.int32)
    for op in range(5):
        assert B.time_op(0, op, x, y, 3) > 0
    assert B.time_op(0, B.OP_LU, reps=3) > 0
    assert B.time_op(0, B.OP_VCYCLE, x, y, 3) > 0
    # cold timing (the L2 flushed before every call, the flush's time subtracted)
    assert B.time_op(0, 0, x, y, 3, cold=True) > 0
    x.close(); y.close()
    B.close()


def test_tail_barrier_timeout_is_detected(ctx):
    """Failure detection of the persistent tail's grid barrier without a GPU
    fault: a launch whose first barrier waits for one CTA more than the grid
    has runs out its bounded wait (50 ms), every CTA returns and the status
    reports the timeout; the context and the engine stay usable."""
    systems, _ = _systems(SYSTEMS, 1)
    B = sagb.Batch(ctx, systems, 1)
    vin = np.random.default_rng(12).integers(-(1 << 28), 1 << 28, size=B.rows).astype(np.int32)
    B.tail(0)
    ref = B.precondition(vin)
    st = B.tail_selftest(B.depth - 1, 50.0)
    assert st & sagb.FLAG_TIMEOUT
    assert B.tail() == 0  # the setting is restored
    np.testing.assert_array_equal(B.precondition(vin), ref)
    B.tail(1)
    np.testing.assert_array_equal(B.precondition(vin), ref)
    B.close()


def test_early_restart_matches_oracle(ctx):
    """sa_solver_params.cycle_bits: a pair's cycle ends once its estimate has
    fallen 2^K below the cycle's start.  Per system the batched solve takes
    the iterations of the oracle's Restarted(FGMRESflex) with the same rule
    on the same hierarchy (within 2: the FP64 residual norm is a parallel sum
    on the GPU) and far fewer than with full cycles."""
    nrhs = 1
    systems, bs = _systems(SYSTEMS[:4], nrhs)
    B = sagb.Batch(ctx, systems, nrhs)
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(bs[s][:, 0]) for s in range(B.nsys)])
    its = {}
    for K in (0, 12):
        x = np.zeros(B.rows)
        it, cv, fb = B.solve(sagb.solver_params(m=30, explicit_stop=1, cycle_bits=K), [29] * B.nsys, b, nrm_b, x)
        assert cv.all(), (K, it)
        its[K] = it
        for s, (r, c, v) in enumerate(systems):
            keep = of.Keep()
            h = sv.oracle_amg(keep, B.system_setup(s))
            dA = of.csr_f(keep, r, c, v, np.float64)
            bq = np.ascontiguousarray(bs[s][:, 0])
            xo = np.zeros(len(bq))
            res = C.c_double()
            of.lib().or_set_cycle_bits(K)
            try:
                it_o = of.lib().or_ir_solve_i32x(C.byref(dA), C.byref(h.A0), C.byref(h), 30, 1e-10, 29,
                                                 of.ptr(bq, of.f64p), float(nrm_b[s]), of.ptr(xo, of.f64p), 100, 1,
                                                 C.byref(res))
            finally:
                of.lib().or_set_cycle_bits(0)
            assert it_o > 0 and abs(int(it[s]) - it_o) <= 2, (K, s, it[s], it_o)
    assert its[12].sum() < its[0].sum(), (its[0], its[12])
    B.close()


@pytest.mark.parametrize("nrhs", [1, 4])
def test_fused_one_colour_sweeps(ctx, nrhs):
    """With one colour below the finest level (caps [8, 1]) those levels'
    sweeps are fused into the SpMVs around them (sa_batch_fused_sweeps): the
    pre-smoothing sweep into the restriction that produces the level's e, the
    post-smoothing sweep into its U residual.  The V-cycle is still the
    oracle's bit for bit per system and right-hand side, the same with fusion
    on and off, and a solve gives the same iterations and x.  The systems end
    at different depths, so some levels also hold other systems' coarsest rows
    (there the post-smoothing sweep stays a launch of its own)."""
    systems, bs = _systems(SYSTEMS, nrhs)
    B = sagb.Batch(ctx, systems, nrhs)
    B.set_colour_caps([8, 1])
    nf = B.fused_sweeps()
    assert 0 < nf <= B.depth - 1, (nf, B.depth)
    rng = np.random.default_rng(40 + nrhs)
    vin = rng.integers(-(1 << 28), 1 << 28, size=B.rows * nrhs).astype(np.int32)
    out_on = B.precondition(vin)
    assert B.fused_sweeps(0) == 0
    np.testing.assert_array_equal(B.precondition(vin), out_on)
    assert B.fused_sweeps(1) == nf
    out2, vin2 = out_on.reshape(B.rows, nrhs), vin.reshape(B.rows, nrhs)
    keep = of.Keep()
    for s in range(B.nsys):
        h = sv.oracle_amg(keep, B.system_setup(s))
        a, e = B.offsets[s], B.offsets[s + 1]
        for r in range(nrhs):
            x = np.ascontiguousarray(vin2[a:e, r])
            ref = np.zeros_like(x)
            of.lib().or_vcycle_i32(C.byref(h), of.ptr(x, of.i32p), of.ptr(ref, of.i32p))
            np.testing.assert_array_equal(out2[a:e, r], ref, err_msg=f"system {s} rhs {r}")
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(x[:, r]) for x in bs for r in range(nrhs)])
    params = sagb.solver_params(m=20, explicit_stop=1, cycle_bits=12)
    res = []
    for on in (1, 0):
        B.fused_sweeps(on)
        x = np.zeros(B.rows * nrhs)
        it, cv, _ = B.solve(params, [29] * B.nsys, b, nrm_b, x)
        assert cv.all(), it
        res.append((it.copy(), x))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])
    B.close()


def test_ell_copy_same_results(ctx):
    """The ELL copy of short-row square operators (sa_batch_ell; the finest
    levels of the 7- and 5-point systems here): the V-cycle with every ELL
    copy in use is the oracle's bit for bit, and a solve (whose Arnoldi SpMV
    and dot then run on the level-0 ELL copy) gives the same iterations and x
    as with the CSR."""
    specs = [(sagb.GEN_POISSON3D, 17, 0.0), (sagb.GEN_POISSON2D, 40, 0.0), (sagb.GEN_CONVDIFF3D, 14, 20.0)]
    nrhs = 2
    systems, bs = _systems(specs, nrhs)
    B = sagb.Batch(ctx, systems, nrhs)
    rng = np.random.default_rng(77)
    vin = rng.integers(-(1 << 28), 1 << 28, size=B.rows * nrhs).astype(np.int32)
    ref = B.precondition(vin)
    n_ell = 0
    for lv in range(B.depth):
        for op in (0, 2):
            try:
                n_ell += B.ell(lv, op, 1)
            except sagb.SagbError:
                pass
    assert n_ell >= 1 and B.ell(0, 0) == 1
    got = B.precondition(vin)
    np.testing.assert_array_equal(got, ref)
    out2, vin2 = got.reshape(B.rows, nrhs), vin.reshape(B.rows, nrhs)
    keep = of.Keep()
    for s in range(B.nsys):
        h = sv.oracle_amg(keep, B.system_setup(s))
        a, e = B.offsets[s], B.offsets[s + 1]
        for r in range(nrhs):
            x = np.ascontiguousarray(vin2[a:e, r])
            o = np.zeros_like(x)
            of.lib().or_vcycle_i32(C.byref(h), of.ptr(x, of.i32p), of.ptr(o, of.i32p))
            np.testing.assert_array_equal(out2[a:e, r], o, err_msg=f"system {s} rhs {r}")
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(x[:, r]) for x in bs for r in range(nrhs)])
    params = sagb.solver_params(m=20, explicit_stop=1, cycle_bits=12)
    res = []
    for on in (1, 0):
        B.ell(0, 0, on)
        x = np.zeros(B.rows * nrhs)
        it, cv, _ = B.solve(params, [29] * B.nsys, b, nrm_b, x)
        assert cv.all(), it
        res.append((it.copy(), x))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])
    B.close()


def test_colour_caps_rebuild_and_tune(ctx):
    """sa_batch_set_colour_caps rebuilds every system's split with caps per
    level (the coarsening kept): the V-cycle is still the oracle's, in the new
    colour order, bit for bit; colour counts respect the caps; the
    time-to-solution tuner leaves the batch on its fastest candidate."""
    systems, bs = _systems(SYSTEMS, 1)
    B = sagb.Batch(ctx, systems, 1)
    depth = B.depth
    B.set_colour_caps([8, 4, 1])
    caps = B.colour_caps()
    assert B.depth == depth and caps[:3] == [8, 4, 1] and all(c == 1 for c in caps[2:])
    for lv in range(B.depth):
        assert B.level_info(lv, 1)[3] <= caps[lv], lv
    vin = np.random.default_rng(21).integers(-(1 << 28), 1 << 28, size=B.rows).astype(np.int32)
    out = B.precondition(vin)
    keep = of.Keep()
    for s in range(B.nsys):
        h = sv.oracle_amg(keep, B.system_setup(s))
        a, e = B.offsets[s], B.offsets[s + 1]
        x = np.ascontiguousarray(vin[a:e])
        ref = np.zeros_like(x)
        of.lib().or_vcycle_i32(C.byref(h), of.ptr(x, of.i32p), of.ptr(ref, of.i32p))
        np.testing.assert_array_equal(out[a:e], ref, err_msg=f"system {s}")
    b = _interleave(B, bs)
    nrm_b = np.array([np.linalg.norm(x[:, 0]) for x in bs])
    db = sagb.DeviceArray.from_host(ctx, b)
    dx = sagb.DeviceArray(ctx, B.rows, np.float64)
    params = sagb.solver_params(m=20, explicit_stop=1, cycle_bits=12)
    table = B.tune_colour_caps(params, [29] * B.nsys, db, nrm_b, dx, [[8, 2], [8, 1], [0, 2]], reps=1)
    assert len(table) == 3 and all(t[1] < float("inf") for t in table), table
    best = min(table, key=lambda t: t[1])[0]
    assert B.colour_caps()[:len(best)] == best
    it, cv, _ = B.solve(params, [29] * B.nsys, db, nrm_b, dx)
    assert cv.all()
    db.close(); dx.close()
    B.close()
