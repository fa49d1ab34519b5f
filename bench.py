#!/usr/bin/env python
"""Time to explicit relative residual 1e-10 on one GB300: batched int-AMG-FGMRES
with learned fractional bits against the plain drop-in integer solver.

Workload: 3D 7-point Poisson 128^3 (2,097,152 rows, 14,581,760 nonzeros, 6/-1,
Dirichlet), b = A x* with x* ~ U[-1, 1] (splitmix64 seed), LMax1 row scaling,
x0 = 0, m = 30, eps = 1e-10 on the explicit residual, one right-hand side.  A
step is one full solve (Restarted + FGMRESflex + V-cycles) by the batched
engine: multicolour SOR (8 colours on the finest level, 2 on the coarser
ones), a 400-row coarsest level, autotuned launch shapes, graph-captured
Arnoldi steps chained by programmatic dependent launch, and the F chosen by the
trained selector with the reference's rule (Work/main.cpp:153-161) as default
and fallback.  Beside it, on the same GPU: the plain drop-in (the reference's
bit-exact SOR order and bit rule), FP64-AMG-FGMRES, the single-system
multicolour solver and four right-hand sides at once.  The host AMG setup is
outside the timed region, as in the reference's own timer.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload poisson128|batch256|convdiff128|precision|vcycle]

Prints one JSON line (rank 0).  `value` is seconds per solve with b and x
resident in HBM (max over ranks); `e2e` is the same through the C ABI with
page-locked host b and x (copies inside the timed region).  `--impl reference`
times the reference's plain integer solver on the host cores (the C
restatement in oracle/, all threads) on the same system.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sc23-ad_gb300"))

def workload(n, m):
    return (f"3D 7-point Poisson {n}^3, one right-hand side: batched int-AMG-FGMRES({m}) with FP64 refinement, "
            "multicolour SOR smoother, learned fractional bits (rule as fallback), cycles restarted once their "
            "estimate has fallen 2^12; the plain drop-in (rule bits, bit-exact level-scheduled SOR, full cycles), "
            "FP64-AMG-FGMRES on the same batched design and the CPU reference reported beside it")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=128, help="grid side (128 for the benchmark)")
    ap.add_argument("--m", type=int, default=30)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-multicolor", action="store_true", help="skip the multicolour-smoother row")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-engine rows")
    ap.add_argument("--no-fp-batched", action="store_true", help="skip the FP64 / FP32 batched rows")
    ap.add_argument("--no-tune-caps", action="store_true", help="keep the default colour caps (8 / 2)")
    ap.add_argument("--no-learned-gain", action="store_true",
                    help="skip the learned-vs-rule rows (convection-diffusion 128^3, anisotropic 1024^2)")
    ap.add_argument("--cycle-bits", type=int, default=12,
                    help="batched integer engine: end a restart cycle once its estimate has fallen 2^K below its "
                         "start (the fixed-point basis stops gaining about 2^20 down); 0: full FGMRESflex cycles")
    ap.add_argument("--profile", action="store_true", help="skip extras (for profilers)")
    ap.add_argument("--tune-file", default=None,
                    help="vcycle workload: launch shapes to apply (written by a run without it, so that a run under "
                         "a profiler does not autotune under the profiler)")
    ap.add_argument("--caps", default="8,1", help="vcycle / solve workloads: colour caps per level")
    ap.add_argument("--no-graphs", action="store_true", help="solve workload: launches without CUDA graphs")
    ap.add_argument("--workload", choices=["poisson128", "batch256", "convdiff128", "precision", "vcycle", "solve",
                                           "plain_vcycle"],
                    default="poisson128",
                    help="poisson128: the headline; batch256: 256 27-point systems x 4 right-hand sides; "
                         "convdiff128: learned vs rule bits on convection-diffusion 128^3, Pe 50")
    ap.add_argument("--nsys", type=int, default=256)
    return ap.parse_args()


class Dist:
    """torchrun-style ranks; replicas only (no data-path collective)."""

    def __init__(self, ngpus):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, v):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def build_system(n, seed):
    import sagb
    A = sagb.HostCsr.generate(sagb.GEN_POISSON3D, n)
    xs, b = A.rhs(seed)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    return r, c, v, b


def explicit_res(r, c, v, b, x):
    rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
    Ax = np.bincount(rows, weights=v * x[c], minlength=len(r) - 1)
    return float(np.linalg.norm(b - Ax) / np.linalg.norm(b))


class Clocks:
    """nvidia-smi sampler during the timed region (read-only queries)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [s.strip() for s in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


# ------------------------------------------------------------------ our arm

def learned_bits(ctx, setup_int, ratio):
    """F from the trained selector (sc23-ad_gb300/data/bitsel_mlp.npz), or None."""
    import bitsel
    import sagb
    if not os.path.exists(bitsel.WEIGHTS):
        return None
    sel = bitsel.Selector(ctx)
    f = sel.choose(sagb.setup_features(setup_int, ratio), bitsel.rule_of(ratio))
    sel.net.close()
    return f


# colour caps per level tried by the headline's tuner (the last entry holds for
# deeper levels): 8 colours properly colour 7- and 27-point fine grids; below,
# fewer colours mean fewer dependent steps per sweep and a weaker smoother
CAP_CANDIDATES = [[8, 2], [8, 1], [8, 3], [8, 4], [8, 2, 1], [8, 4, 2], [8, 1, 2]]


def run_ours(a, dist):
    """Headline: the batched engine (multicolour colour-pass sweeps, autotuned
    lanes per row, graph-captured Arnoldi steps) with the learned F and the
    rule's F as fallback, on one 128^3 system and one right-hand side."""
    import bitsel
    import sagb
    dev = dist.local
    ctx = sagb.Context(dev)
    r, c, v, b = build_system(a.n, seed=1 + dist.rank)
    N = len(b)
    nrm_b = float(np.linalg.norm(b))
    t0 = time.time()
    B = sagb.Batch(ctx, [(r, c, v)], 1)
    t_setup = time.time() - t0
    t0 = time.time()
    B.autotune(2)
    t_tune = time.time() - t0
    ratio = float(B.rule_ratios(b, [nrm_b])[0])
    rule = bitsel.rule_of(ratio)
    params = sagb.solver_params(m=a.m, explicit_stop=1, cycle_bits=a.cycle_bits)
    db = sagb.DeviceArray.from_host(ctx, b)
    dx = sagb.DeviceArray(ctx, N, np.float64)
    zeros = sagb.DeviceArray.from_host(ctx, np.zeros(N))
    nb = np.array([nrm_b])
    caps_table = None
    if not a.no_tune_caps:
        # colour caps by measured time to solution (setup, outside the timed region)
        t0 = time.time()
        caps_table = B.tune_colour_caps(params, [rule], db, nb, dx, CAP_CANDIDATES)
        t_tune += time.time() - t0
    s0 = B.system_setup(0)
    learned = learned_bits(ctx, s0, ratio)
    bits = learned if learned is not None else rule
    state = {"fallbacks": 0}

    def one_solve():
        sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * N))
        it, cv, fb = B.solve(params, [bits], db, nb, dx)
        if not cv[0]:  # the learned F failed: the rule's F (part of the method, timed)
            state["fallbacks"] += 1
            sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * N))
            it2, cv, fb = B.solve(params, [rule], db, nb, dx)
            it = it + it2
        return int(it[0]), int(cv[0]), int(fb[0])

    for _ in range(a.warmup):
        one_solve()
    its = []
    clocks = Clocks(dev)
    e0, e1 = sagb.Event(), sagb.Event()
    dist.barrier()
    ctx.sync()
    l0 = ctx.launches()
    clocks.start()
    e0.record(ctx)
    for _ in range(a.steps):
        its.append(one_solve())
    e1.record(ctx)
    ctx.sync()
    clk = clocks.stop()
    launches = ctx.launches() - l0
    ms = e0.elapsed_ms(e1)
    dist.barrier()
    sec = dist.max(ms / 1000.0 / a.steps)
    x = dx.download()
    out = {"iters": its[-1][0], "converged": all(q[1] for q in its), "explicit_res": explicit_res(r, c, v, b, x),
           "frac_bits": bits, "rule_bits": rule, "learned_bits": learned, "final_bits": its[-1][2],
           "selector_fallbacks": state["fallbacks"], "setup_s": t_setup, "autotune_s": t_tune,
           "launches": launches, "clocks": clk, "colour_caps": B.colour_caps()}
    if caps_table is not None:
        out["colour_cap_tuning"] = [{"caps": t[0], "ms": round(t[1], 3), "iters": t[2][0]} for t in caps_table]
    if a.profile:
        return sec, out, ctx, None
    # ---- the same engine with full FGMRESflex cycles (no early restart)
    if a.cycle_bits:
        full = sagb.solver_params(m=a.m, explicit_stop=1)
        sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * N))
        B.solve(full, [bits], db, nb, dx)
        tf = []  # the median of three solves, each timed on its own
        for _ in range(3):
            sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * N))
            ctx.sync()
            e0.record(ctx)
            itf, cvf, _ = B.solve(full, [bits], db, nb, dx)
            e1.record(ctx)
            ctx.sync()
            tf.append(e0.elapsed_ms(e1) / 1000.0)
        out["full_cycles"] = {"value": float(np.median(tf)), "iters": int(itf[0]),
                              "converged": bool(cvf[0]), "explicit_res": explicit_res(r, c, v, b, dx.download())}
    # ---- end to end through the C ABI with page-locked host b and x
    if not a.no_e2e:
        hb = sagb.PinnedArray(N, np.float64)
        hx = sagb.PinnedArray(N, np.float64)
        hb.a[:] = b
        ts = []
        for k in range(max(2, a.steps // 2) + 1):
            hx.a[:] = 0
            t = time.perf_counter()
            it, cv, fb = B.solve(params, [bits], hb, nb, hx)
            ts.append(time.perf_counter() - t)
        out["e2e_s"] = dist.max(float(np.mean(ts[1:])))
        out["e2e_res"] = explicit_res(r, c, v, b, np.array(hx.a))
        hb.close()
        hx.close()
    out["kernels"] = batch_rooflines(ctx, B, a)
    for arr in (db, dx, zeros):
        arr.close()
    # ---- the FP64 and FP32-mixed siblings on the same batched design
    if not a.no_fp_batched:
        out["fp32_batched"] = fp_batched_row(ctx, a, B, r, c, v, b, nrm_b, sagb.F32)
        out["fp64_batched"] = fp_batched_row(ctx, a, B, r, c, v, b, nrm_b, sagb.F64,
                                             None if a.no_tune_caps else FP_CAP_CANDIDATES)
    B.close()
    # ---- comparison rows on the same GPU
    out["plain"] = plain_row(ctx, a, r, c, v, b, nrm_b)
    if not a.no_multicolor:
        out["multicolor"] = multicolor_row(ctx, a, r, c, v, b, nrm_b)
    if not a.no_batched:
        out["batched"] = batched_rows(ctx, a, r, c, v, b, nrm_b, dist, bits, rule, out.get("colour_caps"))
    out["setup"] = setup_row(ctx, r, c, v)
    if not a.no_learned_gain:
        out["learned_gain"] = learned_gain_rows(ctx, a)
    return sec, out, ctx, out["plain"].pop("state")


FP_CAP_CANDIDATES = [[8, 2], [8, 1], [8, 4], [8, 2, 1]]


def fp_batched_row(ctx, a, B, r, c, v, b, nrm_b, prec, cap_candidates=None):
    """FP64-AMG-FGMRES (or FP32-mixed) on the headline's batched design: the
    same coarsening, coarsest-level size, graph-captured Arnoldi steps and
    autotuned launch shapes as the integer engine, the colour caps either the
    integer batch's or tuned for this solver by its own time to solution
    (cap_candidates); b, x in HBM, explicit-residual stop, CUDA events on the
    library's stream."""
    import sagb
    N = len(b)
    params = sagb.solver_params(m=a.m, explicit_stop=1)
    db = sagb.DeviceArray.from_host(ctx, b)
    dx = sagb.DeviceArray(ctx, N, np.float64)
    zeros = sagb.DeviceArray.from_host(ctx, np.zeros(N))
    nb = np.array([nrm_b])
    e0, e1 = sagb.Event(), sagb.Event()

    def timed(F, reps):
        def one():
            sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * N))
            return F.solve(params, db, nb, dx)
        one()
        ctx.sync()
        e0.record(ctx)
        for _ in range(reps):
            it, cv = one()
        e1.record(ctx)
        ctx.sync()
        return e0.elapsed_ms(e1) / 1000.0 / reps, it, cv

    table = None
    if cap_candidates:
        table = []
        keep_caps = B.colour_caps()
        for caps in cap_candidates:
            B.set_colour_caps(caps)
            F = sagb.BatchFp(ctx, B, prec)
            F.autotune(2)
            sec, it, cv = timed(F, 2)
            table.append((caps, sec if cv[0] else float("inf"), int(it[0])))
            F.close()
        B.set_colour_caps(min(table, key=lambda t: t[1])[0])
    t0 = time.time()
    F = sagb.BatchFp(ctx, B, prec)
    t_setup = time.time() - t0
    t0 = time.time()
    F.autotune(2)
    t_tune = time.time() - t0
    sec, it, cv = timed(F, 3)
    row = {"value": sec, "iters": int(it[0]), "converged": bool(cv[0]),
           "explicit_res": explicit_res(r, c, v, b, dx.download()), "vcycle_ms": F.time_vcycle(10),
           "setup_s": t_setup, "autotune_s": t_tune, "colour_caps": B.colour_caps()}
    if table is not None:
        row["colour_cap_tuning"] = [{"caps": t[0], "ms": round(t[1] * 1e3, 3), "iters": t[2]} for t in table]
        B.set_colour_caps(keep_caps)
        B.autotune(2)
    for arr in (db, dx, zeros):
        arr.close()
    F.close()
    return row


def learned_gain_rows(ctx, a):
    """The learned F against the method without the network (the rule's F
    with the overflow fallback) on the selector's evaluation system
    (upwinded convection-diffusion 128^3, Peclet 50) and on the anisotropic
    1024^2 system of the precision workload (eps 1e-3), both through the
    batched engine with its defaults: time per solve (best of three, CUDA
    events, discarded cycles included) and iterations."""
    import bitsel
    import sagb
    out = {}
    sel = bitsel.Selector(ctx)
    for name, spec in (("convdiff128_pe50", (sagb.GEN_CONVDIFF3D, 128, 50.0, 1, 0)),
                       ("aniso1024_eps1e-3", (sagb.GEN_ANISO2D, 1024, 1e-3, 1, 0))):
        r, c, v, b = bitsel.make_system(spec)
        B = sagb.Batch(ctx, [(r, c, v)], 1)
        B.autotune(1)
        nrm = float(np.linalg.norm(b))
        q = float(B.rule_ratios(b, [nrm])[0])
        rule = bitsel.rule_of(q)
        f = sel.choose(sagb.setup_features(B.system_setup(0), q), rule)
        db = sagb.DeviceArray.from_host(ctx, b)
        dx = sagb.DeviceArray(ctx, len(b), np.float64)
        nb = np.array([nrm])
        p = sagb.solver_params(m=a.m, explicit_stop=1, overflow_fallback=1, cycle_bits=a.cycle_bits)
        row = {"rows": len(b), "rule_bits": rule, "learned_bits": f}
        for key, F in (("rule", rule), ("learned", f)):
            dx.upload(np.zeros(len(b)))
            B.solve(p, [F], db, nb, dx)
            best = None
            for _ in range(3):
                dx.upload(np.zeros(len(b)))
                e0, e1 = sagb.Event(), sagb.Event()
                ctx.sync()
                e0.record(ctx)
                it, cv, fb = B.solve(p, [F], db, nb, dx)
                e1.record(ctx)
                ctx.sync()
                ms = e0.elapsed_ms(e1)
                best = ms if best is None else min(best, ms)
            row[key] = {"ms": round(best, 3), "iters": int(it[0]), "converged": bool(cv[0]),
                        "final_bits": int(fb[0]), "explicit_res": explicit_res(r, c, v, b, dx.download())}
        row["speedup"] = row["rule"]["ms"] / row["learned"]["ms"]
        out[name] = row
        db.close()
        dx.close()
        B.close()
    sel.net.close()
    return out


def setup_row(ctx, r, c, v):
    """The AMG setup of the same system (the headline's parameters: multicolour
    smoother, 8 colours on the finest level and 2 below, 400-row coarsest
    level) on the host and with the
    Ruge-Stueben levels on the GPU; the two hierarchies are compared array by
    array (they must be identical)."""
    import sagb
    params = sagb.amg_params(multicolor=1, max_colours=sagb.Batch.DEFAULT_MAX_COLOURS,
                             coarse_colours=sagb.Batch.DEFAULT_COARSE_COLOURS,
                             coarse_size=sagb.Batch.DEFAULT_COARSE_SIZE)
    t = time.perf_counter()
    g = sagb.Setup(sagb.INT, r, c, v, params, ctx=ctx)
    t_gpu = time.perf_counter() - t
    t = time.perf_counter()
    h = sagb.Setup(sagb.INT, r, c, v, params)
    t_host = time.perf_counter() - t
    same = g.depth == h.depth
    for i in range(h.depth):
        for op in (sagb.OP_P, sagb.OP_R, sagb.OP_LD, sagb.OP_U) + ((sagb.OP_CA,) if i < h.depth - 1 else ()):
            x, y = g.view(op, i), h.view(op, i)
            same = same and all(np.array_equal(p, q) for p, q in zip(x[:3], y[:3])) and x[3:] == y[3:]
    return {"gpu_s": t_gpu, "host_s": t_host, "host_threads": os.cpu_count(), "levels": h.depth,
            "identical": bool(same)}


def plain_row(ctx, a, r, c, v, b, nrm_b):
    """The plain drop-in: bit-exact level-scheduled SOR sweeps, the rule's F
    (the reference's algorithm on the GPU), and the FP64 solver beside it."""
    import sagb
    N = len(b)
    t0 = time.time()
    s_int = sagb.Setup(sagb.INT, r, c, v)
    s_f64 = s_int.derive(sagb.F64)
    t_setup = time.time() - t0
    M = sagb.Amg(ctx, sagb.INT, setup=s_int)
    M64 = sagb.Amg(ctx, sagb.F64, setup=s_f64)
    dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
    A0 = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
    bits = sagb.rule_bits(ctx, M64, b, nrm_b)
    S = sagb.Solver(ctx, sagb.INT, dA, A0, M, sagb.solver_params(m=a.m, frac_bits=bits, explicit_stop=1))
    db = sagb.DeviceArray.from_host(ctx, b)
    dx = sagb.DeviceArray(ctx, N, np.float64)
    e0, e1 = sagb.Event(), sagb.Event()

    def timed(solver, reps):
        dx.upload(np.zeros(N))
        solver.solve(db, nrm_b, dx)
        it = None
        e0.record(ctx)
        for _ in range(reps):
            dx.upload(np.zeros(N))
            it = solver.solve(db, nrm_b, dx)
        e1.record(ctx)
        ctx.sync()
        return e0.elapsed_ms(e1) / 1000.0 / reps, it
    sec, it = timed(S, 2)
    row = {"value": sec, "iters": it[0], "converged": bool(it[1]), "explicit_res": explicit_res(r, c, v, b, dx.download()),
           "frac_bits": bits, "setup_s": t_setup}
    k = kernel_rooflines(ctx, M, A0, N, a)
    row["vcycle_ms"] = k["vcycle"]["ms"]
    row["sweep_ms_per_vcycle"] = k["sweeps"]["ms_per_vcycle"]
    row["coarse_lu_ms"] = k["coarse_lu"]["ms"]
    row["sweep_levels"] = [(p["level"], p["n"], p["levels"], round(p["ms"], 4)) for p in k["sweeps"]["per_level"]]
    l0 = k["sweeps"]["per_level"][0]
    row["sweep_level0"] = {"ms": l0["ms"], "bytes": l0["bytes"], "traffic": ncu_traffic("k_tri_level0")}
    row["spmv_A0"] = k["spmv_A0"]
    S.close()
    S64 = sagb.Solver(ctx, sagb.F64, dA, dA, M64, sagb.solver_params(m=a.m, explicit_stop=1))
    sec64, it64 = timed(S64, 2)
    row["fp64_gpu"] = {"value": sec64, "iters": it64[0], "explicit_res": explicit_res(r, c, v, b, dx.download())}
    S64.close()
    row["state"] = (s_int, r, c, v, b, bits)
    for o in (db, dx):
        o.close()
    return row


def batch_rooflines(ctx, B, a):
    """Average time per call and algorithmic bytes of every batched level
    operator, and the V-cycle they make up.  Each call is timed cold: CUDA
    events on the library stream around a CUDA graph of calls, each preceded
    by a read of a buffer three times the L2, less the time of the reads
    alone, so that every operator comes from HBM as in the solver's V-cycle
    (1.3 GB streamed between two uses of one operator); `ms_warm` is the same
    call repeated on L2-resident data."""
    import sagb
    R = B.nrhs
    rng = np.random.default_rng(3)
    big = B.rows * R
    xin = sagb.DeviceArray.from_host(ctx, rng.integers(-(1 << 28), 1 << 28, size=big).astype(np.int32))
    xout = sagb.DeviceArray(ctx, big, np.int32)
    reps = 10
    fam = {"spmv": [0.0, 0], "sweep": [0.0, 0]}
    per = []
    for l in range(B.depth):
        for op, name in ((0, "A"), (1, "LD"), (2, "U"), (3, "P"), (4, "R")):
            n, m, nnz, ncol = B.level_info(l, op)
            if n == 0:
                continue
            t = B.time_op(l, op, xin, xout, reps, cold=True)
            t_warm = B.time_op(l, op, xin, xout, reps)
            if op == 1:
                # LD entries, row pointers, two shifts, the colour row list, in once, out written once
                by = 8 * nnz + 4 * (n + 1) + 2 * n + 4 * n + 8 * R * n
                calls = 2  # pre- and post-smoothing
            else:
                # entries (32-bit values and 32-bit columns, or 16-bit column offsets when the
                # autotuner chose the compressed storage), row pointers, the shift, x once, y once
                colb = 2 if op in (0, 2) and B.compressed(l, op) else 4
                by = (4 + colb) * nnz + 4 * (n + 1) + n + 4 * R * m + 4 * R * n
                calls = 1  # A (residual), U (post-smoothing residual), P and R once per V-cycle
            per.append({"level": l, "op": name, "n": n, "nnz": nnz, "colours": ncol if op == 1 else None,
                        "ms": t, "ms_warm": t_warm, "bytes": by, "per_vcycle": calls,
                        "d16": bool(op in (0, 2) and B.compressed(l, op))})
            key = "sweep" if op == 1 else "spmv"
            fam[key][0] += calls * t
            fam[key][1] += calls * by
    t_lu = B.time_op(0, B.OP_LU, reps=reps)
    vin = sagb.DeviceArray.from_host(ctx, rng.integers(-(1 << 28), 1 << 28, size=big).astype(np.int32))
    t_v = B.time_op(0, B.OP_VCYCLE, vin, xout, reps)
    for o in (xin, xout, vin):
        o.close()
    return {"per_op": per, "families": fam, "coarse_lu_ms": t_lu, "vcycle_ms": t_v}


def batched_rows(ctx, a, r, c, v, b, nrm_b, dist, bits, rule, caps=None):
    """Four right-hand sides of the same 128^3 system solved together (the
    matrix entries are read once for all four)."""
    import sagb
    N = len(b)
    nrhs = 4
    t0 = time.time()
    B = sagb.Batch(ctx, [(r, c, v)], nrhs)
    if caps:
        B.set_colour_caps(caps)
    t_setup = time.time() - t0
    B.autotune(2)
    cols = [b] + [build_system(a.n, seed=1 + dist.rank + 1000 * k)[3] for k in range(1, nrhs)]
    bb = np.stack(cols, 1).ravel()
    nb = np.array([np.linalg.norm(col) for col in cols])
    params = sagb.solver_params(m=a.m, explicit_stop=1, cycle_bits=a.cycle_bits)
    db = sagb.DeviceArray.from_host(ctx, bb)
    dx = sagb.DeviceArray(ctx, N * nrhs, np.float64)
    zeros = sagb.DeviceArray.from_host(ctx, np.zeros(N * nrhs))

    def one():
        sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * N * nrhs))
        return B.solve(params, [bits], db, nb, dx)

    one()
    e0, e1 = sagb.Event(), sagb.Event()
    reps = 3
    ctx.sync()
    e0.record(ctx)
    for _ in range(reps):
        it, cv, fb = one()
    e1.record(ctx)
    ctx.sync()
    sec = e0.elapsed_ms(e1) / 1000.0 / reps
    X = dx.download().reshape(N, nrhs)
    res = [explicit_res(r, c, v, cols[k], np.ascontiguousarray(X[:, k])) for k in range(nrhs)]
    k = batch_rooflines(ctx, B, a)
    row = {"nrhs": nrhs, "value": sec, "per_rhs": sec / nrhs, "iters": [int(i) for i in it],
           "converged": bool(cv.all()), "explicit_res": max(res), "frac_bits": bits,
           "final_bits": [int(f) for f in fb], "vcycle_ms": k["vcycle_ms"], "setup_s": t_setup,
           "spmv_A0": next(p for p in k["per_op"] if p["level"] == 0 and p["op"] == "A")}
    for arr in (db, dx, zeros):
        arr.close()
    B.close()
    return row


def multicolor_row(ctx, a, r, c, v, b, nrm_b):
    """The single-system solver with the multicolour split (level-scheduled
    sweep kernels with the colours as levels), rule's F."""
    import sagb
    N = len(b)
    t0 = time.time()
    s_mc = sagb.Setup(sagb.INT, r, c, v, sagb.amg_params(multicolor=1))
    s_mc64 = s_mc.derive(sagb.F64)
    t_setup = time.time() - t0
    Mm = sagb.Amg(ctx, sagb.INT, setup=s_mc)
    Mm64 = sagb.Amg(ctx, sagb.F64, setup=s_mc64)
    dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
    A0 = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
    bits = sagb.rule_bits(ctx, Mm64, b, nrm_b)
    Sm = sagb.Solver(ctx, sagb.INT, dA, A0, Mm, sagb.solver_params(m=a.m, frac_bits=bits, explicit_stop=1))
    db = sagb.DeviceArray.from_host(ctx, b)
    dx = sagb.DeviceArray(ctx, N, np.float64)
    e0, e1 = sagb.Event(), sagb.Event()
    dx.upload(np.zeros(N))
    Sm.solve(db, nrm_b, dx)
    nrep = 2
    itm = None
    e0.record(ctx)
    for _ in range(nrep):
        dx.upload(np.zeros(N))
        itm = Sm.solve(db, nrm_b, dx)
    e1.record(ctx)
    ctx.sync()
    row = {"value": e0.elapsed_ms(e1) / 1000.0 / nrep, "iters": itm[0], "converged": bool(itm[1]),
           "explicit_res": explicit_res(r, c, v, b, dx.download()), "frac_bits": bits, "setup_s": t_setup,
           "colours": [int(s_mc.view(sagb.OP_COLOR, l).max()) + 1 for l in range(s_mc.depth)]}
    k = kernel_rooflines(ctx, Mm, A0, N, a)
    row["vcycle_ms"] = k["vcycle"]["ms"]
    row["sweep_ms_per_vcycle"] = k["sweeps"]["ms_per_vcycle"]
    row["sweep_levels"] = [(p["level"], p["n"], p["levels"], round(p["ms"], 4)) for p in k["sweeps"]["per_level"]]
    for o in (Sm, Mm, Mm64, dA, A0, db, dx):
        o.close()
    return row


def kernel_rooflines(ctx, M, A0, N, a):
    """Average launch time (CUDA events on the library stream) and algorithmic
    bytes of the hot kernels, one V-cycle's worth at a time."""
    import sagb
    rng = np.random.default_rng(3)
    vin = sagb.DeviceArray.from_host(ctx, rng.integers(-(1 << 28), 1 << 28, size=N).astype(np.int32))
    vout = sagb.DeviceArray(ctx, N, np.int32)
    e0, e1 = sagb.Event(), sagb.Event()
    reps = 10

    def timed(fn):
        fn()
        ctx.sync()
        e0.record(ctx)
        for _ in range(reps):
            fn()
        e1.record(ctx)
        return e0.elapsed_ms(e1) / reps

    res = {}
    # fine-level SpMV (CSR<Fixed<30>>): 8 nnz + 4(N+1) + 4 N (x) + 4 N (y)
    nnz = A0.nnz
    t = timed(lambda: sagb.check(sagb.lib().sa_spmv(ctx.h, A0.h, vin.ptr, vout.ptr)))
    res["spmv_A0"] = {"ms": t, "bytes": 8 * nnz + 4 * (N + 1) + 8 * N}
    # V-cycle
    t = timed(lambda: sagb.check(sagb.lib().sa_amg_precondition(ctx.h, M.h, vin.ptr, vout.ptr)))
    res["vcycle"] = {"ms": t}
    # Gauss-Seidel sweeps of every level (two per level per V-cycle)
    sweep_ms, sweep_bytes = 0.0, 0
    per = []
    for l in range(M.depth):
        n, _, nnz_ld, _, nlev = M.level_info(sagb.OP_LD, l)
        bufi = sagb.DeviceArray(ctx, n, np.int32)
        bufo = sagb.DeviceArray(ctx, n, np.int32)
        t = timed(lambda: sagb.check(sagb.lib().sa_amg_sweep(ctx.h, M.h, l, bufi.ptr, bufo.ptr)))
        # LD values+indices (off-diagonal and D^-1), row pointers, in, out
        by = 8 * nnz_ld + 4 * (n + 1) + 8 * n
        per.append({"level": l, "n": n, "nnz": nnz_ld, "levels": nlev, "ms": t, "bytes": by})
        sweep_ms += 2 * t
        sweep_bytes += 2 * by
        bufi.close()
        bufo.close()
    res["sweeps"] = {"ms_per_vcycle": sweep_ms, "bytes_per_vcycle": sweep_bytes, "per_level": per}
    # coarse LU (dense L and U read once)
    nlu = M.level_info(sagb.OP_LUL)[0]
    bi = sagb.DeviceArray(ctx, nlu, np.int32)
    bo = sagb.DeviceArray(ctx, nlu, np.int32)
    t = timed(lambda: sagb.check(sagb.lib().sa_amg_coarse_solve(ctx.h, M.h, bi.ptr, bo.ptr)))
    res["coarse_lu"] = {"ms": t, "bytes": 2 * 4 * nlu * nlu + 4 * nlu + 8 * nlu}
    return res


def cpu_baseline(state, threads, m):
    """The oracle (C restatement of the reference) on the host cores: one full
    solve of the same system with the same hierarchy, to explicit residual
    1e-10 as the GPU arm."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_ffi as of
    s_int, r, c, v, b, bits = state
    keep = of.Keep()
    h = oracle_hierarchy(of, keep, s_int)
    dA = of.csr_f(keep, r, c, v, np.float64)
    L = of.lib()
    L.or_set_threads(threads)
    x = np.zeros(len(b))
    res = C.c_double()
    t = time.perf_counter()
    it = L.or_ir_solve_i32x(C.byref(dA), C.byref(h.A0), C.byref(h), m, 1e-10, bits, of.ptr(b, of.f64p),
                            float(np.linalg.norm(b)), of.ptr(x, of.f64p), 1000 // m, 1, C.byref(res))
    return time.perf_counter() - t, it, explicit_res(r, c, v, b, x)


def oracle_hierarchy(of, keep, setup):
    import sagb
    g = {"depth": np.array([setup.depth])}

    def put(pfx, op, level=0):
        rr, cc, vv, bit, dbit, mm = setup.view(op, level)
        g[pfx + "_rptr"], g[pfx + "_cind"], g[pfx + "_val"] = rr, cc, vv
        g[pfx + "_meta"] = np.array([len(rr) - 1, mm, bit, dbit])
    put("A0", sagb.OP_A0)
    for i in range(setup.depth):
        if i < setup.depth - 1:
            put(f"L{i}_CA", sagb.OP_CA, i)
        put(f"L{i}_P", sagb.OP_P, i)
        put(f"L{i}_R", sagb.OP_R, i)
        put(f"S{i}_LD", sagb.OP_LD, i)
        put(f"S{i}_U", sagb.OP_U, i)
    put("LU_L", sagb.OP_LUL)
    put("LU_U", sagb.OP_LUU)
    g["A0_meta"][2] = 30
    return of.golden_amg_i32(keep, g)


METRIC = "time to 1e-10 rel. residual: batched+learned-bits vs plain int-AMG-FGMRES on GB300"


def bench_config(a, world):
    """The workload of both arms (the same dict in each line)."""
    return {"workload": workload(a.n, a.m), "rows": a.n ** 3, "m": a.m, "eps": 1e-10,
            "stop": "explicit relative residual", "parallelism": f"replicas{world}",
            "l2": "inputs larger than L2 (hierarchy ~1.5 GB, Krylov basis 0.5 GB per solve)"}


def main_ours(a):
    dist = Dist(a.gpus)
    sec, out, ctx, state = run_ours(a, dist)
    if dist.rank != 0:
        dist.close()
        return
    N = a.n ** 3
    peak, peak_kind = measured_peak()
    line = {
        "metric": METRIC,
        "value": sec, "unit": "s", "n_gpus": dist.world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": sec * 1000.0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (b = A x*, x* ~ U[-1,1] seeded; SuiteSparse inputs not shipped)",
        "config": bench_config(a, dist.world),
        "iters": out["iters"], "converged": out["converged"], "explicit_res": out["explicit_res"],
        "frac_bits": out["frac_bits"], "rule_bits": out["rule_bits"], "learned_bits": out["learned_bits"],
        "final_bits": out["final_bits"], "selector_fallbacks": out["selector_fallbacks"],
        "setup_s": out["setup_s"], "autotune_s": out["autotune_s"],
        "gpu_launches": out["launches"], "clocks": out["clocks"],
    }
    if "e2e_s" in out:
        line["e2e"] = {"value": out["e2e_s"], "unit": "s", "h2d_bytes_per_step": 8 * N + 8,
                       "d2h_bytes_per_step": 8 * N, "explicit_res": out["e2e_res"]}
    if "kernels" in out:
        k = out["kernels"]
        fam = k["families"]
        # dominant kernel family of the V-cycle: the colour-pass sweeps or the SpMVs
        name = max(fam, key=lambda f: fam[f][0])
        ms, by = fam[name]
        ach = by / (ms * 1e-3) / 1e9
        kern = "k_bcolour_packed / k_bcolour / k_bsweep_packed / k_bsweep_cluster (the autotuned multicolour " \
            "Gauss-Seidel sweeps, all levels)" if name == "sweep" else \
            "k_bspmv / k_bspmv_stream (level SpMVs, all levels)"
        line["roofline"] = {"kernel": kern, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                            "frac": ach / peak, "peak_kind": peak_kind, "traffic": ncu_traffic(name + "_per_vcycle"),
                            "bytes_per_vcycle": by, "ms_per_vcycle": ms, "share_of_vcycle": ms / k["vcycle_ms"]}
        sp = next(p for p in k["per_op"] if p["level"] == 0 and p["op"] == "A")
        spa = sp["bytes"] / (sp["ms"] * 1e-3) / 1e9
        line["spmv_A0"] = {"kernel": "k_bspmv level 0 (the autotuned form)", "achieved": spa, "peak": peak, "unit": "GB/s",
                           "frac": spa / peak, "ms": sp["ms"], "bytes": sp["bytes"],
                           "columns": "16-bit offsets" if sp["d16"] else "32-bit",
                           "traffic": ncu_traffic("spmv_A0_d16" if sp["d16"] else "spmv_A0")}
        line["vcycle_ms"] = k["vcycle_ms"]
        line["coarse_lu_ms"] = k["coarse_lu_ms"]
        line["families_ms_per_vcycle"] = {f: fam[f][0] for f in fam}
        # per level and operator: rows, colours (sweeps), ms per launch set, algorithmic GB/s
        line["ops"] = [(p["level"], p["op"], p["n"], p["colours"], round(p["ms"], 4),
                        round(p["bytes"] / (p["ms"] * 1e-3) / 1e9, 1)) for p in k["per_op"]]
    line["cycle_bits"] = a.cycle_bits
    line["colour_caps"] = out.get("colour_caps")
    if "colour_cap_tuning" in out:
        line["colour_cap_tuning"] = out["colour_cap_tuning"]
    for key in ("plain", "multicolor", "batched", "setup", "full_cycles", "learned_gain"):
        if key in out:
            line[key] = out[key]
    for key in ("fp64_batched", "fp32_batched"):
        if key in out:
            line[key] = out[key]
    if "plain" in out:
        line["speedup_vs_plain"] = out["plain"]["value"] / sec
        line["speedup_vs_fp64_plain_gpu"] = out["plain"]["fp64_gpu"]["value"] / sec
    if "fp64_batched" in out:
        # FP64-AMG-FGMRES on the same batched GPU design: the honest FP64 comparison
        line["speedup_vs_fp64_gpu"] = out["fp64_batched"]["value"] / sec
    if state is not None and not a.no_cpu_baseline and dist.world == 1:
        threads = os.cpu_count() or 1
        t, it, res = cpu_baseline(state, threads, a.m)
        line["cpu_baseline"] = {"value": t, "unit": "s", "cores": threads, "kind": "port",
                                "sample": "one full plain int solve of the same 128^3 system (same hierarchy and "
                                          f"rule bit), oracle C restatement, {threads} threads; iters={it} "
                                          f"res={res:.2e}"}
    print(json.dumps(tail_last(line)), flush=True)
    dist.close()


# the comparisons a reader of the line looks for first, in this order at its
# end (a log that keeps only the end of a long line still shows them)
TAIL_KEYS = ("vcycle_ms", "families_ms_per_vcycle", "spmv_A0", "full_cycles", "batched", "fp32_batched",
             "fp64_batched", "learned_gain", "speedup_vs_plain", "speedup_vs_fp64_plain_gpu", "speedup_vs_fp64_gpu",
             "roofline", "cpu_baseline", "e2e")


def tail_last(line):
    """A copy of the line with the bulky per-level diagnostics first and
    TAIL_KEYS last (the siblings' colour-cap tables moved to keys of their own)."""
    line = dict(line)
    out = {k: v for k, v in line.items() if k not in TAIL_KEYS}
    for k in ("fp64_batched", "fp32_batched"):
        if k in line and "colour_cap_tuning" in line[k]:
            line[k] = dict(line[k])
            out[k + "_colour_cap_tuning"] = line[k].pop("colour_cap_tuning")
    out.update((k, line[k]) for k in TAIL_KEYS if k in line)
    return out


# ------------------------------------------------------------- reference arm

def main_reference(a):
    """The reference's solve phase on the host cores, without this repository's
    library: the system from the numpy generators (tests/golden/gen_matrices.py,
    the same arrays as the library's generators), LMax1 scaling, the hierarchy
    from the oracle's own C restatement of the reference's AMG setup
    (oracle/oracle_setup.c, pinned to the reference's hierarchies), the rule's
    F from the oracle's FP64 V-cycle, and Restarted(FGMRESflex) from the
    oracle's C restatement (pinned to the reference bit for bit), run until the
    explicit residual reaches 1e-10 as the GPU arm is."""
    dist = Dist(a.gpus)
    if dist.rank != 0:
        dist.close()
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import gen_matrices as gm
    import oracle_ffi as of
    r, c, v = gm.poisson3d(a.n)
    _, b = gm.rhs(r, c, v, 1)
    rmax = np.maximum.reduceat(np.abs(v), r[:-1])  # CSRMat::LMax1Scaling (csrmat.hpp:70-80)
    v = v / np.repeat(rmax, np.diff(r))
    b = b / rmax
    t0 = time.time()
    S = of.OracleSetup(r, c, v)
    t_setup = time.time() - t0
    L = of.lib()
    threads = os.cpu_count() or 1
    L.or_set_threads(threads)
    nrm_b = float(np.linalg.norm(b))
    cvec = np.zeros(len(b))
    L.or_vcycle_f64(C.byref(S.h_f64), of.ptr(b, of.f64p), of.ptr(cvec, of.f64p))  # Work/main.cpp:153-161
    q = np.abs(cvec).max() / nrm_b
    bits = 29 if q < 1 else 31 - (int(np.ceil(np.log2(int(q) + 1))) + 1)
    keep = of.Keep()
    dA = of.csr_f(keep, r, c, v, np.float64)
    ts, it, x = [], 0, np.zeros(len(b))
    res = C.c_double()
    for k in range(a.warmup + a.steps):
        x[:] = 0
        t = time.perf_counter()
        it = L.or_ir_solve_i32x(C.byref(dA), C.byref(S.h_i32.A0), C.byref(S.h_i32), a.m, 1e-10, bits,
                                of.ptr(b, of.f64p), nrm_b, of.ptr(x, of.f64p), 1000 // a.m, 1, C.byref(res))
        if k >= a.warmup:
            ts.append(time.perf_counter() - t)
    val = float(np.mean(ts))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": val, "unit": "s", "n_gpus": dist.world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": val * 1000, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic (b = A x*, x* ~ U[-1,1] seeded; SuiteSparse inputs not shipped)",
        "config": bench_config(a, dist.world),
        "iters": it, "explicit_res": explicit_res(r, c, v, b, x), "frac_bits": bits, "setup_s": t_setup,
        "cpu_baseline": {"value": val, "unit": "s", "cores": threads, "kind": "port",
                         "sample": f"full solves of the {a.n}^3 system to explicit residual 1e-10, the oracle's C "
                                   f"restatement of the reference's setup and solve phase, {threads} threads (SpMV "
                                   f"and integer BLAS parallel, SOR sweeps sequential as in the reference)"},
        "e2e": {"value": val, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    S.close()
    print(json.dumps(line), flush=True)
    dist.close()


def fp64_oracle_hierarchy(of, keep, s, r, c, v):
    import sagb
    D = s.depth
    st = of.CsrF64

    def mk(op, level=0):
        rr, cc, vv, _, _, mm = s.view(op, level)
        return of.csr_f(keep, rr, cc, vv, np.float64, m=mm)
    CA = (st * max(D - 1, 1))(*[mk(sagb.OP_CA, i) for i in range(D - 1)])
    P = (st * D)(*[mk(sagb.OP_P, i) for i in range(D)])
    R = (st * D)(*[mk(sagb.OP_R, i) for i in range(D)])
    LD = (st * D)(*[mk(sagb.OP_LD, i) for i in range(D)])
    U = (st * D)(*[mk(sagb.OP_U, i) for i in range(D)])
    keep.refs += [CA, P, R, LD, U]
    h = of.AmgF64()
    h.depth = D
    h.A0 = of.csr_f(keep, r, c, v, np.float64)
    h.CA, h.P, h.R, h.LD, h.U = CA, P, R, LD, U
    h.smooth_iter = 1
    h.LUL = mk(sagb.OP_LUL)
    h.LUU = mk(sagb.OP_LUU)
    return h


# ----------------------------------------------------------- other workloads

def batch_systems(nsys, nrhs, seed=2024):
    """256 SPD 27-point systems (diagonal 26 + U[0.1, 1], off-diagonals -1),
    cube sides uniform in 16..64, nrhs right-hand sides U[-1, 1] each; rows and
    right-hand sides scaled by the row maxima (LMax1Scaling)."""
    import sagb
    rng = np.random.default_rng(seed)
    sides = rng.integers(16, 65, size=nsys)
    systems, bs = [], []
    for s, n in enumerate(sides):
        A = sagb.HostCsr.generate(sagb.GEN_STENCIL27, int(n), 0.0, seed=int(seed + s))
        r, c, v = A.arrays()
        rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
        rmax = np.zeros(len(r) - 1)
        np.maximum.at(rmax, rows, np.abs(v))
        B = rng.uniform(-1.0, 1.0, size=(len(r) - 1, nrhs))
        b0 = B[:, 0].copy()
        A.lmax1_scaling(b0)
        systems.append(A.arrays())
        bs.append(B / rmax[:, None])
    return systems, bs, sides


def main_batch(a):
    import bitsel
    import sagb
    dist = Dist(a.gpus)
    ctx = sagb.Context(dist.local)
    nrhs = 4
    t0 = time.time()
    systems, bs, sides = batch_systems(a.nsys, nrhs, seed=2024 + dist.rank)
    t_gen = time.time() - t0
    t0 = time.time()
    B = sagb.Batch(ctx, systems, nrhs)
    t_setup = time.time() - t0
    t0 = time.time()
    B.autotune(2)
    t_tune = time.time() - t0
    bvec = np.zeros((B.rows, nrhs))
    for s in range(B.nsys):
        bvec[B.offsets[s]:B.offsets[s + 1]] = bs[s]
    bvec = bvec.ravel()
    nrm_b = np.array([np.linalg.norm(bs[s][:, r]) for s in range(B.nsys) for r in range(nrhs)])
    t0 = time.time()
    ratios = B.rule_ratios(bvec, nrm_b)
    t_rule = time.time() - t0
    rule = [min(bitsel.rule_of(q) for q in ratios[s * nrhs:(s + 1) * nrhs]) for s in range(B.nsys)]
    params = sagb.solver_params(m=20, explicit_stop=1, cycle_bits=a.cycle_bits)
    db = sagb.DeviceArray.from_host(ctx, bvec)
    dx = sagb.DeviceArray(ctx, B.rows * nrhs, np.float64)
    caps_table = None
    if not a.no_tune_caps:
        # the coarse colour cap by measured time to solution with the rule's
        # bits (outside the timed region); the ratios, the rule and the
        # selector's features then describe the kept smoother
        t0 = time.time()
        caps_table = B.tune_colour_caps(params, rule, db, nrm_b, dx, [[8, 2], [8, 1]], reps=1)
        t_tune += time.time() - t0
        ratios = B.rule_ratios(bvec, nrm_b)
        rule = [min(bitsel.rule_of(q) for q in ratios[s * nrhs:(s + 1) * nrhs]) for s in range(B.nsys)]
    bits = list(rule)
    learned = None
    if os.path.exists(bitsel.WEIGHTS):
        sel = bitsel.Selector(ctx)
        learned = [sel.choose(sagb.setup_features(B.system_setup(s), float(ratios[s * nrhs])), rule[s])
                   for s in range(B.nsys)]
        sel.net.close()
        bits = learned
    zeros = sagb.DeviceArray.from_host(ctx, np.zeros(B.rows * nrhs))

    def one(bb):
        sagb.check(sagb.lib().sa_memcpy(ctx.h, dx.ptr, zeros.ptr, 8 * B.rows * nrhs))
        return B.solve(params, bb, db, nrm_b, dx)

    for _ in range(a.warmup):
        one(bits)
    clocks = Clocks(dist.local)
    e0, e1 = sagb.Event(), sagb.Event()
    dist.barrier()
    ctx.sync()
    l0 = ctx.launches()
    clocks.start()
    e0.record(ctx)
    for _ in range(a.steps):
        it, cv, fb = one(bits)
    e1.record(ctx)
    ctx.sync()
    clk = clocks.stop()
    launches = ctx.launches() - l0
    sec = dist.max(e0.elapsed_ms(e1) / 1000.0 / a.steps)
    X = dx.download().reshape(B.rows, nrhs)
    worst = 0.0
    for s, (r, c, v) in enumerate(systems):
        rows = np.repeat(np.arange(len(r) - 1), np.diff(r))
        xs = X[B.offsets[s]:B.offsets[s + 1]]
        for q in range(nrhs):
            res = np.linalg.norm(bs[s][:, q] - np.bincount(rows, weights=v * xs[c, q], minlength=len(r) - 1))
            worst = max(worst, res / nrm_b[s * nrhs + q])
    # the rule's bits on the same batch, for comparison
    rule_row = None
    if learned is not None:
        one(rule)
        e0.record(ctx)
        itr, cvr, fbr = one(rule)
        e1.record(ctx)
        ctx.sync()
        rule_row = {"value": e0.elapsed_ms(e1) / 1000.0, "iters_total": int(itr.sum()),
                    "iters_max": int(itr.max()), "converged": int(cvr.sum())}
    k = batch_rooflines(ctx, B, a)
    peak, peak_kind = measured_peak()
    sp = next(p for p in k["per_op"] if p["level"] == 0 and p["op"] == "A")
    spa = sp["bytes"] / (sp["ms"] * 1e-3) / 1e9
    fam = k["families"]
    name = max(fam, key=lambda f: fam[f][0])
    ach = fam[name][1] / (fam[name][0] * 1e-3) / 1e9
    if dist.rank == 0:
        line = {
            "metric": "time to 1e-10 explicit relative residual, 256 x 4 batched solves, int-AMG-FGMRES(20)",
            "value": sec, "unit": "s", "n_gpus": dist.world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": sec * 1000, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic 27-point SPD systems, sides U{16..64}, b ~ U[-1,1]",
            "config": {"workload": "batch of 27-point systems x 4 right-hand sides", "nsys": B.nsys,
                       "rows": int(B.rows), "nrhs": nrhs, "m": 20, "depth_max": B.depth,
                       "sides_min_max": [int(sides.min()), int(sides.max())]},
            "pairs_converged": int(cv.sum()), "pairs": int(len(cv)), "iters_total": int(it.sum()),
            "iters_max": int(it.max()), "worst_explicit_res": worst,
            "bits": "learned" if learned is not None else "rule", "rule_row": rule_row,
            "colour_caps": B.colour_caps()[:3], "cycle_bits": a.cycle_bits,
            "colour_cap_tuning": None if caps_table is None else
            [{"caps": t[0], "ms": round(t[1], 3), "iters_max": int(np.max(t[2]))} for t in caps_table],
            "gen_s": t_gen, "setup_s": t_setup, "autotune_s": t_tune, "rule_s": t_rule,
            "gpu_launches": launches, "clocks": clk, "vcycle_ms": k["vcycle_ms"], "coarse_lu_ms": k["coarse_lu_ms"],
            "roofline": {"kernel": name, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                         "frac": ach / peak, "peak_kind": peak_kind, "traffic": None},
            "spmv_A0": {"achieved": spa, "frac": spa / peak, "ms": sp["ms"], "bytes": sp["bytes"]},
            "families_ms_per_vcycle": {f: fam[f][0] for f in fam},
        }
        print(json.dumps(line), flush=True)
    dist.close()


def main_convdiff(a):
    """Learned against rule bits on 3D convection-diffusion 128^3, Pe = 50,
    through the batched engine (one system, one right-hand side)."""
    import bitsel
    import sagb
    dist = Dist(a.gpus)
    ctx = sagb.Context(dist.local)
    A = sagb.HostCsr.generate(sagb.GEN_CONVDIFF3D, a.n, 50.0)
    xs, b = A.rhs(1)
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    nrm_b = float(np.linalg.norm(b))
    B = sagb.Batch(ctx, [(r, c, v)], 1)
    B.autotune(2)
    ratio = float(B.rule_ratios(b, [nrm_b])[0])
    rule = bitsel.rule_of(ratio)
    learned = learned_bits(ctx, B.system_setup(0), ratio)
    rows = {}
    for name, f in (("rule", rule), ("learned", learned)):
        if f is None:
            continue
        x = sagb.DeviceArray(ctx, len(b), np.float64)
        db = sagb.DeviceArray.from_host(ctx, b)
        p = sagb.solver_params(m=a.m, explicit_stop=1, cycle_bits=a.cycle_bits)
        x.upload(np.zeros(len(b)))
        B.solve(p, [f], db, [nrm_b], x)
        e0, e1 = sagb.Event(), sagb.Event()
        x.upload(np.zeros(len(b)))
        e0.record(ctx)
        it, cv, fb = B.solve(p, [f], db, [nrm_b], x)
        e1.record(ctx)
        ctx.sync()
        rows[name] = {"bits": f, "final_bits": int(fb[0]), "iters": int(it[0]), "converged": int(cv[0]),
                      "seconds": e0.elapsed_ms(e1) / 1000.0,
                      "explicit_res": explicit_res(r, c, v, b, x.download())}
        x.close()
        db.close()
    if dist.rank == 0:
        print(json.dumps({"workload": f"3D convection-diffusion {a.n}^3, Pe 50, batched engine, m={a.m}",
                          "ratio": ratio, **rows}), flush=True)
    dist.close()


def profiled_batch(a, ctx, r, c, v):
    """The headline's batch with colour caps --caps and launch shapes from
    --tune-file when it exists (else autotuned and written there), so that a
    run under a profiler does not autotune under the profiler."""
    import sagb
    B = sagb.Batch(ctx, [(r, c, v)], 1)
    if a.caps:
        B.set_colour_caps([int(t) for t in a.caps.split(",")])
    if a.tune_file and os.path.exists(a.tune_file):
        with open(a.tune_file) as f:
            tune = json.load(f)
        for l, (form, groups) in enumerate(zip(tune["forms"], tune["groups"])):
            B.sweep_form(l, form)
            for op, g in enumerate(groups):
                B.set_group(l, op, g)
            for op, on in zip((0, 2), tune.get("compressed", [[0, 0]] * B.depth)[l]):
                B.compressed(l, op, on)
    else:
        B.autotune(2)
        if a.tune_file:
            with open(a.tune_file, "w") as f:
                json.dump({"forms": [B.sweep_form(l) for l in range(B.depth)],
                           "groups": [[B.group(l, op) for op in range(5)] for l in range(B.depth)],
                           "compressed": [[B.compressed(l, 0), B.compressed(l, 2)] for l in range(B.depth)]}, f)
    return B


def main_vcycle(a):
    """Profiling aid: the headline's batched V-cycle (autotuned) on the 128^3
    system (--n), --steps V-cycles inside a profiler collection range (run
    under a profiler started with collection off)."""
    import sagb
    ctx = sagb.Context(0)
    r, c, v, b = build_system(a.n, seed=1)
    B = profiled_batch(a, ctx, r, c, v)
    x = sagb.DeviceArray.from_host(ctx, np.random.default_rng(3).integers(-(1 << 28), 1 << 28, size=B.rows)
                                   .astype(np.int32))
    y = sagb.DeviceArray(ctx, B.rows, np.int32)
    for _ in range(a.warmup):
        B.precondition(x, y)
    ctx.sync()
    l0 = ctx.launches()
    sagb.check(sagb.lib().sa_profiler_range(1))
    for _ in range(a.steps):
        B.precondition(x, y)
    ctx.sync()
    sagb.check(sagb.lib().sa_profiler_range(0))
    print(json.dumps({"workload": f"batched V-cycle, Poisson {a.n}^3", "vcycles": a.steps,
                      "launches": ctx.launches() - l0}), flush=True)


def main_plain_vcycle(a):
    """Profiling aid: the plain drop-in's V-cycle (reference parameters,
    natural-order SOR sweeps) on the 128^3 system (--n), --steps V-cycles
    inside a profiler collection range."""
    import sagb
    ctx = sagb.Context(0)
    r, c, v, b = build_system(a.n, seed=1)
    M = sagb.Amg(ctx, sagb.INT, setup=sagb.Setup(sagb.INT, r, c, v))
    N = len(b)
    x = sagb.DeviceArray.from_host(ctx, np.random.default_rng(3).integers(-(1 << 28), 1 << 28, size=N)
                                   .astype(np.int32))
    y = sagb.DeviceArray(ctx, N, np.int32)
    for _ in range(a.warmup):
        M.precondition(x, y)
    ctx.sync()
    l0 = ctx.launches()
    sagb.check(sagb.lib().sa_profiler_range(1))
    for _ in range(a.steps):
        M.precondition(x, y)
    ctx.sync()
    sagb.check(sagb.lib().sa_profiler_range(0))
    print(json.dumps({"workload": f"plain V-cycle, Poisson {a.n}^3", "vcycles": a.steps,
                      "launches": ctx.launches() - l0}), flush=True)


def main_solve_profile(a):
    """Profiling aid: --steps whole headline solves (rule's F, early restart,
    --caps colour caps, --tune-file shapes) inside a profiler collection range."""
    import sagb
    ctx = sagb.Context(0)
    if a.no_graphs:  # every kernel a launch of its own (a profiler lists them one by one)
        ctx.set_option(sagb.OPT_GRAPHS, 0)
    r, c, v, b = build_system(a.n, seed=1)
    B = profiled_batch(a, ctx, r, c, v)
    N = len(b)
    nb = np.array([np.linalg.norm(b)])
    db = sagb.DeviceArray.from_host(ctx, b)
    dx = sagb.DeviceArray(ctx, N, np.float64)
    p = sagb.solver_params(m=a.m, explicit_stop=1, cycle_bits=a.cycle_bits)
    zeros = np.zeros(N)
    for _ in range(a.warmup):
        dx.upload(zeros)
        B.solve(p, [29], db, nb, dx)
    ctx.sync()
    l0 = ctx.launches()
    its = []
    for _ in range(a.steps):
        dx.upload(zeros)
        ctx.sync()
        sagb.check(sagb.lib().sa_profiler_range(1))
        it, cv, fb = B.solve(p, [29], db, nb, dx)
        ctx.sync()
        sagb.check(sagb.lib().sa_profiler_range(0))
        its.append(int(it[0]))
    print(json.dumps({"workload": f"batched solve, Poisson {a.n}^3", "solves": a.steps, "iters": its,
                      "launches": ctx.launches() - l0}), flush=True)


def main_precision(a):
    """Precision split: int32 fixed-point inner solve with FP64 refinement,
    FP32-mixed and FP64 AMG-FGMRES(30) (all with the bit-exact SOR smoother and
    the reference's algorithms) on the two systems of the precision config.
    Each solution is compared with the exact x* (b = A x*) and with an FP64
    solve run to 1e-14."""
    import sagb
    dist = Dist(a.gpus)
    ctx = sagb.Context(dist.local)
    cases = [("varcoef3d_96_sigma2", sagb.GEN_VARCOEF3D, 96, 2.0), ("aniso2d_1024_eps1e-3", sagb.GEN_ANISO2D, 1024, 1e-3)]
    rows = {}
    for name, kind, n, prm in cases:
        A = sagb.HostCsr.generate(kind, n, prm, seed=7)
        xs, b = A.rhs(11)
        A.lmax1_scaling(b)
        r, c, v = A.arrays()
        N = len(b)
        nrm_b = float(np.linalg.norm(b))
        t0 = time.time()
        s_int = sagb.Setup(sagb.INT, r, c, v)
        s64, s32 = s_int.derive(sagb.F64), s_int.derive(sagb.F32)
        t_setup = time.time() - t0
        M, M64, M32 = (sagb.Amg(ctx, p, setup=st) for p, st in ((sagb.INT, s_int), (sagb.F64, s64), (sagb.F32, s32)))
        dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
        iA = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
        fA = sagb.Matrix(ctx, sagb.MAT_F32, r, c, v)
        bits = sagb.rule_bits(ctx, M64, b, nrm_b)
        db = sagb.DeviceArray.from_host(ctx, b)
        dx = sagb.DeviceArray(ctx, N, np.float64)

        def run(prec, A_, M_, eps, fb=1):
            S = sagb.Solver(ctx, prec, dA, A_, M_, sagb.solver_params(m=a.m, eps=eps, frac_bits=bits,
                                                                      explicit_stop=1, overflow_fallback=fb))
            dx.upload(np.zeros(N))
            e0, e1 = sagb.Event(), sagb.Event()
            e0.record(ctx)
            it, cv = S.solve(db, nrm_b, dx)
            e1.record(ctx)
            ctx.sync()
            _, flags = S.history()
            nb = C.c_int()
            sagb.check(sagb.lib().sa_solver_bits(S.h, C.byref(nb)))
            S.close()
            return it, cv, e0.elapsed_ms(e1) / 1000.0, dx.download(), flags, nb.value

        *_, x_ref, _, _ = run(sagb.F64, dA, M64, 1e-14)
        row = {"rows": N, "setup_s": t_setup, "rule_bits": bits}
        for label, prec, A_, M_ in (("int_fp64ir", sagb.INT, iA, M), ("fp32_mixed", sagb.F32, fA, M32),
                                    ("fp64", sagb.F64, dA, M64)):
            it, cv, sec, x, flags, fbits = run(prec, A_, M_, 1e-10)
            row[label] = {"iters": it, "converged": bool(cv), "seconds": sec,
                          "explicit_res": explicit_res(r, c, v, b, x),
                          "err_vs_xstar": float(np.linalg.norm(x - xs) / np.linalg.norm(xs)),
                          "err_vs_fp64": float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref)),
                          "status_flags": flags, "final_bits": fbits if prec == sagb.INT else None}
        rows[name] = row
        for o in (M, M64, M32, dA, iA, fA, db, dx):
            o.close()
    if dist.rank == 0:
        print(json.dumps({"workload": "precision split (int + FP64 IR / FP32-mixed / FP64), m=%d" % a.m, **rows}),
              flush=True)
    dist.close()


if __name__ == "__main__":
    args = parse()
    if args.impl == "reference":
        main_reference(args)
    elif args.workload == "batch256":
        main_batch(args)
    elif args.workload == "convdiff128":
        main_convdiff(args)
    elif args.workload == "precision":
        main_precision(args)
    elif args.workload == "vcycle":
        main_vcycle(args)
    elif args.workload == "solve":
        main_solve_profile(args)
    elif args.workload == "plain_vcycle":
        main_plain_vcycle(args)
    else:
        main_ours(args)
