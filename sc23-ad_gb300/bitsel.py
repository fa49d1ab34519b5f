"""Learned fractional-bit selector for int-AMG-FGMRES.

The reference chooses F_G with a fixed rule (Work/main.cpp:153-161) or by a
manual sweep (Work/sub.cpp, Work/run_sub.sh).  Here the integer solver itself
runs the sweep on synthetic matrices (F = 8..29), a 3-layer 64-wide FP32 MLP
(trained by the library's own CUDA kernels, sagb.Mlp) learns the log2
iteration count of every F from matrix features (sagb.setup_features), and
the selector takes the F with the smallest prediction.  A solve with the
selected F that overflows, or does not converge, is redone with the rule's F.

Training mixture: 5-point 2D (anisotropy 1e-4..1), 7-point 3D Poisson,
27-point, lognormal-coefficient diffusion (sigma 0..3) and upwinded
convection-diffusion (Peclet 0..100); cube sides from a range.
"""
import json
import os
import time

import numpy as np

import sagb

F_LO, F_HI = 8, 29  # the config's 8..28 plus 29, the top value of the rule
N_OUT = F_HI - F_LO + 1
PENALTY = float(np.log2(2000.0))  # target of a sweep point that did not converge
HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(HERE, "data")
WEIGHTS = os.path.join(DATA, "bitsel_mlp.npz")
DATASET = os.path.join(DATA, "bitsel_dataset.npz")


def rule_of(ratio):
    """Work/main.cpp:160."""
    return 29 if ratio < 1 else 31 - (int(np.ceil(np.log2(int(ratio) + 1))) + 1)


def training_specs(count, seed, side=(16, 64)):
    """(kind, nx, param, seed, rhs) of `count` matrices from the training
    mixture; rhs 0: b = A x* with x* ~ U[-1, 1], rhs 1: b ~ U[-1, 1]."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(count):
        fam = int(rng.integers(0, 5))
        s3 = int(rng.integers(side[0], side[1] + 1))
        rhs = int(rng.integers(0, 2))
        if fam == 0:    # 5-point 2D, anisotropy 1e-4..1 (side^1.5 rows ~ a 3D cube's)
            n2 = int(round(s3 ** 1.5))
            specs.append((sagb.GEN_ANISO2D, n2, float(10 ** rng.uniform(-4, 0)), k + 1, rhs))
        elif fam == 1:  # 7-point 3D Poisson
            specs.append((sagb.GEN_POISSON3D, s3, 0.0, k + 1, rhs))
        elif fam == 2:  # 27-point
            specs.append((sagb.GEN_STENCIL27, s3, 0.0, k + 1, rhs))
        elif fam == 3:  # lognormal coefficients
            specs.append((sagb.GEN_VARCOEF3D, s3, float(rng.uniform(0, 3)), k + 1, rhs))
        else:           # upwinded convection-diffusion
            specs.append((sagb.GEN_CONVDIFF3D, s3, float(rng.uniform(0, 100)), k + 1, rhs))
    return specs


def make_system(spec):
    kind, nx, prm, sd = spec[:4]
    rhs = spec[4] if len(spec) > 4 else 0
    A = sagb.HostCsr.generate(kind, nx, prm, seed=sd)
    xs, b = A.rhs(sd)
    if rhs == 1:
        b = np.random.default_rng(sd).uniform(-1.0, 1.0, size=len(b))
    A.lmax1_scaling(b)
    r, c, v = A.arrays()
    return r, c, v, b


class Prepared:
    """Setup, GPU operators, rule ratio and features of one system."""

    def __init__(self, ctx, r, c, v, b, multicolor=1):
        self.r, self.c, self.v, self.b = r, c, v, b
        self.nrm_b = float(np.linalg.norm(b))
        t0 = time.time()
        self.s_int = sagb.Setup(sagb.INT, r, c, v, sagb.amg_params(multicolor=multicolor))
        s64 = self.s_int.derive(sagb.F64)
        self.setup_s = time.time() - t0
        self.M = sagb.Amg(ctx, sagb.INT, setup=self.s_int)
        M64 = sagb.Amg(ctx, sagb.F64, setup=s64)
        self.dA = sagb.Matrix(ctx, sagb.MAT_F64, r, c, v)
        self.iA = sagb.Matrix(ctx, sagb.MAT_FIXED, r, c, v, bit=30)
        self.ratio = sagb.rule_ratio(ctx, M64, b, self.nrm_b)
        self.rule = rule_of(self.ratio)
        self.features = sagb.setup_features(self.s_int, self.ratio)
        M64.close()
        self.ctx = ctx

    def solve(self, bit, m=30, max_outer=33, fallback=0):
        """One solve at F = bit: (iterations, converged, explicit residual, seconds, flags)."""
        ctx = self.ctx
        p = sagb.solver_params(m=m, frac_bits=bit, explicit_stop=1, overflow_fallback=fallback,
                               max_outer=max_outer)
        S = sagb.Solver(ctx, sagb.INT, self.dA, self.iA, self.M, p)
        x = sagb.DeviceArray.from_host(ctx, np.zeros(len(self.b)))
        db = sagb.DeviceArray.from_host(ctx, self.b)
        e0, e1 = sagb.Event(), sagb.Event()
        ctx.flags(clear=True)
        e0.record(ctx)
        it, conv = S.solve(db, self.nrm_b, x)
        e1.record(ctx)
        ctx.sync()
        sec = e0.elapsed_ms(e1) / 1000.0
        _, flags = S.history()
        xs = x.download()
        rows = np.repeat(np.arange(len(self.r) - 1), np.diff(self.r))
        res = float(np.linalg.norm(self.b - np.bincount(rows, weights=self.v * xs[self.c], minlength=len(self.b)))
                    / self.nrm_b)
        S.close()
        x.close()
        db.close()
        return int(it), int(conv), res, sec, int(flags)

    def close(self):
        for o in (self.M, self.dA, self.iA):
            o.close()


def sweep(ctx, prep, bits=range(F_LO, F_HI + 1), m=30, max_outer=4):
    """Iterations of the integer solver for every F (no overflow fallback, so an
    overflowing F counts as a failure)."""
    out = []
    for f in bits:
        it, conv, res, sec, flags = prep.solve(f, m=m, max_outer=max_outer, fallback=0)
        out.append({"bit": f, "iters": it, "converged": int(conv and res <= 1e-10), "res": res, "seconds": sec,
                    "flags": flags})
    return out


def targets(rows):
    T = np.full(N_OUT, PENALTY, np.float32)
    for q in rows:
        if q["converged"] and q["iters"] > 0:
            T[q["bit"] - F_LO] = np.log2(q["iters"])
    return T


# the engine the labels come from: the batched solver's early restart (a cycle
# ends once its estimate has fallen 2^12) and a cap on restarts for the sweep
CYCLE_BITS = 12
SWEEP_MAX_OUTER = 16


def _chunks(specs, chunk, max_rows, nb):
    """Consecutive groups of at most `chunk` matrices whose nb copies stay
    under max_rows rows together."""
    k0 = 0
    while k0 < len(specs):
        rows, k1 = 0, k0
        while k1 < len(specs) and k1 - k0 < chunk:
            kind, nx = specs[k1][0], specs[k1][1]
            n = nx * nx if kind in (sagb.GEN_POISSON2D, sagb.GEN_ANISO2D) else nx ** 3
            if k1 > k0 and rows + n * nb > max_rows:
                break
            rows += n * nb
            k1 += 1
        yield k0, specs[k0:k1]
        k0 = k1


def build_dataset(ctx, specs, chunk=16, m=30, max_outer=SWEEP_MAX_OUTER, cycle_bits=CYCLE_BITS,
                  max_rows=24_000_000, log=None, done=None):
    """Sweep every F of every matrix with the batched solver: the copies of one
    matrix (one per F) share one setup, and up to `chunk` matrices (at most
    max_rows rows with all copies) run together.  A point counts as converged
    when the explicit residual reaches 1e-10 within max_outer restarts without
    overflow fallback.  done(X, T, meta), if given, is called after every
    chunk with everything so far."""
    bits = list(range(F_LO, F_HI + 1))
    nb = len(bits)
    X, T, meta = [], [], []
    for k0, part in _chunks(specs, chunk, max_rows, nb):
        t0 = time.time()
        mats = [make_system(sp) for sp in part]
        systems = []
        for r, c, v, b in mats:
            systems += [(r, c, v)] * nb
        B = sagb.Batch(ctx, systems, 1)
        t_setup = time.time() - t0
        feats, rules, ratios = [], [], []
        for i, (r, c, v, b) in enumerate(mats):
            s_int = B.system_setup(i * nb)
            M64 = sagb.Amg(ctx, sagb.F64, setup=s_int.derive(sagb.F64))
            q = sagb.rule_ratio(ctx, M64, b, float(np.linalg.norm(b)))
            M64.close()
            feats.append(sagb.setup_features(s_int, q))
            ratios.append(q)
            rules.append(rule_of(q))
        bvec = np.concatenate([np.tile(b, 1) for r, c, v, b in mats for _ in range(nb)])
        nrm_b = np.array([np.linalg.norm(b) for r, c, v, b in mats for _ in range(nb)])
        x = np.zeros(B.rows)
        p = sagb.solver_params(m=m, max_outer=max_outer, explicit_stop=1, overflow_fallback=0,
                               cycle_bits=cycle_bits)
        t1 = time.time()
        it, cv, fb = B.solve(p, bits * len(mats), bvec, nrm_b, x)
        t_solve = time.time() - t1
        for i, (r, c, v, b) in enumerate(mats):
            rows_i = np.repeat(np.arange(len(r) - 1), np.diff(r))
            out = []
            for j, f in enumerate(bits):
                s = i * nb + j
                xs = x[B.offsets[s]:B.offsets[s + 1]]
                res = float(np.linalg.norm(b - np.bincount(rows_i, weights=v * xs[c], minlength=len(b)))
                            / np.linalg.norm(b))
                out.append({"bit": f, "iters": int(it[s]), "converged": int(cv[s] and res <= 1e-10), "res": res})
            X.append(feats[i])
            T.append(targets(out))
            meta.append({"spec": [int(part[i][0]), int(part[i][1]), float(part[i][2]), int(part[i][3]),
                                  int(part[i][4]) if len(part[i]) > 4 else 0],
                         "rule": rules[i], "ratio": ratios[i], "rows": len(r) - 1, "sweep": out})
            if log:
                best = min(out, key=lambda q: (not q["converged"], q["iters"]))
                rule_pt = next((q for q in out if q["bit"] == rules[i]), None)
                log(f"[{k0 + i + 1}/{len(specs)}] spec={part[i]} rule={rules[i]} "
                    f"({rule_pt['iters'] if rule_pt else '-'} it) best={best['bit']} ({best['iters']} it)")
        B.close()
        if log:
            log(f"  chunk of {len(part)} setup {t_setup:.1f}s solve {t_solve:.1f}s")
        if done:
            done(np.array(X, np.float32), np.array(T, np.float32), meta)
    return np.array(X, np.float32), np.array(T, np.float32), meta


def train(ctx, X, T, epochs=400, batch=64, lr=2e-3, seed=1, hidden=64):
    M = np.ones_like(T)
    mu = X.mean(0)
    sd = X.std(0)
    sd[sd < 1e-6] = 1.0
    net = sagb.Mlp(ctx, X.shape[1], hidden, T.shape[1], seed=seed)
    net.set_norm(mu, sd)
    hist = net.train(X, T, M, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, mu, sd, hist


def save(path, net, mu, sd, info=None, x_range=None):
    """Weights, input standardisation and the range of every feature over the
    training matrices (x_range = (lo, hi))."""
    os.makedirs(os.path.dirname(path), exist_ok=True)
    lo, hi = x_range if x_range is not None else (np.full(net.n_in, -np.inf), np.full(net.n_in, np.inf))
    np.savez(path, params=net.params(), mu=mu, sd=sd, n_in=net.n_in, n_out=net.n_out, hidden=64,
             f_lo=F_LO, x_lo=np.asarray(lo, np.float32), x_hi=np.asarray(hi, np.float32),
             info=json.dumps(info or {}))


def load(ctx, path=WEIGHTS):
    """(network, first F, (lo, hi) feature range of the training matrices)."""
    z = np.load(path)
    net = sagb.Mlp(ctx, int(z["n_in"]), int(z["hidden"]), int(z["n_out"]))
    net.set_params(z["params"])
    net.set_norm(z["mu"], z["sd"])
    n = int(z["n_in"])
    lo = z["x_lo"] if "x_lo" in z else np.full(n, -np.inf, np.float32)
    hi = z["x_hi"] if "x_hi" in z else np.full(n, np.inf, np.float32)
    return net, int(z["f_lo"]), (lo, hi)


def clamp_features(features, x_range):
    """Features moved into the training range: the network is never asked about
    a point outside what it was trained on (a larger system than any training
    one is described as the largest one)."""
    lo, hi = x_range
    return np.clip(np.asarray(features, np.float32), lo, hi)


# the selector leaves the rule's F only when the network predicts at least this
# much (log2 iterations: a factor of 2.8) fewer iterations.  On the held-out
# sweeps a margin of 1.5 keeps nearly all of the gain of a margin of 1 (-8.7 %
# against -9.2 % iterations) with fewer matrices worse than the rule (9 against
# 10) and no failing choice; a margin of 2 keeps the rule's F on more of the
# anisotropic systems where that F overflows.  It also keeps the rule where a
# prediction extrapolates smaller systems, e.g. convection-diffusion 128^3
# (predicted 1.3 apart at F = 27; measured 59 against 34 iterations)
MARGIN = 1.5


class Selector:
    """Learned F with the rule as default and as fallback."""

    def __init__(self, ctx, path=WEIGHTS, margin=MARGIN):
        self.net, self.f_lo, self.x_range = load(ctx, path)
        self.margin = margin

    def choose(self, features, rule=None):
        y = self.net.predict(clamp_features(features, self.x_range))[0]
        f = self.f_lo + int(np.argmin(y))
        if rule is not None and F_LO <= rule <= F_HI and y[rule - self.f_lo] - y[f - self.f_lo] < self.margin:
            return rule
        return f

    def solve(self, prep, m=30):
        """Solve with the learned F; on overflow or failure, with the rule's F.
        Returns (bit used, iterations, converged, residual, seconds, fell_back)."""
        f = self.choose(prep.features, prep.rule)
        it, conv, res, sec, flags = prep.solve(f, m=m, fallback=0)
        if conv and res <= 1e-10:
            return f, it, conv, res, sec, False
        it2, conv2, res2, sec2, _ = prep.solve(prep.rule, m=m, fallback=1)
        return prep.rule, it + it2, conv2, res2, sec + sec2, True
