"""Build the bit-sweep dataset on the GPU and train the selector's MLP.

    python sc23-ad_gb300/train_bitsel.py [--count 600] [--side 16 64] [--seed 7]
                                         [--epochs 400] [--train-only]

Writes data/bitsel_dataset.npz (features, targets and every sweep point) and
data/bitsel_mlp.npz (weights and input standardisation), and prints a JSON
line with the held-out comparison against the rule of Work/main.cpp:160 with its
overflow fallback: for the last 20 % of the matrices, the iterations of the
solve at the selected F (plus the rule's solve when the selected F fails)
against the rule's F or, where it fails, the first F below it that converges,
all read from the sweep.
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import bitsel  # noqa: E402
import sagb  # noqa: E402


def rule_with_fallback(sw, rule, fail_cost):
    """Iterations of the rule's F with the overflow fallback (a failing F is
    redone with one bit less), read from the sweep: the first F at or below the
    rule's that converges.  The discarded attempts are not charged, so this
    favours the rule."""
    for f in range(rule, bitsel.F_LO - 1, -1):
        q = sw.get(f)
        if q is not None and q["converged"]:
            return q["iters"], f == rule
    return fail_cost, False


def evaluate(net, f_lo, X, meta, x_range, fail_cost=120, margin=bitsel.MARGIN):
    """Iterations at the selected F (the network's argmin over the features
    clamped to the training range, kept only when it beats the rule's
    predicted cost by `margin` log2 units) against the rule's F with its
    fallback, from the sweep; a selected F that fails costs fail_cost
    iterations plus the rule's solve with fallback."""
    rows = []
    Y = net.predict(bitsel.clamp_features(X, x_range))
    for k in range(len(X)):
        sw = {q["bit"]: q for q in meta[k]["sweep"]}
        rule = meta[k]["rule"]
        if rule not in sw:
            continue
        f = f_lo + int(np.argmin(Y[k]))
        if Y[k][rule - f_lo] - Y[k][f - f_lo] < margin:
            f = rule
        r_it, rule_ok = rule_with_fallback(sw, rule, fail_cost)
        q = sw[f]
        ok = bool(q["converged"])
        it_sel = q["iters"] if ok else fail_cost + r_it
        best = min(sw.values(), key=lambda z: (not z["converged"], z["iters"]))
        rows.append({"bit": f, "rule": rule, "best": best["bit"], "it_sel": it_sel, "it_rule": r_it,
                     "it_best": best["iters"], "fallback": not ok, "rule_ok": rule_ok,
                     "worse": it_sel > r_it})
    return rows


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=600)
    ap.add_argument("--side", type=int, nargs=2, default=[16, 64])
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--epochs", type=int, default=400)
    ap.add_argument("--train-only", action="store_true", help="reuse the dataset file")
    ap.add_argument("--parts", nargs="*", default=None,
                    help="dataset files (written by partial sweeps) to merge instead of sweeping")
    ap.add_argument("--out", default=bitsel.DATA, help="folder for the dataset and the weights")
    a = ap.parse_args()
    ctx = sagb.Context(0)
    if a.parts:
        Xs, Ts, meta = [], [], []
        for path in a.parts:
            z = np.load(path)
            Xs.append(z["X"])
            Ts.append(z["T"])
            meta += json.loads(str(z["meta"]))
        X, T = np.concatenate(Xs), np.concatenate(Ts)
        # one seeded shuffle, so that every part (a later part may hold larger
        # systems) lands in both the training and the held-out share
        perm = np.random.default_rng(a.seed).permutation(len(X))
        X, T, meta = X[perm], T[perm], [meta[i] for i in perm]
        os.makedirs(a.out, exist_ok=True)
        np.savez_compressed(os.path.join(a.out, os.path.basename(bitsel.DATASET)), X=X, T=T, meta=json.dumps(meta))
    elif a.train_only:
        z = np.load(os.path.join(a.out, os.path.basename(bitsel.DATASET)))
        X, T, meta = z["X"], z["T"], json.loads(str(z["meta"]))
    else:
        specs = bitsel.training_specs(a.count, a.seed, tuple(a.side))
        t0 = time.time()
        X, T, meta = bitsel.build_dataset(ctx, specs, log=lambda s: print(s, file=sys.stderr, flush=True))
        print(f"sweeps: {time.time() - t0:.1f}s", file=sys.stderr)
        os.makedirs(a.out, exist_ok=True)
        np.savez_compressed(os.path.join(a.out, os.path.basename(bitsel.DATASET)), X=X, T=T, meta=json.dumps(meta))
    n = len(X)
    ntr = int(round(0.8 * n))
    t0 = time.time()
    net, mu, sd, hist = bitsel.train(ctx, X[:ntr], T[:ntr], epochs=a.epochs, seed=a.seed)
    t_train = time.time() - t0
    x_range = (X[:ntr].min(0), X[:ntr].max(0))
    ev = evaluate(net, bitsel.F_LO, X[ntr:], meta[ntr:], x_range)
    summ = {
        "train_matrices": ntr, "heldout_matrices": len(ev), "epochs": a.epochs, "train_seconds": t_train,
        "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
        "heldout_iters_selected": int(sum(r["it_sel"] for r in ev)),
        "heldout_iters_rule_with_fallback": int(sum(r["it_rule"] for r in ev)),
        "heldout_selected_worse_than_rule": int(sum(r["worse"] for r in ev)),
        "heldout_iters_best": int(sum(r["it_best"] for r in ev)),
        "heldout_selected_is_best": int(sum(r["bit"] == r["best"] for r in ev)),
        "heldout_rule_is_best": int(sum(r["rule"] == r["best"] for r in ev)),
        "heldout_fallbacks": int(sum(r["fallback"] for r in ev)),
        "heldout_rule_failures": int(sum(not r["rule_ok"] for r in ev)),
    }
    bitsel.save(os.path.join(a.out, os.path.basename(bitsel.WEIGHTS)), net, mu, sd, info=summ,
                x_range=x_range)
    print(json.dumps(summ))


if __name__ == "__main__":
    main()
