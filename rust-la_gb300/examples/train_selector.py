"""Trains the precision selector and writes its weights.

    python rust-la_gb300/examples/train_selector.py [--train 200000] [--test 50000]
        [--out rust-la_gb300/selector_weights.npy] [--summary path.json] [--gate-only]
        [--dump path.npz] [--gate-from path.npz] [--loss cost|xent]

Training data: --train Householder-conditioned systems (n uniform in [16, 512],
1-4 right-hand sides, log10 kappa_2 uniform in [1, 12]) generated on the GPU
in chunks with their own seeds. Each chunk is solved by the batched mixed plan
three times, with every system's factors stored in FP8, BF16 and FP32 in turn
(the FP64 pass redoing whatever refinement cannot finish); the label of a
system is the class with the fewest SM cycles spent on it, redo included. The
MLP (16 -> 64 -> 64 -> 3) is then trained on the GPU by the library's own
forward, backward and Adam kernels. Each chunk also runs the plain FP64 plan,
whose per-system cycles are the cost of sending a system straight to the FP64
pass; the gate (straight to the FP64 pass where a linear score of the features
and the class probabilities is >= 0, fitted by logistic regression) is fitted on
them and written beside the weights
(<out>.gate.json). --gate-only keeps the weights in --out and fits the gate
alone; --dump writes the labelled training arrays, and --gate-from fits the
gate from such a dump without running the GPU labelling again.

Evaluation: a separately seeded batch of --test systems. Reports the label
accuracy, the summed per-system cycles of the selector's choices against
always-FP32 factors and against the best class per system, and wall-clock
batch times of (features + inference + solve) against always-FP32 factors and
against the plain FP64 plan.

--loss xent (the default) trains the MLP on the cross-entropy of the cheapest
class; --loss cost on the expected cycles (each system's measured cycles of
the three classes, scaled by their overall mean), which weighs a system by
what a wrong class costs it. On the 50,000-system evaluation the expected-cost
network with its gate came out slower (1.016x always-FP32 factors, against
1.060x for the cross-entropy network retrained the same way).
"""
import argparse
import json
import os
import sys
import time

import numpy as np
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import la_gpu  # noqa: E402
import selector as S  # noqa: E402

TRAIN_SEED0 = 1000
TEST_SEED = 7


def labelled_chunk(ctx, count, seed, ctas, warps):
    systems, da, db, dx, kappa = S.conditioned_batch(ctx, count, seed)
    feats = S.features(ctx, systems, da)
    cyc, conv = S.measure_costs(ctx, systems, da, db, dx, ctas_per_sm=ctas,
                                warps_per_system=warps)
    cyc64 = S.fp64_costs(ctx, systems, da, db, dx)
    out = (systems, da, db, dx, kappa, feats, cyc, conv, cyc64)
    return out


def wall(ctx, fn, reps=3):
    best = np.inf
    for _ in range(reps):
        ctx.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        ctx.synchronize()
        best = min(best, time.perf_counter() - t0)
    return best * 1e3


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=200000)
    ap.add_argument("--chunk", type=int, default=25000)
    ap.add_argument("--test", type=int, default=50000)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "..",
                                                  "selector_weights.npy"))
    ap.add_argument("--summary", default=None)
    ap.add_argument("--gate-only", action="store_true")
    ap.add_argument("--dump", default=None)
    ap.add_argument("--gate-from", default=None)
    ap.add_argument("--loss", default="xent", choices=["xent", "cost"])
    args = ap.parse_args()
    if args.gate_from:  # the gate alone, from a dump of labelled data (no GPU)
        d = np.load(args.gate_from)
        coef, bias, gratio = S.fit_gate(d["probs"], d["feats"], d["cycles"], d["cycles64"])
        with open(os.path.splitext(args.out)[0] + ".gate.json", "w") as fh:
            json.dump({"coef": [float(v) for v in coef], "bias": bias}, fh, indent=1)
        print("gate fitted: cycles x%.4f of the ungated choice on %d systems"
              % (gratio, len(d["probs"])))
        return
    ctx = la_gpu.Context(0)
    t_start = time.perf_counter()

    # plan shape for this distribution (mixed plan, FP32 factors)
    probe = S.conditioned_batch(ctx, min(args.chunk, 8000), TRAIN_SEED0 - 1)
    ctas, warps, _ = la_gpu.batch_autotune(ctx, probe[1].data_ptr(), probe[2].data_ptr(),
                                           probe[3].data_ptr(), probe[0], la_gpu.BATCH_MIXED)
    del probe
    print("plan shape: %d CTAs/SM x %d warps" % (ctas, warps), flush=True)

    feats, labels, cycs, cyc64s, convs, ns = [], [], [], [], [], []
    done, k = 0, 0
    while done < args.train:
        m = min(args.chunk, args.train - done)
        systems, da, db, dx, kappa, f, cyc, conv, cyc64 = labelled_chunk(ctx, m, TRAIN_SEED0 + k,
                                                                         ctas, warps)
        feats.append(f.cpu())
        labels.append(S.labels_from_costs(cyc))
        cycs.append(cyc)
        cyc64s.append(cyc64)
        convs.append(conv)
        ns.append(np.array([s.n for s in systems]))
        del systems, da, db, dx
        torch.cuda.empty_cache()
        done += m
        k += 1
        print("labelled %d / %d (class counts %s)" % (done, args.train,
                                                      np.bincount(labels[-1], minlength=3)),
              flush=True)
    X = torch.cat(feats).cuda()
    y = np.concatenate(labels)
    cyc_all, cyc64_all = np.concatenate(cycs), np.concatenate(cyc64s)
    if args.gate_only:
        sel = S.PrecisionSelector.from_file(ctx, args.out, gate=False)
        log, t_fit = [], 0.0
    else:
        sel = S.PrecisionSelector(ctx, seed=1)
        t0 = time.perf_counter()
        costs = None
        if args.loss == "cost":
            c = cyc_all.astype(np.float64)
            costs = torch.from_numpy((c / c.mean()).astype(np.float32)).cuda()
        log = sel.fit(X, y, steps=args.steps, lr=args.lr, batch=4096, log_every=500, costs=costs)
        t_fit = time.perf_counter() - t0
        sel.save(args.out)
    train_acc = float((sel.predict(X).cpu().numpy() == y).mean())
    print("fit %.1f s, loss %s, train accuracy %.3f" % (t_fit, log, train_acc), flush=True)
    probs = sel.probs(X).cpu().numpy()
    fx = X.cpu().numpy()
    coef, bias, gratio = S.fit_gate(probs, fx, cyc_all, cyc64_all)
    print("gate fitted: cycles x%.3f of the ungated choice on the training set" % gratio,
          flush=True)
    sel.set_gate(coef, bias)
    sel.save_gate(os.path.splitext(args.out)[0] + ".gate.json")
    if args.dump:
        np.savez_compressed(args.dump, feats=fx, labels=y, cycles=cyc_all, cycles64=cyc64_all,
                            converged=np.concatenate(convs), n=np.concatenate(ns), probs=probs)
    del X

    # held-out evaluation
    systems, da, db, dx, kappa, f, cyc, conv, cyc64 = labelled_chunk(ctx, args.test, TEST_SEED,
                                                                     ctas, warps)
    lab = S.labels_from_costs(cyc)
    pred = sel.predict(f).cpu().numpy()  # with the gate: 3 = straight to the FP64 pass
    test_acc = float((np.minimum(pred, 2) == lab).mean())
    idx = np.arange(len(lab))
    cyc4 = np.concatenate([cyc, cyc64[:, None]], axis=1)
    c_sel = float(cyc4[idx, pred].sum())
    c_best = float(cyc4.min(axis=1).sum())
    c_f32 = float(cyc[:, 2].sum())
    plan = la_gpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems,
                            la_gpu.BATCH_MIXED, ctas_per_sm=ctas, warps_per_system=warps)
    count = len(systems)
    fp32 = torch.full((count,), 2, dtype=torch.int32, device="cuda")
    best_cls = torch.from_numpy(np.argmin(cyc4, axis=1).astype(np.int32)).cuda()
    cls = torch.empty(count, dtype=torch.int32, device="cuda")
    fbuf = torch.empty((count, 16), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def run_fixed():
        plan.select_device(fp32.data_ptr())
        plan.run()

    def run_best():
        plan.select_device(best_cls.data_ptr())
        plan.run()

    def run_selected():
        la_gpu.batch_features_device(ctx, da.data_ptr(), systems, fbuf.data_ptr())
        sel.predict(fbuf, out=cls, sync=False)
        plan.select_device(cls.data_ptr())
        plan.run()

    def run_features():
        la_gpu.batch_features_device(ctx, da.data_ptr(), systems, fbuf.data_ptr())
        sel.predict(fbuf, out=cls, sync=False)

    t_fixed = wall(ctx, run_fixed)
    t_best = wall(ctx, run_best)
    t_feat = wall(ctx, run_features)
    t_sel = wall(ctx, run_selected)
    its, eta, fb = plan.stats()
    plan.free()
    c64, w64, _ = la_gpu.batch_autotune(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems,
                                        la_gpu.BATCH_FP64)
    p64 = la_gpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems,
                           la_gpu.BATCH_FP64, ctas_per_sm=c64, warps_per_system=w64)
    t_64 = wall(ctx, p64.run)
    p64.free()
    summary = {
        "train_systems": args.train, "test_systems": count, "plan": [ctas, warps],
        "loss": args.loss,
        "train_accuracy": train_acc, "test_accuracy": test_acc,
        "test_label_counts": np.bincount(lab, minlength=3).tolist(),
        "test_pred_counts": np.bincount(pred, minlength=4).tolist(),
        "gate_train_cycle_ratio": gratio, "test_all_classes_fail": int((~conv.any(axis=1)).sum()),
        "cycles_selector_over_fp32": c_sel / c_f32, "cycles_best_over_fp32": c_best / c_f32,
        "ms_fixed_fp32": t_fixed, "ms_best_labels": t_best, "ms_features_inference": t_feat,
        "ms_selector_total": t_sel, "ms_fp64_plan": t_64, "fp64_plan": [c64, w64],
        "selector_fell_back": int(fb.sum()), "max_eta_refined": float(eta.max()),
        "seconds": time.perf_counter() - t_start,
    }
    print(json.dumps(summary), flush=True)
    if args.summary:
        with open(args.summary, "w") as fh:
            json.dump(summary, fh, indent=1)


if __name__ == "__main__":
    main()
