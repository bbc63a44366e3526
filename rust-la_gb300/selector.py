"""Learned precision selector for batched mixed-precision solves.

Each system of a batch is factored in FP32 arithmetic with its LU factors
stored in FP8 (e4m3), BF16 or FP32, then refined in FP64; systems whose
refinement stalls are redone by the plan's FP64 pass, which is also the arbiter
of every answer (backward error <= tol or FP64). Narrow storage lets larger
systems factor in shared memory, but converges only for well-conditioned
systems: the best class depends on n and on the conditioning.

``PrecisionSelector`` picks the class per system from 16 cheap features
(la_batch_features_device) with a 16 -> 64 -> 64 -> 3 MLP trained on the GPU
(la_mlp_*). Labels come from running the batch once per class and taking, per
system, the class with the fewest measured SM cycles including the FP64 redo
(``measure_costs``). A gate on top of the network (``fit_gate``, applied on the
device by la_mlp_set_gate) sends the systems that the network's outputs and the
features mark as beyond what refinement of low-precision factors can
reach straight to the plan's FP64 pass, so that they do not pay for a mixed
attempt first: a linear score of the raw features and the class
probabilities, fitted by logistic regression on the same labelled data against
the cycles of the plain FP64 plan. Everything runs through the C ABI of liblagpu.so; torch
only provides device memory.
"""
import json
import os

import numpy as np
import torch

import la_gpu

CLASS_NAMES = ("fp8", "bf16", "fp32")
CLASS_PREC = la_gpu.SELECTOR_CLASSES


def conditioned_batch(ctx, count, seed, n_range=(16, 512), nrhs_range=(1, 4),
                      log10_kappa=(1.0, 12.0)):
    """count Householder-conditioned systems on the device: n uniform in
    n_range, nrhs uniform in nrhs_range, log10 kappa_2 uniform in log10_kappa.
    Returns (systems, dA, dB, dX, kappa) with dA/dB/dX torch FP64 tensors."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=count)
    rs = rng.integers(nrhs_range[0], nrhs_range[1] + 1, size=count)
    systems, na, nb = la_gpu.batch_systems(ns, rs)
    da = torch.empty(na, dtype=torch.float64, device="cuda")
    db = torch.empty(nb, dtype=torch.float64, device="cuda")
    dx = torch.zeros(nb, dtype=torch.float64, device="cuda")
    dk = torch.empty(count, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    la_gpu.generate_conditioned_batch(ctx, systems, log10_kappa[0], log10_kappa[1],
                                      int(seed) * 7919 + 17, da.data_ptr(), db.data_ptr(),
                                      dk.data_ptr())
    return systems, da, db, dx, dk.cpu().numpy()


def features(ctx, systems, da):
    """[count, 16] FP32 features on the device."""
    f = torch.empty((len(systems), 16), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    la_gpu.batch_features_device(ctx, da.data_ptr(), systems, f.data_ptr())
    return f


def measure_costs(ctx, systems, da, db, dx, ctas_per_sm=2, warps_per_system=8, tol=1e-14,
                  max_iters=10, reps=1):
    """Runs the mixed plan with every system in each class in turn. Returns
    (cycles [count, 3] int64, converged [count, 3] bool): SM cycles spent per
    system (mixed attempt plus FP64 redo) and whether refinement converged."""
    count = len(systems)
    cyc = np.zeros((count, 3), dtype=np.int64)
    conv = np.zeros((count, 3), dtype=bool)
    plan = la_gpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems,
                            la_gpu.BATCH_MIXED, ctas_per_sm=ctas_per_sm,
                            warps_per_system=warps_per_system, tol=tol, max_iters=max_iters)
    try:
        sel = torch.empty(count, dtype=torch.int32, device="cuda")
        for c in range(3):
            sel.fill_(c)
            torch.cuda.synchronize()
            plan.select_device(sel.data_ptr())
            best = None
            for _ in range(reps):
                plan.run()
                cur = plan.cycles()
                best = cur if best is None else np.minimum(best, cur)
            cyc[:, c] = best
            _, _, fb = plan.stats()
            conv[:, c] = fb == 0
    finally:
        plan.free()
    return cyc, conv


def fp64_costs(ctx, systems, da, db, dx, ctas_per_sm=1, warps_per_system=8):
    """SM cycles per system of the plain FP64 plan (the cost of sending a
    system straight to the FP64 pass). One 8-warp CTA per SM: a system of
    n = 512 in FP64 needs a whole SM's shared memory."""
    plan = la_gpu.BatchPlan(ctx, da.data_ptr(), db.data_ptr(), dx.data_ptr(), systems,
                            la_gpu.BATCH_FP64, ctas_per_sm=ctas_per_sm,
                            warps_per_system=warps_per_system)
    try:
        plan.run()
        return plan.cycles()
    finally:
        plan.free()


def fit_gate(probs, feats, cycles, cycles64, steps=3000, lr=0.5, seed=0):
    """Fits the gate that sends a system straight to the FP64 pass: a linear
    score of the 16 raw features and the network's 3 class probabilities,
    learned by logistic regression (gradient descent on standardised inputs)
    on whether the FP64 plan costs fewer cycles than the network's class, each
    system weighted by the cycles at stake; the bias is then shifted to the
    value that minimises the summed cycles. probs [m,3], feats [m,16] raw,
    cycles [m,3], cycles64 [m]. Returns (coef[19] in raw units, bias, cost
    ratio to the ungated choice)."""
    pred = np.argmax(probs, axis=1)
    base = cycles[np.arange(len(pred)), pred].astype(np.float64)
    gain = base - cycles64.astype(np.float64)  # cycles saved by gating each system
    X = np.concatenate([feats, probs], axis=1).astype(np.float64)
    mu, sd = X.mean(0), X.std(0) + 1e-9
    Z = (X - mu) / sd
    y = (gain > 0).astype(np.float64)
    w = np.abs(gain) / max(np.abs(gain).mean(), 1e-30)
    W = np.zeros(Z.shape[1])
    b = 0.0
    for _ in range(steps):
        p = 1.0 / (1.0 + np.exp(-(Z @ W + b)))
        g = (p - y) * w
        W -= lr * (Z.T @ g) / len(Z)
        b -= lr * g.mean()
    score = Z @ W + b
    total0 = base.sum()
    best_t, best_ratio = 0.0, 1.0
    for t in np.quantile(score, np.linspace(0.0, 1.0, 401)):
        ratio = (total0 - gain[score >= t].sum()) / total0
        if ratio < best_ratio:
            best_t, best_ratio = float(t), float(ratio)
    coef = W / sd
    bias = b - float((W * mu / sd).sum()) - best_t
    return coef.astype(np.float32), float(bias), best_ratio


def labels_from_costs(cycles):
    """Cheapest class per system."""
    return np.argmin(cycles, axis=1).astype(np.int32)


class PrecisionSelector:
    """MLP precision selector (la_mlp) with feature normalisation."""

    def __init__(self, ctx, seed=0):
        self.ctx = ctx
        self.mlp = la_gpu.Mlp(ctx, seed)
        self.gate = None

    def fit(self, feats, labels, steps=1500, lr=3e-3, batch=4096, seed=0, log_every=0,
            costs=None):
        """Adam on minibatches of (feats [m,16] FP32 device, labels [m] int32):
        the cross-entropy of the labels, or, with costs ([m, 3], each system's
        cost of each class, e.g. measured cycles scaled to a mean near 1), the
        expected cost. Sets the input normalisation from feats. Returns the
        loss log."""
        feats = feats.contiguous()
        labels = torch.as_tensor(labels, dtype=torch.int32, device="cuda").contiguous()
        if costs is not None:
            costs = torch.as_tensor(costs, dtype=torch.float32, device="cuda").contiguous()
        m = feats.shape[0]
        p = self.mlp.get_params()
        npar = self.mlp.nparam
        mean = feats.double().mean(0)
        std = feats.double().std(0).clamp_min(1e-3)
        p[npar:npar + 16] = mean.cpu().numpy()
        p[npar + 16:npar + 32] = std.cpu().numpy()
        self.mlp.set_params(p)
        rng = np.random.default_rng(seed)
        batch = min(batch, m)
        log = []
        perm = torch.from_numpy(rng.permutation(m)).cuda()
        pos = 0
        for step in range(steps):
            if pos + batch > m:
                perm = torch.from_numpy(rng.permutation(m)).cuda()
                pos = 0
            idx = perm[pos:pos + batch]
            pos += batch
            xb = feats.index_select(0, idx).contiguous()
            yb = labels.index_select(0, idx).contiguous()
            cb = costs.index_select(0, idx).contiguous() if costs is not None else None
            torch.cuda.synchronize()
            want = bool(log_every) and (step % log_every == 0 or step == steps - 1)
            if cb is not None:
                loss = self.mlp.train_step_cost(xb.data_ptr(), cb.data_ptr(), batch, lr,
                                                want_loss=want)
            else:
                loss = self.mlp.train_step(xb.data_ptr(), yb.data_ptr(), batch, lr,
                                           want_loss=want)
            if want:
                log.append((step, loss))
        self.ctx.synchronize()
        return log

    def set_gate(self, coef, bias=0.0):
        """Class 3 (straight to the FP64 pass) where the gate's score
        coef[:16] . x + coef[16:] . p + bias >= 0; coef None: no gate."""
        self.gate = None if coef is None else (np.asarray(coef, dtype=np.float32), float(bias))
        self.mlp.set_gate(coef, bias)

    def probs(self, feats):
        """[m, 3] class probabilities (device FP32 tensor)."""
        pr = torch.empty((feats.shape[0], 3), dtype=torch.float32, device="cuda")
        self.mlp.predict(feats.data_ptr(), feats.shape[0], pr.data_ptr(), None)
        self.ctx.synchronize()
        return pr

    def predict(self, feats, out=None, sync=True):
        """Class per system (device int32 tensor). With sync=False the result
        is ordered on the context's stream only (e.g. for a plan's
        select_device)."""
        cls = out if out is not None else torch.empty(feats.shape[0], dtype=torch.int32,
                                                      device="cuda")
        self.mlp.predict(feats.data_ptr(), feats.shape[0], None, cls.data_ptr())
        if sync:
            self.ctx.synchronize()
        return cls

    def loss(self, feats, labels):
        labels = torch.as_tensor(labels, dtype=torch.int32, device="cuda").contiguous()
        torch.cuda.synchronize()
        return self.mlp.gradients(feats.data_ptr(), labels.data_ptr(), feats.shape[0])[1]

    def params(self):
        return self.mlp.get_params()

    def load(self, params):
        self.mlp.set_params(np.asarray(params, dtype=np.float32))

    def save(self, path):
        np.save(path, self.params())

    def save_gate(self, path):
        with open(path, "w") as f:
            json.dump({"coef": [float(v) for v in self.gate[0]], "bias": self.gate[1]}, f,
                      indent=1)

    @classmethod
    def from_file(cls, ctx, path, gate=True):
        """Weights from `path`; the gate from the .gate.json file beside it
        when it exists and `gate` is true."""
        s = cls(ctx)
        s.load(np.load(path))
        gpath = os.path.splitext(path)[0] + ".gate.json"
        if gate and os.path.exists(gpath):
            g = json.load(open(gpath))
            s.set_gate(g["coef"], g["bias"])
        return s
