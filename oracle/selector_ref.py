"""CPU oracle for the learned precision selector (test infrastructure only).

The selector has no counterpart in the reference crate: it decides the storage
precision of the LU factors of each system of a batched mixed-precision solve.
This module restates, in numpy, what the CUDA kernels of
rust-la_gb300/csrc/selector.cu compute, so that tests can check them:

* ``mlp_forward`` / ``mlp_loss_grad``: the 16 -> 64 -> 64 -> 3 ReLU/softmax
  network and the analytic gradient of its mean cross-entropy (float64), with
  ``numeric_grad`` (central differences) to pin the analytic gradient itself;
* ``features``: the 16 per-system features on the FP32 rounding of A, with
  the same 4-step Lanczos on A^T A (fixed start vector, full
  reorthogonalisation), the same bisection for the extreme Ritz values and the
  same asymmetry probe ||A q0 - A^T q0|| / ||A q0||.

Nothing here is on the product path.
"""
import numpy as np

NF, H1, H2, NC = 16, 64, 64, 3
SHAPES = [("W1", (H1, NF)), ("b1", (H1,)), ("W2", (H2, H1)), ("b2", (H2,)), ("W3", (NC, H2)),
          ("b3", (NC,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)  # 5443
LK = 4


def unpack(p):
    """Flat parameter vector (+ optional 32 normalisation floats) -> dict."""
    out, o = {}, 0
    for name, shp in SHAPES:
        k = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + k], dtype=np.float64).reshape(shp)
        o += k
    if len(p) >= NPARAM + 2 * NF:
        out["mean"] = np.asarray(p[NPARAM:NPARAM + NF], dtype=np.float64)
        out["std"] = np.asarray(p[NPARAM + NF:NPARAM + 2 * NF], dtype=np.float64)
    else:
        out["mean"], out["std"] = np.zeros(NF), np.ones(NF)
    return out


def _forward(P, X):
    x = (np.asarray(X, dtype=np.float64) - P["mean"]) / P["std"]
    z1 = x @ P["W1"].T + P["b1"]
    h1 = np.maximum(z1, 0.0)
    z2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(z2, 0.0)
    lg = h2 @ P["W3"].T + P["b3"]
    lg = lg - lg.max(axis=1, keepdims=True)
    e = np.exp(lg)
    pr = e / e.sum(axis=1, keepdims=True)
    return x, h1, h2, pr


def mlp_forward(p, X):
    """Class probabilities [count, 3]."""
    return _forward(unpack(p), X)[3]


def mlp_loss_grad(p, X, y):
    """Mean softmax cross-entropy and its gradient w.r.t. the NPARAM weights."""
    P = unpack(p)
    x, h1, h2, pr = _forward(P, X)
    m = x.shape[0]
    y = np.asarray(y)
    loss = -np.mean(np.log(np.maximum(pr[np.arange(m), y], 1e-300)))
    d3 = pr.copy()
    d3[np.arange(m), y] -= 1.0
    d2 = (d3 @ P["W3"]) * (h2 > 0)
    d1 = (d2 @ P["W2"]) * (h1 > 0)
    g = {"W3": d3.T @ h2 / m, "b3": d3.sum(0) / m, "W2": d2.T @ h1 / m, "b2": d2.sum(0) / m,
         "W1": d1.T @ x / m, "b1": d1.sum(0) / m}
    return loss, np.concatenate([g[name].ravel() for name, _ in SHAPES])


def mlp_cost_grad(p, X, cost):
    """Mean expected cost sum_c p_c cost_c (cost [m, 3]) and its gradient
    w.r.t. the NPARAM weights (logit delta p_c (cost_c - sum_j p_j cost_j))."""
    P = unpack(p)
    x, h1, h2, pr = _forward(P, X)
    m = x.shape[0]
    cost = np.asarray(cost, dtype=np.float64)
    ec = (pr * cost).sum(1)
    loss = float(ec.mean())
    d3 = pr * (cost - ec[:, None])
    d2 = (d3 @ P["W3"]) * (h2 > 0)
    d1 = (d2 @ P["W2"]) * (h1 > 0)
    g = {"W3": d3.T @ h2 / m, "b3": d3.sum(0) / m, "W2": d2.T @ h1 / m, "b2": d2.sum(0) / m,
         "W1": d1.T @ x / m, "b1": d1.sum(0) / m}
    return loss, np.concatenate([g[name].ravel() for name, _ in SHAPES])


def numeric_grad(p, X, y, idx, h=1e-6, loss_fn=None):
    """Central-difference derivative of the loss for the parameters in idx."""
    p = np.asarray(p, dtype=np.float64)
    out = []
    for i in idx:
        a, b = p.copy(), p.copy()
        a[i] += h
        b[i] -= h
        f = loss_fn or mlp_loss_grad
        out.append((f(a, X, y)[0] - f(b, X, y)[0]) / (2 * h))
    return np.array(out)


def _tridiag_min_eig(al, be):
    k = len(al)
    lo, hi = np.inf, -np.inf
    for i in range(k):
        r = (abs(be[i - 1]) if i > 0 else 0.0) + (abs(be[i]) if i + 1 < k else 0.0)
        lo, hi = min(lo, al[i] - r), max(hi, al[i] + r)
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        cnt = 0
        q = al[0] - mid
        cnt += q < 0
        for i in range(1, k):
            q = al[i] - mid - be[i - 1] * be[i - 1] / (q if q != 0.0 else 1e-300)
            cnt += q < 0
        if cnt >= 1:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


def _lg(x):
    return np.log10(max(x, 1e-300))


def features(A, nrhs):
    """The 16 selector features of one system. The kernel reads A once in FP64
    and works on its FP32 rounding (FP32 arithmetic, FP64 accumulation of the
    length-n dot products); this restatement uses the same FP32 matrix, FP32
    start vector and FP32-rounded Lanczos vectors, in float64 arithmetic."""
    A = np.asarray(A, dtype=np.float64).astype(np.float32).astype(np.float64)
    n = A.shape[0]
    aa = np.abs(A)
    rs = aa.sum(1)
    cs = aa.sum(0)
    di = np.abs(np.diag(A))
    off = rs - di
    ratio = di / np.maximum(off, 1e-30)
    fro = np.sqrt((aa * aa).sum())
    amax = aa.max()
    f32 = lambda v: np.asarray(v, dtype=np.float32).astype(np.float64)
    q0 = f32(1.0 + 0.5 * np.sin(1.0 + np.arange(n, dtype=np.float32)))
    q = [f32(q0 / np.linalg.norm(q0))]
    aq0 = A @ q[0]
    asym = np.linalg.norm(aq0 - A.T @ q[0]) / max(np.linalg.norm(aq0), 1e-300)
    al, be = [], []
    for j in range(min(LK, n)):
        t2 = f32(A.T @ f32(A @ q[j]))
        aj = q[j] @ t2
        for p in range(j + 1):
            t2 = f32(t2 - (q[p] @ t2) * q[p])
        bj = np.linalg.norm(t2)
        al.append(aj)
        be.append(bj)
        if not (bj > 1e-6 * abs(aj)) or j + 1 >= LK:
            break
        q.append(f32(t2 / bj))
    emax = -_tridiag_min_eig([-v for v in al], be)
    emin = max(_tridiag_min_eig(al, be), emax * 1e-32)
    return np.array([
        np.log2(n) / 9.0, nrhs / 4.0, _lg(rs.max()), _lg(cs.max()), _lg(fro), _lg(amax),
        _lg(np.sqrt(max(emax, 0.0))), _lg(fro / np.sqrt(max(emax, 1e-300))), _lg(ratio.min()),
        np.mean(np.log10(np.maximum(ratio, 1e-30))), np.mean(ratio > 1.0),
        _lg(rs.max() / max(rs.min(), 1e-300)), _lg(cs.max() / max(cs.min(), 1e-300)),
        asym, _lg(di.min() / max(amax, 1e-300)),
        _lg(np.sqrt(max(emax, 1e-300) / emin)),
    ])
