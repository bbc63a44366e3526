"""Writes the golden fixtures of the QR path.

qr_kats.json   the reference crate's own known-answer tests for
               QRDecomposition (src/decomp/qr.rs:241-260 in xasmx/rust-la
               0.2.0), restated as data: Q * R approx_eq A.
qr_small.npz   seeded small matrices with the oracle's outputs (qr, rdiag, Q,
               R, the square solves and pinverse). The oracle restates
               src/decomp/qr.rs:26-238 and src/matrix/mod.rs:1049-1057.

Run from the repository root: python tests/golden/make_golden_qr.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
import oracle  # noqa: E402

KATS = [
    {"ref": "src/decomp/qr.rs:241-246", "kind": "qr_reconstruct_approx",
     "a": [[12.0, -51.0, 4.0], [6.0, 167.0, -68.0], [-4.0, 24.0, -41.0]]},
    {"ref": "src/decomp/qr.rs:248-253", "kind": "qr_reconstruct_approx",
     "a": [[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]]},
    {"ref": "src/decomp/qr.rs:255-260", "kind": "qr_reconstruct_approx",
     "a": [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]},
]

# (name, m, n, seed, nrhs)
RANDOM_CASES = [("sq1", 1, 1, 41, 1), ("sq7", 7, 7, 42, 2), ("sq64", 64, 64, 43, 3),
                ("sq65", 65, 65, 44, 1), ("tall50x20", 50, 20, 45, 1),
                ("wide20x50", 20, 50, 46, 1), ("sq130", 130, 130, 47, 4)]


def main():
    with open(os.path.join(HERE, "qr_kats.json"), "w") as f:
        json.dump({"source": "xasmx/rust-la 0.2.0 #[test] functions", "kats": KATS}, f, indent=1)
    out = {}
    for name, m, n, seed, nrhs in RANDOM_CASES:
        rng = np.random.default_rng(seed)
        a = rng.uniform(-1.0, 1.0, size=(m, n))
        b = rng.uniform(-1.0, 1.0, size=(m, nrhs))
        f = oracle.qr_new(a)
        out[name + "_a"] = a
        out[name + "_b"] = b
        out[name + "_qr"] = f.qr
        out[name + "_rdiag"] = f.rdiag
        out[name + "_q"] = oracle.qr_get_q(f)
        out[name + "_r"] = oracle.qr_get_r(f)
        if m == n:
            out[name + "_x"] = oracle.qr_solve(f, b)
        if m >= n:
            out[name + "_pinv"] = oracle.pinverse(a)
    np.savez_compressed(os.path.join(HERE, "qr_small.npz"), **out)
    print("wrote qr_kats.json (%d) and qr_small.npz (%d cases)" % (len(KATS), len(RANDOM_CASES)))


if __name__ == "__main__":
    main()
