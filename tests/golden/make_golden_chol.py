"""Writes the golden fixtures of the Cholesky path.

chol_kats.json  the reference crate's own known-answer tests for
                CholeskyDecomposition (src/decomp/cholesky.rs:147-182 in
                xasmx/rust-la 0.2.0), restated as data.
chol_small.npz  seeded small symmetric matrices with the oracle's outputs
                (L, or None, and the solution). The oracle restates
                src/decomp/cholesky.rs:56-145; these fixtures let the GPU tests
                compare against committed bits and let the CPU tests check
                that the oracle still produces them.

Run from the repository root: python tests/golden/make_golden_chol.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
import oracle  # noqa: E402

# kind: "chol_l_exact"   assert!(l * l.t() == a); assert!(l.data == expect)
#       "chol_none"      CholeskyDecomposition::new(&a).is_none()
#       "chol_solve_approx"  c.solve(&b).approx_eq(&x)
#       "chol_solve_panic"   #[should_panic] c.solve(&b)
KATS = [
    {"ref": "src/decomp/cholesky.rs:147-153", "kind": "chol_l_exact",
     "a": [[4.0, 12.0, -16.0], [12.0, 37.0, -43.0], [-16.0, -43.0, 98.0]],
     "expect": [2.0, 0.0, 0.0, 6.0, 1.0, 0.0, -8.0, 5.0, 3.0]},
    {"ref": "src/decomp/cholesky.rs:155-159", "kind": "chol_none",
     "a": [[4.0, 12.0, -16.0], [12.0, 37.0, 43.0], [-16.0, 43.0, 98.0]]},
    {"ref": "src/decomp/cholesky.rs:161-165", "kind": "chol_none",
     "a": [[4.0, 12.0, -16.0], [12.0, 37.0, 43.0]]},
    {"ref": "src/decomp/cholesky.rs:167-173", "kind": "chol_solve_approx",
     "a": [[2.0, 1.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
     "b": [[1.0], [2.0], [3.0]], "x": [[-1.0], [3.0], [3.0]]},
    {"ref": "src/decomp/cholesky.rs:175-182", "kind": "chol_solve_panic",
     "a": [[2.0, 1.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
     "b": [[1.0], [2.0], [3.0], [4.0]]},
]

# (name, n, seed, nrhs, kind): "spd" = (G + G')/2 + n I; "indef" = symmetric,
# one negative pivot; "asym" = spd with one off-diagonal entry moved by an ulp.
RANDOM_CASES = [
    ("n1", 1, 21, 1, "spd"), ("n2", 2, 22, 2, "spd"), ("n7", 7, 23, 1, "spd"),
    ("n33", 33, 24, 3, "spd"), ("n64", 64, 25, 1, "spd"), ("n65", 65, 26, 4, "spd"),
    ("n130", 130, 27, 5, "spd"), ("n200", 200, 28, 2, "spd"),
    ("indef40", 40, 29, 1, "indef"), ("asym50", 50, 30, 1, "asym"),
]


def make_matrix(n, seed, kind):
    rng = np.random.default_rng(seed)
    g = rng.uniform(-1.0, 1.0, size=(n, n))
    a = (g + g.T) / 2.0
    a += n * np.eye(n)
    if kind == "indef":
        a[n // 2, n // 2] = -1.0
    if kind == "asym":
        a[n - 1, 3] = np.nextafter(a[n - 1, 3], np.inf)
    return a


def main():
    with open(os.path.join(HERE, "chol_kats.json"), "w") as f:
        json.dump({"source": "xasmx/rust-la 0.2.0 #[test] functions", "kats": KATS}, f, indent=1)
    out = {}
    for name, n, seed, nrhs, kind in RANDOM_CASES:
        a = make_matrix(n, seed, kind)
        b = np.random.default_rng(seed + 1000).uniform(-1.0, 1.0, size=(n, nrhs))
        lo = oracle.chol_new(a)
        out[name + "_a"] = a
        out[name + "_b"] = b
        out[name + "_some"] = np.array([lo is not None])
        if lo is not None:
            out[name + "_l"] = lo
            out[name + "_x"] = oracle.chol_solve(lo, b)
    np.savez_compressed(os.path.join(HERE, "chol_small.npz"), **out)
    print("wrote chol_kats.json (%d) and chol_small.npz (%d cases)" % (len(KATS), len(RANDOM_CASES)))


if __name__ == "__main__":
    main()
