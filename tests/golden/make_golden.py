"""Writes the golden fixtures of the LU path.

kats.json      the reference crate's own known-answer tests for the LU path,
               restated as data (inputs and expected outcome, with the test's
               file:line in xasmx/rust-la 0.2.0).
random_small.npz  seeded small matrices with the oracle's outputs (packed LU,
               pivot vector, sign, det, solution). The oracle is a restatement
               of src/decomp/lu.rs; these fixtures let the GPU tests compare
               against committed bits and let the CPU tests check that the
               oracle still produces them on every host.

Run from the repository root: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
import oracle  # noqa: E402

# kind: "lu_reconstruct_exact"  assert!(l * u == p * a)
#       "solve_approx"          assert!(lu.solve(&b).unwrap().approx_eq(&x))
#       "solve_exact"           assert!(a.solve(&b).unwrap().eq(&x))
#       "solve_panic"           #[should_panic] lu.solve(&b)
#       "solve_none"            lu.solve(&b).is_none()
#       "is_singular"           lu.is_singular() == expect
#       "is_non_singular"       lu.is_non_singular() == expect
#       "lu_det_exact"          lu.det() == expect
#       "lu_det_panic"          #[should_panic] lu.det()
#       "matrix_det_le"         (a.det() - expect) <= f32::EPSILON
#       "matrix_det_panic"      #[should_panic] a.det()
#       "inverse_approx"        a.inverse().unwrap().approx_eq(&expect)
#       "inverse_panic"         #[should_panic] a.inverse()
#       "inverse_none"          a.inverse() == None
#       "matrix_is_singular"    a.is_singular() == expect
#       "matrix_is_singular_panic"
#       "matrix_is_non_singular"
#       "mul_exact"             (&a).mul(&b).data == expect
#       "mul_panic"
#       "mmul_exact"            a.mmul(&b, &mut dst); dst.data == expect
#       "mmul_panic"            (dst_shape given)
KATS = [
    {"ref": "src/decomp/lu.rs:281-289", "kind": "lu_reconstruct_exact",
     "a": [[1.0, 2.0, 0.0], [3.0, 6.0, -1.0], [1.0, 2.0, 1.0]]},
    {"ref": "src/decomp/lu.rs:291-299", "kind": "lu_reconstruct_exact",
     "a": [[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]]},
    {"ref": "src/decomp/lu.rs:301-309", "kind": "lu_reconstruct_exact",
     "a": [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]},
    {"ref": "src/decomp/lu.rs:311-317", "kind": "solve_approx",
     "a": [[2.0, 1.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
     "b": [[1.0], [2.0], [3.0]], "x": [[-1.0], [3.0], [3.0]]},
    {"ref": "src/decomp/lu.rs:319-326", "kind": "solve_panic",
     "a": [[2.0, 1.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
     "b": [[1.0], [2.0], [3.0], [4.0]]},
    {"ref": "src/decomp/lu.rs:328-334", "kind": "solve_none",
     "a": [[2.0, 6.0], [1.0, 3.0]], "b": [[1.0], [2.0]]},
    {"ref": "src/decomp/lu.rs:336-345", "kind": "is_singular",
     "a": [[2.0, 6.0], [1.0, 3.0]], "expect": True},
    {"ref": "src/decomp/lu.rs:336-345", "kind": "is_singular",
     "a": [[2.0, 6.0], [1.0, 4.0]], "expect": False},
    {"ref": "src/decomp/lu.rs:347-356", "kind": "is_non_singular",
     "a": [[4.0, 8.0], [3.0, 4.0]], "expect": True},
    {"ref": "src/decomp/lu.rs:347-356", "kind": "is_non_singular",
     "a": [[4.0, 6.0], [2.0, 3.0]], "expect": False},
    {"ref": "src/decomp/lu.rs:358-367", "kind": "lu_det_exact",
     "a": [[4.0, 8.0], [3.0, 4.0]], "expect": -8.0},
    {"ref": "src/decomp/lu.rs:358-367", "kind": "lu_det_exact",
     "a": [[4.0, 8.0], [2.0, 4.0]], "expect": 0.0},
    {"ref": "src/decomp/lu.rs:369-375", "kind": "lu_det_panic",
     "a": [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]},
    {"ref": "src/matrix/mod.rs:1506-1510", "kind": "matrix_det_le",
     "a": [[6.0, -7.0, 10.0], [0.0, 3.0, -1.0], [0.0, 5.0, -7.0]], "expect": -96.0},
    {"ref": "src/matrix/mod.rs:1512-1516", "kind": "matrix_det_panic",
     "a": [[6.0, -7.0, 10.0], [0.0, 3.0, -1.0]]},
    {"ref": "src/matrix/mod.rs:1518-1523", "kind": "solve_exact",
     "a": [[1.0, 1.0, 1.0], [1.0, -1.0, 4.0], [2.0, 3.0, -5.0]],
     "b": [[3.0], [4.0], [0.0]], "x": [[1.0], [1.0], [1.0]]},
    {"ref": "src/matrix/mod.rs:1527-1533", "kind": "inverse_approx",
     "a": [[6.0, -7.0, 10.0], [0.0, 3.0, -1.0], [0.0, 5.0, -7.0]],
     "expect": [[v / 96.0 for v in row] for row in
                [[16.0, -1.0, 23.0], [0.0, 42.0, -6.0], [0.0, 30.0, -18.0]]]},
    {"ref": "src/matrix/mod.rs:1535-1540", "kind": "inverse_panic",
     "a": [[6.0, -7.0, 10.0], [0.0, 3.0, -1.0]]},
    {"ref": "src/matrix/mod.rs:1542-1546", "kind": "inverse_none",
     "a": [[2.0, 6.0], [1.0, 3.0]]},
    {"ref": "src/matrix/mod.rs:1554-1558", "kind": "matrix_is_singular",
     "a": [[2.0, 6.0], [1.0, 3.0]], "expect": True},
    {"ref": "src/matrix/mod.rs:1560-1565", "kind": "matrix_is_singular_panic",
     "a": [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]},
    {"ref": "src/matrix/mod.rs:1567-1571", "kind": "matrix_is_non_singular",
     "a": [[2.0, 6.0], [6.0, 3.0]], "expect": True},
    {"ref": "src/matrix/mod.rs:1479-1484", "kind": "mul_exact",
     "a": [[1.0, 2.0], [3.0, 4.0]], "b": [[3.0, 4.0], [5.0, 6.0]],
     "expect": [[13.0, 16.0], [29.0, 36.0]]},
    {"ref": "src/matrix/mod.rs:1486-1492", "kind": "mul_panic",
     "a": [[1.0, 2.0], [3.0, 4.0]], "b": [[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]]},
    {"ref": "src/matrix/mmatrix.rs:234-241", "kind": "mmul_exact",
     "a": [[1.0, 2.0], [3.0, 4.0]], "b": [[3.0, 4.0], [5.0, 6.0]], "dst_shape": [2, 2],
     "expect": [[13.0, 16.0], [29.0, 36.0]]},
    {"ref": "src/matrix/mmatrix.rs:243-250", "kind": "mmul_panic",
     "a": [[1.0, 2.0], [3.0, 4.0]], "b": [[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]],
     "dst_shape": [2, 2]},
    {"ref": "src/matrix/mmatrix.rs:252-259", "kind": "mmul_panic",
     "a": [[1.0, 2.0], [3.0, 4.0]], "b": [[1.0, 2.0], [3.0, 4.0]], "dst_shape": [3, 3]},
]

# (name, rows, cols, seed, nrhs)
RANDOM_CASES = [
    ("sq5", 5, 5, 11, 1), ("sq16", 16, 16, 12, 3), ("sq37", 37, 37, 13, 2),
    ("sq64", 64, 64, 14, 1), ("sq65", 65, 65, 15, 4), ("sq130", 130, 130, 16, 5),
    ("tall40x25", 40, 25, 17, 1), ("wide25x40", 25, 40, 18, 1),
]


def main():
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump({"source": "xasmx/rust-la 0.2.0 #[test] functions", "kats": KATS}, f, indent=1)
    out = {}
    for name, r, c, seed, nrhs in RANDOM_CASES:
        rng = np.random.default_rng(seed)
        a = rng.uniform(-1.0, 1.0, size=(r, c))
        b = rng.uniform(-1.0, 1.0, size=(r, nrhs))
        f = oracle.lu_factor(a)
        out[name + "_a"] = a
        out[name + "_b"] = b
        out[name + "_lu"] = f.lu
        out[name + "_piv"] = f.piv
        out[name + "_sign"] = np.array([int(f.pospivsign)])
        if r == c:
            out[name + "_det"] = np.array([oracle.det(f)])
            out[name + "_x"] = oracle.solve(f, b)
    np.savez_compressed(os.path.join(HERE, "random_small.npz"), **out)
    print("wrote kats.json (%d) and random_small.npz (%d cases)" % (len(KATS), len(RANDOM_CASES)))


if __name__ == "__main__":
    main()
