"""Writes the golden fixtures of the SVD::direct path.

svd_kats.json  the reference crate's own known-answer tests of
               EigenDecomposition (src/decomp/eigen.rs:841-856) and
               SVD::direct (src/decomp/svd.rs:532-559) in xasmx/rust-la 0.2.0,
               restated as data: the eigenvalues approx_eq the listed values,
               U * S * V' approx_eq A.
svd_small.npz  seeded small matrices with the oracle's outputs (eigenvalues
               and eigenvectors of A'A, U, S, V of SVD::direct). The oracle
               restates src/decomp/svd.rs:454-497 and eigen.rs:33-247, 755-790.

Run from the repository root: python tests/golden/make_golden_svd.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))
import oracle  # noqa: E402

A3 = [[3.0, 1.0, 6.0], [2.0, 1.0, 0.0], [-1.0, 0.0, -3.0]]
KATS = [
    {"ref": "src/decomp/eigen.rs:841-848", "kind": "eig_sym_of_ata_approx", "a": A3,
     "eigenvalues": [56.661209, 4.301868, 0.036923]},
    {"ref": "src/decomp/svd.rs:532-539", "kind": "svd_direct_reconstruct_approx",
     "a": [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 9.0]]},
    {"ref": "src/decomp/svd.rs:541-548", "kind": "svd_direct_reconstruct_approx",
     "a": [[1.0, 2.0, 3.0], [4.0, 5.0, 6.0], [7.0, 8.0, 9.0], [10.0, 11.0, 12.0]]},
    {"ref": "src/decomp/svd.rs:550-557", "kind": "svd_direct_reconstruct_approx",
     "a": [[1.0, 2.0, 3.0, 4.0], [5.0, 6.0, 7.0, 8.0], [9.0, 10.0, 11.0, 12.0]]},
]

# (name, m, n, seed)
RANDOM_CASES = [("sq1", 1, 1, 51), ("sq5", 5, 5, 52), ("sq40", 40, 40, 53),
                ("tall30x12", 30, 12, 54), ("wide12x30", 12, 30, 55), ("sq97", 97, 97, 56)]


def main():
    with open(os.path.join(HERE, "svd_kats.json"), "w") as f:
        json.dump({"source": "xasmx/rust-la 0.2.0 #[test] functions", "kats": KATS}, f, indent=1)
    out = {}
    for name, m, n, seed in RANDOM_CASES:
        a = np.random.default_rng(seed).uniform(-1.0, 1.0, size=(m, n))
        d, e, v = oracle.eig_sym(oracle.matmul(np.ascontiguousarray(a.T), a))
        u, s, vs = oracle.svd_direct(a)
        out[name + "_a"] = a
        out[name + "_d"] = d
        out[name + "_v"] = v
        out[name + "_u"] = u
        out[name + "_s"] = s
        out[name + "_vs"] = vs
    np.savez_compressed(os.path.join(HERE, "svd_small.npz"), **out)
    print("wrote svd_kats.json (%d) and svd_small.npz (%d cases)" % (len(KATS), len(RANDOM_CASES)))


if __name__ == "__main__":
    main()
