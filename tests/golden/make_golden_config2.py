"""Fixture of the benchmark workload's reference LU (n = 8192, seed 2, 16 RHS).

The oracle (the CPU restatement of src/decomp/lu.rs:104-278) takes minutes at
n = 8192, so its answer is stored here as SHA-256 digests of its exact bytes:
the input matrix (so that a test can tell its own inputs are the same), the
packed LU, the pivot vector (uint64, lu.rs:99), the solution of the 16
right-hand sides, and the pivot sign. tests/test_bench_configs_gpu.py compares
the GPU's results with these digests and recomputes the oracle only when the
input digest differs (another random generator).

Usage: python tests/golden/make_golden_config2.py [threads]
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

import oracle  # noqa: E402

N, NRHS, SEED = 8192, 16, 2
OUT = os.path.join(HERE, "config2_n8192.json")


def digest(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def inputs():
    rng = np.random.default_rng(SEED)
    a = rng.standard_normal((N, N))
    b = rng.standard_normal((N, NRHS))
    return a, b


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 4)
    oracle.build()
    a, b = inputs()
    t0 = time.time()
    ref = oracle.lu_factor(a, threads=threads)
    x = oracle.solve_mt(ref, b, threads)
    rec = {
        "n": N, "nrhs": NRHS, "seed": SEED,
        "generator": "numpy.random.default_rng(seed).standard_normal: A (n x n), then B (n x nrhs)",
        "sha256_a": digest(a),
        "sha256_b": digest(b),
        "sha256_lu": digest(ref.lu),
        "sha256_piv": digest(ref.piv.astype(np.uint64)),
        "sha256_x": digest(x),
        "pospivsign": int(ref.pospivsign),
        "piv_head": [int(v) for v in ref.piv[:16]],
        "backward_error": oracle.backward_error(a, x, b),
    }
    with open(OUT, "w") as f:
        json.dump(rec, f, indent=1)
    print("wrote %s in %.0f s" % (OUT, time.time() - t0))


if __name__ == "__main__":
    main()
