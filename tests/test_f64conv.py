"""The integer-instruction FP64 <-> FP32 conversions used by the batched
mixed-precision kernel (rust-la_gb300/csrc/f64conv.h) equal the compiler's
IEEE round-to-nearest-even conversions bit for bit (host build of the same
header, no GPU needed)."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "rust-la_gb300", "csrc")


def test_f64conv_matches_compiler_conversions(tmp_path):
    exe = str(tmp_path / "f64conv_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "f64conv_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
