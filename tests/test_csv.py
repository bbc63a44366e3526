"""util::read_csv (src/util.rs:9-35, f64 parser) in the native library against
its oracle restatement (oracle/csv_ref.py): the same matrix bit for bit where
the reference returns one, a Panic wherever the reference panics. CPU only (no
context, no GPU)."""
import math
import os

import numpy as np
import pytest

from oracle import ReferencePanic, csv_ref

VALID = {
    "plain": b"1,2,3\n4,5,6\n",
    "no_final_newline": b"1,2\n3,4",
    "crlf": b"1,2\r\n3,4\r\n",
    "spaces_tabs": b" 1 ,\t2\t\n  3,4  \n",
    "unicode_space": " 1,　2 \n3 , 4\u0085\n".encode(),
    "signs_exponents": b"+1,-2,3e2,-4E-2,.5,6.,+.7e+1\n",
    "special": b"inf,-Infinity,NaN,+nan,INF,infinity\n",
    "zeros": b"0,-0,0.0,-0.0e5,0e-999\n",
    "rounding": (b"0.1000000000000000055511151231257827,1.0000000000000002220446049250313,"
                 b"2.4703282292062328e-324,2.4703282292062327e-324,4.9e-324\n"),
    "range": b"1.7976931348623157e308,1.7976931348623159e308,1e309,-1e400,1e-400\n",
    "long_digits": (b"3." + b"1" * 400 + b",0." + b"0" * 300 + b"1e300\n"),
    "single": b"42\n",
    "one_column": b"1\n2\n3\n",
}

INVALID = {
    "empty_file": b"",
    "empty_line": b"\n",
    "empty_line_inside": b"1,2\n\n3,4\n",
    "ragged": b"1,2\n3\n",
    "empty_item": b"1,,2\n",
    "word": b"abc\n",
    "exp_no_digits": b"1e\n",
    "exp_sign_only": b"1e+\n",
    "hex": b"0x10\n",
    "underscore": b"1_000\n",
    "blank_item": b" \n",
    "double_sign": b"+-1\n",
    "two_dots": b"1.2.3\n",
    "lone_dot": b".\n",
    "nan_payload": b"nan(1)\n",
    "infinity_suffix": b"infinity1\n",
    "bom": "﻿1,2\n".encode(),
    "bad_utf8": b"1,\xff\n",
    "overlong_utf8": b"1,\xc0\xb1\n",
    "arabic_digit": "١\n".encode(),
}


def _write(tmp_path, name, content):
    p = tmp_path / (name + ".csv")
    p.write_bytes(content)
    return str(p)


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", sorted(VALID))
def test_valid_files_match_the_oracle(lagpu, tmp_path, name):
    path = _write(tmp_path, name, VALID[name])
    rows, cols, data = csv_ref.read_csv(path)
    m = lagpu.read_csv(path)
    assert m.data.shape == (rows, cols)
    want = np.array(data, dtype=np.float64)
    got = m.data.ravel()
    nan = np.isnan(want)
    assert np.array_equal(nan, np.isnan(got))
    assert np.array_equal(_bits(got[~nan]), _bits(want[~nan]))
    # the sign of NaN follows the literal's sign
    assert np.array_equal(np.signbit(got[nan]), np.signbit(want[nan]))


@pytest.mark.parametrize("name", sorted(INVALID))
def test_invalid_files_panic_like_the_reference(lagpu, tmp_path, name):
    path = _write(tmp_path, name, INVALID[name])
    with pytest.raises(ReferencePanic):
        csv_ref.read_csv(path)
    with pytest.raises(lagpu.Panic):
        lagpu.read_csv(path)


def test_missing_file_panics(lagpu, tmp_path):
    path = str(tmp_path / "absent.csv")
    with pytest.raises(ReferencePanic):
        csv_ref.read_csv(path)
    with pytest.raises(lagpu.Panic):
        lagpu.read_csv(path)


def test_known_values():
    assert csv_ref.parse_f64("2.4703282292062328e-324") == 5e-324  # above half of the least subnormal
    assert csv_ref.parse_f64("2.4703282292062327e-324") == 0.0     # below it
    assert csv_ref.parse_f64("1.7976931348623159e308") == math.inf
    assert csv_ref.parse_f64("-0") == 0.0 and math.copysign(1.0, csv_ref.parse_f64("-0")) < 0


def test_large_random_file_bitwise(lagpu, tmp_path):
    """Many lines (every host thread gets a share), values printed with random
    precision, spacing and exponent style."""
    rng = np.random.default_rng(12)
    rows, cols = 3000, 40
    vals = rng.standard_normal((rows, cols)) * 10.0 ** rng.integers(-30, 30, size=(rows, cols))
    fmts = ["%r", "%.17g", "%.6e", "%.3f", "%.20E"]
    lines = []
    for r in range(rows):
        items = []
        for c in range(cols):
            f = fmts[(r * 7 + c) % len(fmts)]
            s = (f % vals[r, c]) if f != "%r" else repr(float(vals[r, c]))
            pad = " " * int(rng.integers(0, 3))
            items.append(pad + s + pad)
        lines.append(",".join(items))
    path = _write(tmp_path, "large", ("\r\n".join(lines) + "\n").encode())
    nr, nc, data = csv_ref.read_csv(path)
    m = lagpu.read_csv(path)
    assert (nr, nc) == (rows, cols) == m.data.shape
    assert np.array_equal(_bits(m.data.ravel()), _bits(np.array(data)))
