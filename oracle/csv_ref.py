"""ORACLE — test infrastructure only.

A pure-Python restatement of util::read_csv (xasmx/rust-la 0.2.0,
src/util.rs:9-35) with the f64 parser `|s| s.parse::<f64>().unwrap()`:
BufRead::lines (split at b'\\n', a b'\\r' before it dropped, no empty line after
a final b'\\n', strict UTF-8), str::split(","), str::trim (Unicode White_Space)
and the grammar of Rust's f64::from_str (std 1.55 and later; Python's float()
gives the same correctly rounded value once the syntax is checked). Raises
ReferencePanic wherever the reference panics.
"""
import math
import re

from . import ReferencePanic

# Unicode White_Space (the set str::trim removes)
WHITE_SPACE = "".join(chr(c) for c in list(range(0x09, 0x0E)) + [0x20, 0x85, 0xA0, 0x1680] +
                      list(range(0x2000, 0x200B)) + [0x2028, 0x2029, 0x202F, 0x205F, 0x3000])
_NUMBER = re.compile(r"[+-]?([0-9]+|[0-9]+\.[0-9]*|[0-9]*\.[0-9]+)(e[+-]?[0-9]+)?")


def parse_f64(item):
    """f64::from_str; ReferencePanic where it returns Err (then unwrap panics)."""
    low = item.lower()
    body = low[1:] if low[:1] in "+-" else low
    neg = low[:1] == "-"
    if body in ("inf", "infinity"):
        return -math.inf if neg else math.inf
    if body == "nan":
        return math.copysign(math.nan, -1.0 if neg else 1.0)
    if not item.isascii() or _NUMBER.fullmatch(low) is None:
        raise ReferencePanic("called `Result::unwrap()` on an `Err` value: ParseFloatError")
    return float(low)


def read_csv(path):
    """(rows, cols, data as a flat list) exactly as util::read_csv builds them."""
    try:
        with open(path, "rb") as f:
            raw = f.read()
    except OSError as e:
        raise ReferencePanic("File::open failed: %s" % e)
    try:
        text = raw.decode("utf-8", errors="strict")
    except UnicodeDecodeError as e:
        raise ReferencePanic("stream did not contain valid UTF-8: %s" % e)
    lines = text.split("\n")
    if lines and lines[-1] == "":
        lines.pop()  # no line after a final '\n' (and none at all for an empty file)
    data = []
    col_count = None
    for line in lines:
        if line.endswith("\r"):
            line = line[:-1]
        before = len(data)
        for item in line.split(","):
            data.append(parse_f64(item.strip(WHITE_SPACE)))
        count = len(data) - before
        if col_count is None:
            col_count = count
        elif col_count != count:
            raise ReferencePanic("assertion failed: col_count.unwrap() == line_col_count")
    if col_count is None:
        raise ReferencePanic("assertion failed: col_count != None")
    return len(lines), col_count, data
