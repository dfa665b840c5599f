"""Trajectory serialisation: the reference's JSON and TSV writers.

`ray_result` / `as_json` restate RayResult (src/ray_result.rs:21-150): the
trajectory is cut at the first row with any NaN among x, y, kx, ky
(:134-141) and written as serde_json writes it
(`{"t_vec":[...],"x_vec":[...],"y_vec":[...],"kx_vec":[...],"ky_vec":[...]}`).
`append_tsv` restates output_or_append_to_tsv_file (src/ray.rs:219-243):
a "t x y kx ky" header, one line per row until the first row whose x is NaN,
each value followed by a space and the line by one more, then "END".

Floats are formatted as the two Rust formatters do: serde_json uses the
shortest round-trip digits laid out by ryu's rules (scientific outside
1e-5 <= |x| < 1e16, a ".0" on integral values); Rust's `{}` (the TSV) uses the
shortest round-trip digits in plain decimal notation, integral values without
a fraction.
"""

from __future__ import annotations

import math
import os

import numpy as np

_FIELDS = ("t_vec", "x_vec", "y_vec", "kx_vec", "ky_vec")


def _digits(v: float):
    """(sign, digit string, exponent) with v = sign * int(digits) * 10**exp,
    digits the shortest that round-trip (Python's repr finds the same digits
    as Rust's formatters)."""
    r = repr(abs(v))
    mant, _, exp = r.partition("e")
    e = int(exp) if exp else 0
    if "." in mant:
        a, b = mant.split(".")
        if b == "0":
            b = ""
    else:
        a, b = mant, ""
    digits = (a + b).lstrip("0") or "0"
    e -= len(b)
    # drop trailing zeros into the exponent
    stripped = digits.rstrip("0")
    if stripped:
        e += len(digits) - len(stripped)
        digits = stripped
    return ("-" if math.copysign(1.0, v) < 0 else ""), digits, e


def json_float(v: float) -> str:
    """A float as serde_json prints it (ryu layout)."""
    if not math.isfinite(v):
        return "null"  # serde_json writes non-finite floats as null
    if v == 0.0:
        return "-0.0" if math.copysign(1.0, v) < 0 else "0.0"
    sign, d, e = _digits(v)
    n = len(d)
    kk = n + e  # position of the decimal point relative to the first digit
    if 0 <= e and kk <= 16:
        return f"{sign}{d}{'0' * e}.0"
    if 0 < kk <= 16:
        return f"{sign}{d[:kk]}.{d[kk:]}"
    if -5 < kk <= 0:
        return f"{sign}0.{'0' * (-kk)}{d}"
    exp = kk - 1
    if n == 1:
        return f"{sign}{d}e{exp}"
    return f"{sign}{d[0]}.{d[1:]}e{exp}"


def display_float(v: float) -> str:
    """A float as Rust's `{}` prints it (plain decimal, shortest digits)."""
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    if v == 0.0:
        return "-0" if math.copysign(1.0, v) < 0 else "0"
    sign, d, e = _digits(v)
    if e >= 0:
        return f"{sign}{d}{'0' * e}"
    n = len(d)
    if n + e > 0:
        return f"{sign}{d[:n + e]}.{d[n + e:]}"
    return f"{sign}0.{'0' * (-(n + e))}{d}"


def ray_result(rows) -> dict:
    """RayResult of one ray: rows (m, 5) of (t, x, y, kx, ky), cut before the
    first row with a NaN among x, y, kx, ky."""
    rows = np.asarray(rows, dtype=np.float64).reshape(-1, 5)
    bad = np.isnan(rows[:, 1:]).any(axis=1)
    m = int(np.argmax(bad)) if bad.any() else rows.shape[0]
    return {f: [float(v) for v in rows[:m, q]] for q, f in enumerate(_FIELDS)}


def as_json(result: dict) -> str:
    """RayResult::as_json."""
    return "{" + ",".join(f'"{f}":[' + ",".join(json_float(v) for v in result[f]) + "]"
                          for f in _FIELDS) + "}"


def save_json(result: dict, path) -> int:
    """RayResult::save_file; returns the bytes written."""
    data = as_json(result).encode()
    with open(path, "wb") as fh:
        fh.write(data)
    return len(data)


def append_tsv(path, rows) -> None:
    """output_or_append_to_tsv_file for one ray (rows (m, 5))."""
    rows = np.asarray(rows, dtype=np.float64).reshape(-1, 5)
    out = ["t x y kx ky\n"]
    for r in rows:
        if math.isnan(r[1]):
            break
        out.append("".join(display_float(float(v)) + " " for v in r) + " \n")
    out.append("END\n")
    mode = "a" if os.path.exists(path) else "w"
    with open(path, mode) as fh:
        fh.write("".join(out))


def rays_from_trace(traj, n_rows):
    """Per-ray (rows, 5) arrays from a [5][rows][n] trajectory buffer."""
    traj = np.asarray(traj)
    return [np.ascontiguousarray(traj[:, : int(n_rows[i]), i].T) for i in range(traj.shape[2])]
