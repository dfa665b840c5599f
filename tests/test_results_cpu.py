"""The JSON and TSV trajectory writers (CPU): the reference's own expected
strings (src/ray_result.rs:153-206) and Rust's float formatting rules."""

import math

import numpy as np

from mantaray_gb300 import results as R


def test_as_json_reference_vectors():
    # src/ray_result.rs:170-181
    rr = {"t_vec": [1.0], "x_vec": [2.0], "y_vec": [3.0], "kx_vec": [4.0], "ky_vec": [5.0]}
    assert R.as_json(rr) == ('{"t_vec":[1.0],"x_vec":[2.0],"y_vec":[3.0],"kx_vec":[4.0],'
                             '"ky_vec":[5.0]}')
    # src/ray_result.rs:157-168: an empty result
    assert R.as_json(R.ray_result(np.zeros((0, 5)))) == (
        '{"t_vec":[],"x_vec":[],"y_vec":[],"kx_vec":[],"ky_vec":[]}')


def test_nan_cut():
    # src/ray_result.rs:183-206: cut at the first row with any NaN
    rows = np.array([[0.0, 1.0, 1.0, 1.0, 1.0], [1.0, 1.0, math.nan, math.nan, 1.0],
                     [2.0, math.nan, math.nan, math.nan, math.nan], [3.0, 2.0, 2.0, 2.0, 2.0]])
    assert R.as_json(R.ray_result(rows)) == (
        '{"t_vec":[0.0],"x_vec":[1.0],"y_vec":[1.0],"kx_vec":[1.0],"ky_vec":[1.0]}')


def test_float_layouts():
    cases = {0.1: ("0.1", "0.1"), 1.0: ("1.0", "1"), 1e-7: ("1e-7", "0.0000001"),
             1.5e-10: ("1.5e-10", "0.00000000015"), 1e21: ("1e21", "1000000000000000000000"),
             123456.0: ("123456.0", "123456"), 0.00001: ("0.00001", "0.00001"),
             -2.5: ("-2.5", "-2.5"), 1.565247584249853: ("1.565247584249853", "1.565247584249853"),
             1e16: ("1e16", "10000000000000000"), 1234567890123456.0: ("1234567890123456.0", "1234567890123456")}
    for v, (js, disp) in cases.items():
        assert R.json_float(v) == js, (v, R.json_float(v))
        assert R.display_float(v) == disp, (v, R.display_float(v))
    assert R.display_float(math.nan) == "NaN"


def test_tsv_writer(tmp_path):
    # src/ray.rs:219-243: header, rows until x is NaN, two trailing spaces, END
    rows = np.array([[0.0, 1.5, 2.0, 0.1, 0.0], [1.0, 3.0, 2.0, 0.1, 0.0],
                     [2.0, math.nan, math.nan, math.nan, math.nan]])
    p = tmp_path / "out.tsv"
    R.append_tsv(p, rows)
    R.append_tsv(p, rows[:1])
    assert p.read_text() == ("t x y kx ky\n0 1.5 2 0.1 0  \n1 3 2 0.1 0  \nEND\n"
                             "t x y kx ky\n0 1.5 2 0.1 0  \nEND\n")


def test_trace_result_methods(tmp_path):
    # a [5][rows][n] trajectory buffer with a ray that stopped after 2 rows
    from mantaray_gb300.core import TraceResult

    traj = np.full((5, 3, 2), np.nan)
    traj[:, :, 0] = [[0, 1, 2], [0.5, 1.0, 1.5], [0, 0, 0], [1, 1, 1], [0, 0, 0]]
    traj[:, :2, 1] = [[0, 1], [3.0, 4.0], [1, 1], [0.25, 0.25], [0, 0]]
    res = TraceResult(traj, np.array([3, 2]), np.zeros(2, np.uint8))
    assert res.as_json(1) == ('{"t_vec":[0.0,1.0],"x_vec":[3.0,4.0],"y_vec":[1.0,1.0],'
                              '"kx_vec":[0.25,0.25],"ky_vec":[0.0,0.0]}')
    p = tmp_path / "rays.tsv"
    res.append_tsv(p, 1)
    assert p.read_text() == "t x y kx ky\n0 3 1 0.25 0  \n1 4 1 0.25 0  \nEND\n"

