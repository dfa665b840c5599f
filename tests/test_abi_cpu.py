"""The C-ABI library on the CPU: it builds, loads without a GPU, exports every
symbol include/mantaray_gpu.h declares, and its host-only functions (step
count, NetCDF-3 reader) behave like the reference's.  No kernel runs here."""

import ctypes
import math
import os
import re

import numpy as np
import pytest

from tests import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fname in os.listdir(inc):
        if fname.endswith(".h"):
            text = open(os.path.join(inc, fname)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names.update(re.findall(r"\b(mr_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_symbols()
    for required in ("mr_trace", "mr_trace_device", "mr_single_ray", "mr_ray_tracing_files",
                     "mr_single_ray_files", "mr_bathymetry_grid", "mr_current_grid",
                     "mr_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(native):
    for name in declared_symbols():
        assert hasattr(native, name), name


def test_python_binding_lists_every_symbol():
    from mantaray_gb300 import _native

    assert set(_native.SYMBOLS) == set(declared_symbols())


@pytest.mark.parametrize("t0,t_end,dt", [(0.0, 10.0, 2.0), (0.0, 10.0, 3.0), (1.0, 10.0, 1.0),
                                         (0.0, -1.0, 1.0), (0.0, 1.0, 0.0), (0.0, math.nan, 1.0),
                                         (0.0, 6.8, 0.1), (100.0, 102.0, 1.0), (0.0, 1e6, 20.0),
                                         (0.0, 1000.0, 0.5), (0.0, math.inf, 1.0)])
def test_num_steps_matches_oracle(native, oracle, t0, t_end, dt):
    assert native.mr_num_steps(t0, t_end, dt) == oracle.num_steps(t0, t_end, dt)


def test_version(native):
    assert native.mr_version() >= 100


def _read(path, name):
    from mantaray_gb300 import read_netcdf3_variable

    return read_netcdf3_variable(path, name)


@pytest.mark.parametrize("dtype", [np.int8, np.int16, np.int32, np.float32, np.float64, "S1"])
@pytest.mark.parametrize("version", [1, 2])
def test_netcdf3_types(tmp_path, dtype, version):
    # The reference accepts i8/u8/i16/i32/f32/f64 variables
    # (cartesian_netcdf3.rs:170-253, cartesian_current.rs:67-205); u8 is the
    # NetCDF char type.
    rng = np.random.default_rng(1)
    if dtype == "S1":
        data = rng.integers(0, 255, size=(4, 5)).astype(np.uint8)
        stored = data.view("S1")
    elif np.issubdtype(np.dtype(dtype), np.integer):
        info = np.iinfo(dtype)
        data = rng.integers(info.min, info.max, size=(4, 5)).astype(dtype)
        stored = data
    else:
        data = rng.normal(size=(4, 5)).astype(dtype)
        stored = data
    p = tmp_path / "t.nc"
    H.write_nc(p, {"a": (("y", "x"), stored), "x": (("x",), np.arange(5.0))},
               {"y": 4, "x": 5}, version=version)
    got = _read(p, "a")
    np.testing.assert_array_equal(got, data.astype(np.float64).ravel())
    np.testing.assert_array_equal(_read(p, "x"), np.arange(5.0))


def test_netcdf3_record_variables(tmp_path):
    from scipy.io import netcdf_file

    p = tmp_path / "rec.nc"
    with netcdf_file(str(p), "w") as f:
        f.createDimension("t", None)
        f.createDimension("x", 3)
        a = f.createVariable("a", "f8", ("t", "x"))
        b = f.createVariable("b", "i2", ("t",))
        for r in range(4):
            a[r] = np.arange(3.0) + 10 * r
            b[r] = r
        c = f.createVariable("c", "f4", ("x",))
        c[:] = [1.5, 2.5, 3.5]
    np.testing.assert_array_equal(_read(p, "a"), (np.arange(3.0)[None] + 10 * np.arange(4)[:, None]).ravel())
    np.testing.assert_array_equal(_read(p, "b"), np.arange(4.0))
    np.testing.assert_array_equal(_read(p, "c"), [1.5, 2.5, 3.5])


def test_netcdf3_with_attributes(tmp_path):
    from scipy.io import netcdf_file

    p = tmp_path / "att.nc"
    with netcdf_file(str(p), "w") as f:
        f.title = "test"
        f.history = "made by a test"
        f.createDimension("x", 2)
        v = f.createVariable("depth", "f8", ("x",))
        v.units = "m"
        v.scale = np.array([1.0, 2.0, 3.0])
        v[:] = [7.0, 8.0]
    np.testing.assert_array_equal(_read(p, "depth"), [7.0, 8.0])


def test_netcdf3_errors(tmp_path):
    from mantaray_gb300 import MantarayError, MantarayIOError
    from mantaray_gb300._native import ERR_IO, ERR_READ

    with pytest.raises(MantarayIOError) as ei:
        _read(tmp_path / "missing.nc", "x")
    assert ei.value.code == ERR_IO
    bad = tmp_path / "bad.nc"
    bad.write_bytes(b"HDF\x89 not netcdf")
    with pytest.raises(MantarayError) as ei:
        _read(bad, "x")
    assert ei.value.code == ERR_READ
    good = tmp_path / "good.nc"
    H.write_nc(good, {"x": (("x",), np.arange(1000.0))}, {"x": 1000})
    with pytest.raises(MantarayError) as ei:
        _read(good, "nope")
    assert ei.value.code == ERR_READ and "nope" in str(ei.value)
    trunc = tmp_path / "trunc.nc"
    trunc.write_bytes(good.read_bytes()[:-100])
    with pytest.raises(MantarayError) as ei:
        _read(trunc, "x")
    assert ei.value.code == ERR_READ


def test_bathymetry_fixture_matches_reference_writer(tmp_path):
    # The writer restates src/io/utility.rs:29-90: f32 axes, f64 depth [y][x].
    p = tmp_path / "b.nc"
    x, y, depth = H.write_bathymetry_nc(p, 101, 51, 500.0, 500.0, lambda a, b: float(a) + 2 * float(b))
    np.testing.assert_array_equal(_read(p, "x"), x.astype(np.float64))
    np.testing.assert_array_equal(_read(p, "depth"), depth.ravel())
    assert abs(x[10] - 5000.0) < np.finfo(np.float32).eps  # cartesian_netcdf3.rs:513


def test_error_message_is_thread_local_and_set(native):
    from mantaray_gb300 import MantarayError, read_netcdf3_variable

    with pytest.raises(MantarayError):
        read_netcdf3_variable("/nonexistent/file.nc", "x")
    assert b"nonexistent" in native.mr_last_error()
    _ = ctypes


def test_batch_config_layout_matches_the_header(native, tmp_path):
    # The ctypes mirror of mr_batch_config has the header's size and field
    # offsets (a C program compiled against include/mantaray_gpu.h prints
    # them), and the library's default config fills it as documented.
    import shutil
    import subprocess

    from mantaray_gb300 import _native

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = [f for f, _ in _native.BatchConfig._fields_]
    src = tmp_path / "layout.c"
    src.write_text(
        "#include <stddef.h>\n#include <stdio.h>\n#include \"mantaray_gpu.h\"\n"
        "int main(void) {\n"
        "  printf(\"%zu\\n\", sizeof(mr_batch_config));\n"
        + "".join(f"  printf(\"%zu\\n\", offsetof(mr_batch_config, {f}));\n" for f in fields)
        + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert out[0] == ctypes.sizeof(_native.BatchConfig)
    assert out[1:] == [getattr(_native.BatchConfig, f).offset for f in fields]
    cfg = _native.BatchConfig()
    assert native.mr_batch_default_config(ctypes.byref(cfg)) == 0
    assert (cfg.block, cfg.blocks_per_sm, cfg.rays_per_lane, cfg.rebase_interval, cfg.order,
            cfg.staging, cfg.sweep_steps) == (128, 4, 1, 32, 0, 0, 0)
