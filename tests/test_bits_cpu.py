"""The integer-pipe float / double conversions of mantaray_gb300/csrc/bits.h,
compiled for the host, against the compiler's IEEE conversions on edge cases
and ~12 M pseudo-random bit patterns (exact halfway cases included)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_bits_conversions_are_exact(tmp_path):
    exe = str(tmp_path / "bits_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "bits_check.cpp")], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    bad, n = (int(v) for v in out.stdout.split()[-2:])
    assert out.returncode == 0 and bad == 0, out.stdout
    assert n > 10_000_000
