"""Host checks of the scan kernels' arithmetic: the double-float posterior (df64.h, rb_df.h)
compiled for the host and checked against long double: every building block
to its published bound (a few 2^-48) and the posterior p_r to 1e-12 relative,
far inside the 1e-9 the parity tests require."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_double_float_arithmetic_against_long_double(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "df64_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "df64_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    err = {k: float(v) for k, v in (line.split() for line in out.split("\n") if line.strip())}
    bound = 2.0 ** -44
    for k in ("add", "mul", "div", "rsqrt", "exp"):
        assert err[k] < bound, (k, err[k], out)
    assert err["ll"] < 2.0 ** -47, out
    assert err["pr"] < 1e-12, out


def test_register_decode_of_packed_codes(tmp_path):
    """The scan's table-free decode of 2-bit codes into bf16 codings agrees
    with the codings for all 256 code bytes and every term."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "decode_check")
    subprocess.run([cxx, "-O2", "-std=c++17", os.path.join(HERE, "decode_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout
