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


def test_random_stream(tmp_path):
    """The stream every chain draws from (include/bmg_rng.h), compiled as C
    for the host: Philox4x32-10 reproduces the published known-answer
    vectors of Salmon et al. (SC'11), and the uniform, normal and gamma
    variates have their moments over 4M / 1M draws (six standard errors)."""
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "rng_check")
    subprocess.run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-I" + os.path.join(os.path.dirname(HERE), "include"),
                    os.path.join(HERE, "rng_check.c"), "-o", exe, "-lm"], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    v = dict(line.split() for line in out.splitlines() if line.strip())
    assert v["kat_zero"] == "6627e8d5e169c58dbc57ac4c9b00dbd8"
    assert v["kat_ones"] == "408f276d41c83b0ea20bc7c66d5451fd"
    assert v["kat_pi"] == "d16cfe0994fdcceb5001e42024126ea1"
    f = {k: float(x) for k, x in v.items() if not k.startswith("kat")}
    n = 4e6
    assert abs(f["uniform_mean"] - 0.5) < 6 * (1 / 12) ** 0.5 / n ** 0.5
    assert abs(f["uniform_var"] - 1 / 12) < 6 * (1 / 180) ** 0.5 / n ** 0.5
    assert 0 <= f["uniform_min"] < 1e-5 and 1 - 1e-5 < f["uniform_max"] < 1
    assert abs(f["normal_m1"]) < 6 / n ** 0.5
    assert abs(f["normal_m2"] - 1) < 6 * 2 ** 0.5 / n ** 0.5
    assert abs(f["normal_m3"]) < 6 * 15 ** 0.5 / n ** 0.5
    assert abs(f["normal_m4"] - 3) < 6 * 96 ** 0.5 / n ** 0.5
    m = n / 4
    for a in (0.3, 0.5, 1.0, 2.5, 10.0, 100.0):
        mean, var = f["gamma_mean_%g" % a], f["gamma_var_%g" % a]
        assert abs(mean - a) < 6 * a ** 0.5 / m ** 0.5, a
        # variance of the sample variance of a gamma: (mu4 - var^2) / m, mu4 = 3a^2 + 6a
        assert abs(var - a) < 6 * ((3 * a * a + 6 * a - a * a) / m) ** 0.5, a
    assert f["gamma_nan"] == 0
    assert f["slot_addressable"] == 1


def test_table_driven_log_of_the_move_kernel(tmp_path):
    """flog (bmagwa_gb300/csrc/dev/flog.h), the move kernel's logarithm:
    within 1.5 ulp of the long-double log over the double range, in [0.5, 2],
    near 1 and at the table's break points; special values as log()."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "flog_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "flog_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    err = {k: float(v) for k, v in (line.split() for line in out.split("\n") if line.strip())}
    for k in ("random", "near1", "unit", "breaks"):
        assert err[k] <= 1.5, (k, out)
    assert err["special"] == 1, out
