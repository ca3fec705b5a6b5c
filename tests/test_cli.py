"""The command-line entry `bmagwa-gb300 INIFILE` (the reference's
`bmagwa INIFILE`, src/main.cpp:36-120) up to the first device call: usage,
option and data errors with the reference's messages, and options the GPU
path does not run, all reported before a CUDA call is made."""
import os
import re
import subprocess

import pytest

import helpers as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "bmagwa_gb300", "_build", "bmagwa-gb300")


def run(*args, cwd=None):
    return subprocess.run([CLI, *args], capture_output=True, text=True, cwd=cwd, timeout=120)


@pytest.fixture(scope="module", autouse=True)
def built(bmg):
    if not os.path.exists(CLI):
        pytest.fail("the CLI was not built")


def test_usage():
    r = run()
    assert r.returncode == 0
    assert "Usage:" in r.stdout and "INIFILE" in r.stdout


def test_option_error_is_the_reference_message(tmp_path):
    r = run(str(tmp_path / "absent.ini"))
    assert r.returncode == 1
    assert "Cannot load/parse configuration file." in r.stderr


def test_data_error_is_the_reference_message(tmp_path):
    z = H.golden("ref_small")
    ini = H.materialize(z, tmp_path)
    os.remove(tmp_path / "data.bed")
    r = run(ini)
    assert r.returncode == 1
    assert "BED file could not be opened" in r.stderr


def test_unsupported_option_stops_before_sampling(tmp_path):
    """A sampler type other than PMV (the reference's NK, KSC and G samplers
    are not on this path) stops the command before any trace file is
    written."""
    z = H.golden("ref_small")
    ini = H.materialize(z, tmp_path)
    txt = open(ini).read()
    txt = re.sub(r"(?m)^type\s*=.*$", "type = NK", txt) if re.search(r"(?m)^type\s*=", txt) else \
        txt.replace("[sampler]", "[sampler]\ntype = NK", 1)
    open(ini, "w").write(txt)
    r = run(ini)
    assert r.returncode == 1
    assert "PMV" in r.stderr, r.stderr
    assert not any(f.endswith(".dat") for f in os.listdir(tmp_path / "out"))


def test_default_value_warnings_are_printed(tmp_path):
    """The reference prints a warning for every optional key left out
    (src/options.hpp:326-345); the CLI parses with warnings on."""
    z = H.golden("ref_small")
    ini = H.materialize(z, tmp_path)
    os.remove(tmp_path / "data.bed")
    r = run(ini)
    assert "Warning: using default value of" in r.stdout + r.stderr
