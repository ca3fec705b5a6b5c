"""The C example (bmagwa_gb300/csrc/example.c, quoted in INTEGRATION.md)
compiles against include/bmg.h and links against libbmg (not run: it needs
a GPU and an INI file)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXAMPLE = os.path.join(ROOT, "bmagwa_gb300", "csrc", "example.c")


def test_integration_notes_quote_the_example():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"## C\n\n.*?```c\n(.*?)```", text, re.S)
    assert m, "no C example in INTEGRATION.md"
    assert m.group(1) == open(EXAMPLE).read()


def test_c_example_compiles_and_links(bmg, tmp_path):
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    lib_dir = os.path.join(ROOT, "bmagwa_gb300", "_build")
    assert os.path.exists(os.path.join(lib_dir, "libbmg.so"))
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), EXAMPLE, "-o",
                        str(tmp_path / "example"), "-L" + lib_dir, "-lbmg", "-Wl,--allow-shlib-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
