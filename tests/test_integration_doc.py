"""The C example of INTEGRATION.md compiles against include/bmg.h and links
against libbmg (not run: it needs a GPU and an INI file)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_example_compiles_and_links(bmg, tmp_path):
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"## C\n\n```c\n(.*?)```", text, re.S)
    assert m, "no C example in INTEGRATION.md"
    body = [line for line in m.group(1).splitlines() if not line.startswith("#include")]
    src = tmp_path / "example.c"
    src.write_text("#include <stdint.h>\n#include <stdlib.h>\n#include \"bmg.h\"\nint main(void)\n{\n" +
                   "\n".join(body) + "\n  return 0;\n}\n")
    lib_dir = os.path.join(ROOT, "bmagwa_gb300", "_build")
    assert os.path.exists(os.path.join(lib_dir, "libbmg.so"))
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src), "-o",
                        str(tmp_path / "example"), "-L" + lib_dir, "-lbmg", "-Wl,--allow-shlib-undefined"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
