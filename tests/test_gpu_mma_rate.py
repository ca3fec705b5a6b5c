"""The tensor-core rate the scan's design rests on: a tcgen05.mma of M = 128,
K = 16 (bf16, FP32 accumulator in tensor memory), issued back to back into
one accumulator, has a per-instruction floor: N = 64 costs nearly what
N = 192 costs (94 against 106 SM cycles with A in tensor memory on a GB300,
138 at N = 256), so fewer columns per instruction (fewer residual limbs)
barely shorten a stage, and N = 192 runs at about 0.9 of the tensor pipe's
rate when nothing stalls the issue.  tests/mma_rate.cu is built with nvcc and
run on the GPU; it prints the cycles per instruction."""
import json
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_mma_issue_floor(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "mma_rate")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
                    "-I" + os.path.join(ROOT, "bmagwa_gb300", "csrc", "dev"), "-I" + os.path.join(ROOT, "include"),
                    os.path.join(HERE, "mma_rate.cu"), "-o", exe], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=120).stdout
    rows = [json.loads(line) for line in out.splitlines() if line.startswith("{")]
    print(out)
    assert len(rows) == 8 and all(r.get("ok") == 1 for r in rows)
    for a in (0, 1):
        c = {r["n"]: r["cycles_per_mma"] for r in rows if r["a_tmem"] == a}
        # a floor: a third of the columns costs well over half the time
        assert c[64] >= 0.6 * c[192], c
        # and more columns never cost less
        assert c[64] <= c[128] * 1.02 <= c[192] * 1.04 <= c[256] * 1.06, c
