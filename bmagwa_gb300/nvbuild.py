"""Build recipe of libbmg (the CUDA kernels + C ABI) and the CLI, in-tree.

Every translation unit is compiled for sm_103a only, in parallel, into
bmagwa_gb300/_build/; the outputs are git-ignored.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libbmg.so")
CLI = os.path.join(OUT, "bmagwa-gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(CSRC, "dev")]

CU = ["bmg_api.cu", "dev/sampler.cu", "dev/scan.cu", "dev/prep.cu", "dev/scan_tc.cu", "dev/schur_tc.cu",
      "dev/learned.cu", "dev/noalloc.cu"]
CPP = ["host/options.cpp", "host/plink.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _obj(src):
    return os.path.join(OUT, src.replace("/", "_") + ".o")


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = _obj(src)
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"] + INC + \
              ["-c", path, "-o", obj]
    else:
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC"] + INC + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = []
    for d in (os.path.join(ROOT, "include"), CSRC, os.path.join(CSRC, "dev")):
        hs += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh"))]
    return hs


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers()
    todo = [s for s in CU + CPP if force or _stale(_obj(s), [os.path.join(CSRC, s)] + hdrs)]
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(_compile, todo))
    objs = [_obj(s) for s in CU + CPP]
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.run(cmd, check=True, capture_output=not verbose)
    # the command-line entry; libbmg's own dependencies (the CUDA runtime) are
    # resolved when it runs, not when it links.  A failed link leaves the
    # library usable and is reported, not raised.
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB])):
        cmd = ["g++", "-std=c++17", "-O2"] + INC + [cli_src, "-o", CLI, "-L" + OUT, "-lbmg",
                                                    "-Wl,-rpath,$ORIGIN", "-Wl,--allow-shlib-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            print("warning: the bmagwa-gb300 command was not built:\n%s%s" % (r.stdout, r.stderr),
                  file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
