"""Build recipe of libclue_gb300.so (CUDA for sm_103a + C++ host runtime).

Every .cu file is compiled by nvcc for ``sm_103a`` only, with ``--fmad=false``
(the CLUE arithmetic must not be contracted into FMAs) and ``-lineinfo``;
every .cc file by g++.  Objects go to ``_objs/`` and the shared library to
``lib/``, both in-tree and git-ignored.  Translation units compile in
parallel; a unit is rebuilt when it or any header in csrc/ or include/ is
newer than its object.
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJS = os.path.join(HERE, "_objs")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libclue_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return os.path.getmtime(src) > t or any(os.path.getmtime(d) > t for d in deps)


def compile_commands(extra_nvcc=()):
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    cmds = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJS, os.path.basename(src) + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
               *inc, *extra_nvcc, "-c", src, "-o", obj]
        cmds.append((src, obj, cmd))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cc"))):
        obj = os.path.join(OBJS, os.path.basename(src) + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function",
               "-I" + os.path.join(cuda, "include"), *inc, "-c", src, "-o", obj]
        cmds.append((src, obj, cmd))
    return nvcc, cmds


def build(verbose=False, jobs=None, extra_nvcc=()):
    os.makedirs(OBJS, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc, cmds = compile_commands(extra_nvcc)
    deps = _headers()
    todo = [(s, o, c) for s, o, c in cmds if _stale(o, s, deps) or extra_nvcc]

    def run(item):
        src, obj, cmd = item
        if verbose:
            print(" ".join(cmd), flush=True)
        p = subprocess.run(cmd, capture_output=True, text=True)
        return src, p

    failed = []
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for src, p in ex.map(run, todo):
            if verbose and (p.stdout or p.stderr):
                print(p.stdout + p.stderr, flush=True)
            if p.returncode != 0:
                failed.append((src, p.stdout + p.stderr))
    if failed:
        msg = "\n".join(f"--- {s}\n{e}" for s, e in failed)
        raise RuntimeError(f"libclue_gb300 build failed:\n{msg}")
    objs = [o for _, o, _ in cmds]
    if todo or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        link = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB, "-lpthread"]
        if verbose:
            print(" ".join(link), flush=True)
        p = subprocess.run(link, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stdout}{p.stderr}")
    return LIB


if __name__ == "__main__":
    extra = sys.argv[1:]
    build(verbose=True, extra_nvcc=extra)
