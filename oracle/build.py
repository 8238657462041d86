"""Build recipe for the oracle (test infrastructure, not product code).

* ``oracle/build/libclue_oracle.so``: the CPU restatement in clue_oracle.c.
* ``oracle/_ref/libclue_ref.so``: ref_harness.cc compiled against the
  UNMODIFIED reference sources, only where the reference tree exists
  (``CLUE_REFERENCE_DIR``, default ``/root/reference``).  Nothing from the
  reference is copied; its files are included from where they lie.

Both use ``-O2 -ffp-contract=off`` (no FMA contraction) and no ``-march``.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE_DIR = os.environ.get("CLUE_REFERENCE_DIR", "/root/reference")

ORACLE_SO = os.path.join(HERE, "build", "libclue_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libclue_ref.so")

FLAGS = ["-O2", "-ffp-contract=off", "-fPIC", "-shared"]


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def oracle_cmd():
    src = os.path.join(HERE, "clue_oracle.c")
    return ["gcc", "-std=gnu11", *FLAGS, src, "-o", ORACLE_SO, "-lm", "-lpthread"], ORACLE_SO, [src]


def ref_cmd():
    serial = os.path.join(REFERENCE_DIR, "src", "serial")
    if not os.path.isdir(os.path.join(serial, "plugin-CLUEClusterizer")):
        return None
    src = os.path.join(HERE, "ref_harness.cc")
    cmd = ["g++", "-std=c++17", *FLAGS, "-w", f"-I{serial}", src, "-o", REF_SO]
    deps = [src,
            os.path.join(serial, "plugin-CLUEClusterizer", "CLUEAlgoKernels.h"),
            os.path.join(serial, "plugin-CLUETracksterizer", "CLUE3DAlgoKernels.h")]
    return cmd, REF_SO, deps


def commands():
    out = [oracle_cmd()]
    r = ref_cmd()
    if r is not None:
        out.append(r)
    return out


def build(verbose=False):
    procs = []
    for cmd, out, deps in commands():
        if not _stale(out, deps):
            continue
        os.makedirs(os.path.dirname(out), exist_ok=True)
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stderr=subprocess.PIPE, text=True)))
    for cmd, p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{err}")


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
