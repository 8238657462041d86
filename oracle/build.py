"""Build recipe for the oracle (test infrastructure, not product code).

* ``oracle/build/libclue_oracle.so``: the CPU restatement in clue_oracle.c.
* ``oracle/_ref/libclue_ref.so``: ref_harness.cc compiled against the
  UNMODIFIED reference sources.  They are read from the reference tree
  (``CLUE_REFERENCE_DIR``, else the ``reference`` directory beside this
  repository) where it exists, else from the reference install in
  ``baseline/_ref/src/serial``.
* ``baseline/_ref/src/serial``: the reference install -- a verbatim copy of
  the few reference source files the harness includes (``REF_FILES``),
  refreshed from the reference tree whenever it is present.  It is
  git-ignored (never part of the product) and travels with the working copy
  to machines without the reference tree, where the harness is then built
  from it, so that the timed CPU baseline is the reference itself.

Both libraries use ``-O2 -ffp-contract=off`` (no FMA contraction) and no
``-march``.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
REFERENCE_DIR = os.environ.get("CLUE_REFERENCE_DIR", os.path.join(os.path.dirname(REPO), "reference"))
INSTALL_DIR = os.path.join(REPO, "baseline", "_ref", "src", "serial")
# the reference files the harness compiles (paths under src/serial)
REF_FILES = (
    "plugin-CLUEClusterizer/CLUEAlgoSerial.cc", "plugin-CLUEClusterizer/CLUEAlgoSerial.h",
    "plugin-CLUEClusterizer/CLUEAlgoKernels.h",
    "plugin-CLUETracksterizer/CLUE3DAlgoSerial.cc", "plugin-CLUETracksterizer/CLUE3DAlgoSerial.h",
    "plugin-CLUETracksterizer/CLUE3DAlgoKernels.h",
    "DataFormats/PointsCloud.h", "DataFormats/LayerTilesSerial.h", "DataFormats/LayerTilesConstants.h",
    "DataFormats/ClusterCollection.h", "DataFormats/TICLLayerTile.h", "DataFormats/Common.h",
    "DataFormats/Math/deltaR.h", "DataFormats/Math/deltaPhi.h", "DataFormats/Math/normalizedPhi.h",
    "DataFormats/Math/angle_units.h",
)

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


def _tree_serial():
    serial = os.path.join(REFERENCE_DIR, "src", "serial")
    return serial if os.path.isdir(os.path.join(serial, "plugin-CLUEClusterizer")) else None


def install_reference():
    """Refreshes baseline/_ref/src/serial from the reference tree (when it
    is present).  Returns the install directory, or None when neither the
    tree nor an earlier install exists."""
    tree = _tree_serial()
    if tree is not None:
        for rel in REF_FILES:
            src, dst = os.path.join(tree, rel), os.path.join(INSTALL_DIR, rel)
            if not os.path.exists(dst) or os.path.getmtime(src) > os.path.getmtime(dst):
                os.makedirs(os.path.dirname(dst), exist_ok=True)
                shutil.copy2(src, dst)
    ok = all(os.path.exists(os.path.join(INSTALL_DIR, rel)) for rel in REF_FILES)
    return INSTALL_DIR if ok else None


def reference_sources():
    """Where the harness reads the reference: the tree, else the install."""
    return _tree_serial() or install_reference()


def ref_cmd():
    serial = reference_sources()
    if serial is None:
        return None
    src = os.path.join(HERE, "ref_harness.cc")
    cmd = ["g++", "-std=c++17", *FLAGS, "-w", f"-I{serial}", src, "-o", REF_SO, "-lpthread"]
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
    install_reference()
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
