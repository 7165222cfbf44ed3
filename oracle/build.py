"""Build recipes for the checker side (TEST INFRASTRUCTURE ONLY).

  build_oracle()  compiles the CPU restatement (gd_oracle.cpp) into
                  oracle/_build/libgd_oracle.so with g++ -O2 -fopenmp and
                  -ffp-contract=off (aarch64 GCC would otherwise fuse a*b+c and
                  change the float64 bits the oracle must reproduce).
  build_ref()     compiles the reference's own R-tree DBSCAN from the reference
                  checkout (REF_ROOT, default /root/reference) into
                  oracle/_ref/libref_rtree.so through ref_rtree_harness.cpp.
                  Skipped (returns None) when the checkout is absent.
  build_ref_check() compiles the reference's cluster check
                  (test-results/cluster-check.cpp) into the executable
                  oracle/_ref/ref_cluster_check through ref_check_harness.cpp.
                  Skipped (returns None) when the checkout is absent.
  build_ref_multicore() compiles the reference's multicore CPU DBSCAN
                  (multicore-cpu/) into oracle/_ref/libref_multicore.so through
                  ref_multicore_harness.cpp, for timing only.  Skipped (returns
                  None) when the checkout is absent.

REF_ROOT is where the reference checkout lies on the machine that builds these
checkers (GD_REFERENCE_ROOT overrides it); this recipe reads the reference's
sources there and copies none of them.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libgd_oracle.so")
REF_RTREE_SO = os.path.join(REF_DIR, "libref_rtree.so")
REF_CHECK_EXE = os.path.join(REF_DIR, "ref_cluster_check")
REF_MULTICORE_SO = os.path.join(REF_DIR, "libref_multicore.so")
REF_ROOT = os.environ.get("GD_REFERENCE_ROOT", "/root/reference")

_COMMON = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off"]


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "gd_oracle.cpp")
    if not force and _newer(ORACLE_SO, [src]):
        return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    cmd = ["g++", *_COMMON, "-fopenmp", src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(force: bool = False) -> str | None:
    ref_src_dir = os.path.join(REF_ROOT, "cpu-dbscan")
    ref_src = os.path.join(ref_src_dir, "dbscan_rtree_exp.cpp")
    if not os.path.exists(ref_src):
        return None
    harness = os.path.join(HERE, "ref_rtree_harness.cpp")
    if not force and _newer(REF_RTREE_SO, [harness, ref_src]):
        return REF_RTREE_SO
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_RTREE_SO + f".tmp{os.getpid()}"
    cmd = ["g++", *_COMMON, "-w", "-I", ref_src_dir, harness, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_RTREE_SO)
    return REF_RTREE_SO


def build_ref_check(force: bool = False) -> str | None:
    src_dir = os.path.join(REF_ROOT, "test-results")
    src = os.path.join(src_dir, "cluster-check.cpp")
    if not os.path.exists(src):
        return None
    harness = os.path.join(HERE, "ref_check_harness.cpp")
    if not force and _newer(REF_CHECK_EXE, [harness, src]):
        return REF_CHECK_EXE
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_CHECK_EXE + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-w", "-I", src_dir, harness, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_CHECK_EXE)
    return REF_CHECK_EXE


def build_ref_multicore(force: bool = False) -> str | None:
    """The reference's multicore CPU DBSCAN (multicore-cpu/dbscan.cpp, report.c,
    read_dataset.c) into oracle/_ref/libref_multicore.so through
    ref_multicore_harness.cpp; None when the checkout is absent."""
    src_dir = os.path.join(REF_ROOT, "multicore-cpu")
    srcs = [os.path.join(src_dir, f) for f in ("dbscan.cpp", "report.c", "read_dataset.c")]
    if not all(os.path.exists(s) for s in srcs):
        return None
    harness = os.path.join(HERE, "ref_multicore_harness.cpp")
    if not force and _newer(REF_MULTICORE_SO, [harness, *srcs]):
        return REF_MULTICORE_SO
    os.makedirs(REF_DIR, exist_ok=True)
    tmp = REF_MULTICORE_SO + f".tmp{os.getpid()}"
    # the two .c files are C++ (they include <fstream>)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-w", "-I", src_dir,
           harness, "-x", "c++", srcs[1], srcs[2], "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_MULTICORE_SO)
    return REF_MULTICORE_SO


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
    print(build_ref_check(force="-f" in sys.argv))
    print(build_ref_multicore(force="-f" in sys.argv))
