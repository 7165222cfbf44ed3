"""Build recipe for libgbdbscan.so and its command-line tools (sm_103a only).

Every translation unit under csrc/ is compiled by nvcc in parallel with
  -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17
and linked in-tree:
  <package>/libgbdbscan.so      the C-ABI library (include/gbdbscan.h)
  <package>/gbdbscan_main       the command-line driver (links the library)
  <package>/gbdbscan_check      the label-quality report (links the library)
Objects go to <package>/_build/.  No cmake, no torch extension machinery.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgbdbscan.so")
CLI = os.path.join(PKG, "gbdbscan_main")
CHECK = os.path.join(PKG, "gbdbscan_check")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-I", INCLUDE, "-I", CSRC]
LIB_SOURCES = ["gd_prims.cu", "gd_pipeline.cu", "gd_api.cu", "gd_noalloc.cu", "gd_io.cpp",
               "gd_server.cpp", "gd_quality.cpp"]
CLI_SOURCES = ["gd_main.cpp", "gd_check_main.cpp"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _deps() -> list[str]:
    out = []
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    out.append(os.path.join(INCLUDE, "gbdbscan.h"))
    return out


def source_digest() -> str:
    """Digest of every source the library is built from (csrc/ and the public
    header): profiles record it with their numbers, so a number captured on
    other sources can be told apart from one of this build."""
    import hashlib
    h = hashlib.sha256()
    for path in sorted(_deps()):
        if os.path.isfile(path) and path.endswith((".cu", ".cuh", ".h", ".cpp")):
            h.update(os.path.basename(path).encode())
            with open(path, "rb") as f:
                h.update(f.read())
    return h.hexdigest()[:16]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *NVFLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    deps = _deps()
    if not force and not any(_stale(t, deps) for t in (LIB, CLI, CHECK)):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(LIB_SOURCES) + len(CLI_SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), LIB_SOURCES + CLI_SOURCES))
    lib_objs = objs[: len(LIB_SOURCES)]
    cli_objs = objs[len(LIB_SOURCES):]
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *lib_objs], check=True)
    os.replace(tmp, LIB)
    for exe, obj in zip((CLI, CHECK), cli_objs):
        tmp = exe + f".tmp{os.getpid()}"
        subprocess.run([nvcc(), *ARCH, "-o", tmp, obj, "-L", PKG, "-lgbdbscan",
                        "-Xlinker", "-rpath,$ORIGIN"], check=True)
        os.replace(tmp, exe)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
