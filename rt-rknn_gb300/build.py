"""Build the engine's shared library (librknn_gb300.so) and CLI in-tree.

    python rt-rknn_gb300/build.py [--force]

nvcc for sm_103a only; one translation unit per kernel family, compiled in
parallel.  zone.cu is compiled with -fmad=false so that its double-precision
arithmetic is rounded operation by operation, as the reference's (x86-64
g++ -O2, no FMA contraction) is.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librknn_gb300.so")
CLI = os.path.join(HERE, "rknn-gb300")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# RKNN_CHECKED=1: bounds-checked zone state (records the first bad index)
CHECKED = os.environ.get("RKNN_CHECKED", "0") == "1"
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")

UNITS = {
    "index.cu": [],
    "zone.cu": ["-fmad=false"],
    "zone_cta.cu": ["-fmad=false"],
    "verify.cu": [],
    "slice.cu": [],
    "api.cu": [],
}


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in sorted(paths):
        h.update(p.encode())
        with open(p, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(ARCH).encode())
    h.update(b"checked" if CHECKED else b"plain")
    return h.hexdigest()


def sources():
    out = []
    for d in (CSRC, HOST, os.path.join(REPO, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".c", ".cpp", ".hpp")):
                out.append(os.path.join(d, f))
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "stamp")
    dig = _digest(sources() + [os.path.abspath(__file__)]) + (" checked" if CHECKED else " plain")
    if (not force and os.path.exists(LIB) and os.path.exists(CLI) and os.path.exists(stamp)
            and open(stamp).read() == dig):
        return LIB
    common = [NVCC, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fno-strict-aliasing", f"-I{os.path.join(REPO, 'include')}"]
    if CHECKED:
        common.append("-DRKNN_CHECKED")

    def cc(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT, unit + ".o")
        cmd = common + UNITS[unit] + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(cc, UNITS))
    tmp = LIB + ".tmp"
    r = subprocess.run([NVCC, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    # command-line drop-in for the reference binaries
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{os.path.join(REPO, 'include')}",
                        os.path.join(HOST, "rknn_main.cpp"), "-o", CLI + ".tmp",
                        f"-L{HERE}", "-lrknn_gb300", "-Wl,-rpath,$ORIGIN", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    _build_pycall()
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


def _build_pycall():
    """The CPython fast path for rknn_query_batch (host/pycall.c), where the
    interpreter's headers are installed; rknn.py falls back to ctypes."""
    import sysconfig
    inc = sysconfig.get_paths().get("include") or ""
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    dst = os.path.join(HERE, "_rknn_call" + suffix)
    if not os.path.exists(os.path.join(inc, "Python.h")):
        if os.path.exists(dst):
            os.remove(dst)
        return
    r = subprocess.run(["gcc", "-O2", "-shared", "-fPIC", f"-I{inc}", f"-I{os.path.join(REPO, 'include')}",
                        os.path.join(HOST, "pycall.c"), "-o", dst + ".tmp", f"-L{HERE}", "-lrknn_gb300",
                        "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"pycall build failed:\n{r.stderr}")
    os.replace(dst + ".tmp", dst)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
