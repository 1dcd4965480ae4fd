"""Builds the engine library librtdbs.so for sm_103a with nvcc (no cmake).

    python -m rtdbstream_gb300.build

Sources: csrc/rtdbs_kernels.cu (device code), csrc/rtdbs_engine.cpp (the C
ABI of include/rtdbs.h: engines and pools), csrc/rtdbs_noalloc.cu and
csrc/rtdbs_io.cpp; the translation units compile in parallel.  Also builds
rtdbs_dbscan, the reference-compatible command line (csrc/rtdbs_cli.cpp).
Results land in rtdbstream_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "librtdbs.so")
CLI = os.path.join(OUT_DIR, "rtdbs_dbscan")  # the reference-compatible command line
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")
    return exe


def sources() -> list[str]:
    return [os.path.join(CSRC, "rtdbs_kernels.cu"), os.path.join(CSRC, "rtdbs_engine.cpp"),
            os.path.join(CSRC, "rtdbs_noalloc.cu"), os.path.join(CSRC, "rtdbs_io.cpp")]


def headers() -> list[str]:
    return [os.path.join(CSRC, "rtdbs_internal.h"), os.path.join(ROOT, "include", "rtdbs.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    srcs = sources() + headers() + [__file__, os.path.join(CSRC, "rtdbs_cli.cpp")]
    return os.path.exists(CLI) and all(os.path.getmtime(f) <= t for f in srcs)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    common = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    objs, procs = [], []
    for src in sources():
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
        cmd = common + ["-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd = common + ["-x", "cu", "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{out.decode()}")
    tmp = LIB + ".tmp"
    link = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    if verbose:
        print(" ".join(link))
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    os.replace(tmp, LIB)
    cli = [nvcc(), *ARCH, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
           os.path.join(CSRC, "rtdbs_cli.cpp"), "-o", CLI + ".tmp", "-L", OUT_DIR, "-lrtdbs",
           "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cli, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
