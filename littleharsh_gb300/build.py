"""Build the in-tree CUDA library littleharsh_gb300/_lib/liblh_gb300.so.

nvcc compiles each translation unit for sm_103a only (in parallel), then links
one shared library that exports the C ABI of include/littleharsh.h.
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
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "liblh_gb300.so")
SOURCES = ["lh_kernels.cu", "lh_capi.cu", "lh_host.cpp", "lh_noalloc.cu", "lh_io.cpp", "lh_srnet.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]
    objs, cmds = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + common
        if src.endswith(".cu"):
            cmd += ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]
        cmds.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for msg in ex.map(run, cmds):
            if verbose and msg:
                print(msg, file=sys.stderr)
    tmp = LIB + ".tmp"
    run([cc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"])
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


DRIVER_SRC = os.path.join(PKG, "driver", "lh_driver.c")


def build_driver(out: str | None = None) -> str:
    """Compile the C host driver (littleharsh_gb300/driver/lh_driver.c) against include/littleharsh.h and link
    it to the library; returns the executable's path (default: next to the library)."""
    lib = build()
    exe = out or os.path.join(OUT_DIR, "lh_driver")
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler found")
    cmd = [cc, "-O2", "-std=c99", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include"), DRIVER_SRC, "-o", exe,
           "-L" + OUT_DIR, "-llh_gb300", "-Wl,-rpath," + OUT_DIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 or not os.path.exists(lib):
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return exe


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
