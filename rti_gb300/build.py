"""Builds librtg.so (the CUDA flux engine) in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel to an object under
rti_gb300/_build/, then nvcc links the shared library rti_gb300/librtg.so.
-fmad=false keeps every float operation a separately rounded IEEE operation
(fused multiply-adds only where the source writes fmaf), which is what makes
GPU paths bit-identical to the CPU restatement of the reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librtg.so")
LIB_CHECKED = os.path.join(HERE, "librtg_checked.so")  # -DRTG_CHECKED: device bounds checks (tests)
SOURCES = ["rtg_api.cu", "rtg_batch.cu", "rtg_lbvh.cu", "rtg_noalloc.cu", "rtg_sort.cu", "rtg_surface.cu", "rtg_trace.cu",
           "rtg_trace_batched.cu", "rtg_vtk.cpp", "rtg_wavefront.cu", "rtg_wide.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def zlib_flags() -> tuple[list[str], list[str]]:
    """(-D flag, link flag) when zlib's header and linkable library are present
    (compressed VTK input); empty lists otherwise."""
    inc = any(os.path.exists(os.path.join(d, "zlib.h")) for d in ("/usr/include", "/usr/local/include"))
    lib = None
    for d in ("/usr/lib/x86_64-linux-gnu", "/usr/lib/aarch64-linux-gnu", "/usr/lib64", "/usr/lib", "/lib64"):
        for name in ("libz.so", "libz.so.1"):
            if os.path.exists(os.path.join(d, name)):
                lib = os.path.join(d, name)
                break
        if lib:
            break
    if inc and lib:
        return ["-DRTG_WITH_ZLIB"], [lib]
    return [], []


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "cli", "rtg_cli.cpp"))
    files.append(os.path.join(ROOT, "include", "rtg.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None, checked: bool = False) -> str:
    """librtg.so; checked=True: librtg_checked.so, the same with -DRTG_CHECKED
    (every index read from device data verified before use, a bad one counted
    in the trace's errors), for tests."""
    lib = LIB_CHECKED if checked else LIB
    if not force and up_to_date(lib):
        return lib
    bdir = BUILD + ("_checked" if checked else "")
    os.makedirs(bdir, exist_ok=True)
    exe = nvcc()
    extra = list(extra or [])
    zdef, zlink = zlib_flags()
    extra += zdef
    if checked:
        extra.append("-DRTG_CHECKED")

    def compile_one(src: str) -> str:
        obj = os.path.join(bdir, os.path.splitext(src)[0] + ".o")
        cmd = [exe, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = lib + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, *zlink, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if not checked:
        build_cli()
    return lib


def build_cli() -> str:
    """The command-line driver (cli/rtg_cli.cpp) against librtg.so."""
    gxx = shutil.which("g++") or "g++"
    out = os.path.join(HERE, "rtg")
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = [gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "cli", "rtg_cli.cpp"),
           "-L", HERE, "-lrtg", "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath-link,{cuda_lib}", "-o", out + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for the CLI:\n{r.stderr}")
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(force=True, verbose=v, extra=["-Xptxas", "-v"] if v else None))
