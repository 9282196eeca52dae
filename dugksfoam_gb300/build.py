"""Build recipe for libdugks.so (CUDA sm_103a kernels + C++ host + C ABI).

Compiles every translation unit in parallel with one ``-gencode`` for
sm_103a and links a shared library into ``dugksfoam_gb300/_build/``.
No cmake; nvcc + g++ only, so the same recipe runs on x86_64 and aarch64.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libdugks.so")
# the checked build: the same sources with device-side index checks
# (-DDUGKS_CHECKED=1); its CUDA objects live apart, the host objects are shared
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(BUILD_CHECKED, "libdugks_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# FP64 translation units are built without FMA contraction so the plain FP64
# path performs the same roundings as the CPU oracle, operation by operation.
EXTRA = {
    "ref_pipeline.cu": ["-fmad=false"],
    "common_kernels.cu": ["-fmad=false"],
    "fused_fp64.cu": ["-fmad=false"],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    cu = sorted(glob.glob(os.path.join(PKG, "csrc", "cuda", "*.cu")))
    cpp = sorted(glob.glob(os.path.join(PKG, "csrc", "host", "*.cpp")))
    return cu, cpp


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> str:
    """Compile (incrementally) and link libdugks.so, or with ``checked`` the
    index-checked libdugks_checked.so; returns its path."""
    if checked:
        build(verbose, force)  # the shared host objects
    out_dir = BUILD_CHECKED if checked else BUILD
    lib_path = LIB_CHECKED if checked else LIB
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    cuda_home = os.path.dirname(os.path.dirname(nvcc))
    inc = ["-I", os.path.join(ROOT, "include")]
    headers = (glob.glob(os.path.join(PKG, "csrc", "*", "*.h")) + glob.glob(os.path.join(PKG, "csrc", "*", "*.cuh"))
               + glob.glob(os.path.join(ROOT, "include", "dugks", "*.h")))
    cu, cpp = sources()
    jobs, objs = [], []
    for src in cu:
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                   *EXTRA.get(os.path.basename(src), []), *(["-DDUGKS_CHECKED=1"] if checked else []), *inc, "-c", src,
                   "-o", obj]
            jobs.append(cmd)
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if checked:
            continue  # built by the plain build above
        if force or _stale(obj, [src] + headers):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", *inc,
                   "-I", os.path.join(cuda_home, "include"), "-c", src, "-o", obj]
            jobs.append(cmd)
    procs = [(cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for cmd in jobs]
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out)
        if p.returncode != 0:
            failed.append((cmd, out))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("libdugks build failed:\n" + msg)
    if force or jobs or _stale(lib_path, objs):
        tmp = lib_path + ".tmp"
        subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"],
                       check=True)
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, checked="--checked" in sys.argv))
