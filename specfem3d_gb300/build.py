"""Build of the in-tree shared library libspecfem3d_gb300.so (sm_103a only).

Each translation unit under csrc/ is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked with
the shared CUDA runtime.  The library lands in specfem3d_gb300/_lib/.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libspecfem3d_gb300.so"
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build specfem3d_gb300")


def cuda_lib_dir(nv: str) -> str:
    root = os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(root, sub)
        if os.path.exists(os.path.join(p, "libcudart.so")):
            return p
    return os.path.join(root, "lib64")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    nv = nvcc()
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h"))) + [
        os.path.join(os.path.dirname(HERE), "include", "specfem3d_gb300.h")]
    flags = [GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
             "--expt-relaxed-constexpr"]

    def compile_one(src):
        obj = os.path.join(LIBDIR, "obj", os.path.basename(src).replace(".cu", ".o"))
        if force or _stale(obj, [src] + headers):
            cmd = [nv, *flags, "-c", src, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose and r.stderr:
                print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources))) as ex:
        objs = list(ex.map(compile_one, sources))
    out = lib_path()
    if force or _stale(out, objs):
        libdir = cuda_lib_dir(nv)
        cmd = [nv, "-shared", GENCODE, "-o", out + ".tmp", *objs, "-cudart", "shared", f"-L{libdir}",
               f"-Xlinker", f"-rpath,{libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(verbose=True))
