"""In-tree build of the asdpocs_gb300 shared library (sm_103a only).

``python -m asd_pocs_mex_cuda_demo_gb300.build`` compiles every translation
unit of ``csrc/`` with nvcc in parallel and links
``asd_pocs_mex_cuda_demo_gb300/lib/libasdpocs_gb300.so``.  The projector
unit is compiled with ``-fmad=false`` so that its float operations round one
by one, in the order of the reference expressions.  ``build(checked=True)``
(``--checked``) links the bounds-checked variant
``lib/libasdpocs_gb300_checked.so`` from the same sources with
``-DASDPOCS_CHECKED`` (every projector and TV index checked before its
access; see asdpocs_checked_errors).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libasdpocs_gb300.so")
OBJ_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(LIBDIR, "libasdpocs_gb300_checked.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code (gateway geometry, per-view constants) must round every float
# operation as written on both x86 and Arm hosts: no contraction into FMA
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I", INCLUDE, "--expt-relaxed-constexpr"]
# per-unit extra flags
UNITS = {
    "kernels_proj.cu": ["-fmad=false"],
    "kernels_tv.cu": [],
    "host_api.cu": [],
    "noalloc.cu": [],
    "server.cu": [],
    "phantom.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit: str, extra: list[str], verbose_ptxas: bool, objdir: str = OBJ) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(objdir, unit.replace(".cu", ".o"))
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
    if verbose_ptxas:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale(lib: str = LIB) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if os.path.getmtime(os.path.join(d, f)) > t:
                return True
    return False


def build(force: bool = False, verbose_ptxas: bool = False, checked: bool = False) -> str:
    """Compile the library (or its bounds-checked variant) if any source is
    newer than it; return its path."""
    lib, objdir = (LIB_CHECKED, OBJ_CHECKED) if checked else (LIB, OBJ)
    if not force and not _stale(lib):
        return lib
    os.makedirs(objdir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    flag = ["-DASDPOCS_CHECKED"] if checked else []
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = {u: ex.submit(_compile, u, f + flag, verbose_ptxas, objdir)
                for u, f in UNITS.items()}
        logs = {u: f.result() for u, f in futs.items()}
    objs = [os.path.join(objdir, u.replace(".cu", ".o")) for u in UNITS]
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose_ptxas:
        for u, log in logs.items():
            sys.stderr.write(f"== {u}\n{log}")
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv,
                checked="--checked" in sys.argv))
