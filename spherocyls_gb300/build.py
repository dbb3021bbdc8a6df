"""Build libspherocyl (sm_103a kernels + C++ host runtime + C ABI) in-tree.

Produces ``spherocyls_gb300/lib/libspherocyl.so`` and the command-line drivers
under ``spherocyls_gb300/bin/``.  Translation units compile in parallel; the FP64
units are built with ``-fmad=false`` so that no fused multiply-add changes the
rounding of the reference-order arithmetic.
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
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib")
BIN = os.path.join(PKG, "bin")
LIBNAME = os.path.join(LIB, "libspherocyl.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# .cu units and whether they may contract multiply-adds
CU_UNITS = {
    "sc_pass64.cu": False,
    "sc_cells.cu": False,
    "sc_pass_mixed.cu": True,
    "sc_noalloc.cu": False,
    "sc_fire.cu": True,
    "sc_cg.cu": False,
    "sc_gen_device.cu": False,
}
CPP_UNITS = ["sc_host.cpp", "sc_api.cpp", "sc_generate.cpp", "sc_io.cpp"]
CLI_UNITS = {
    "spherocyl_strain": "cli_strain.cpp",
    "spherocyl_resize": "cli_resize.cpp",
    "spherocyl_minimize": "cli_minimize.cpp",
    "spherocyl_pure_shear": "cli_pure_shear.cpp",
    "spherocyl_find_jam": "cli_find_jam.cpp",
    "spherocyl_qs_compress": "cli_qs_compress.cpp",
    "spherocyl_y_compress": "cli_y_compress.cpp",
    "spherocyl_configmaker": "cli_configmaker.cpp",
}


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("SC_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)


def _newer(src_list: list[str], target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_list)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "spherocyl.h"))
    return hs


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    """Compile everything that is out of date; returns the library path."""
    cuda = cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB, exist_ok=True)
    os.makedirs(BIN, exist_ok=True)
    headers = _headers()
    jobs_list = []
    objs = []
    for name, fmad in CU_UNITS.items():
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   f"-fmad={'true' if fmad else 'false'}", "-Xptxas", "-v" if verbose else "-O3",
                   "-c", src, "-o", obj]
            jobs_list.append(cmd)
    for name in CPP_UNITS:
        src = os.path.join(CSRC, name)
        if not os.path.exists(src):
            continue
        obj = os.path.join(OBJ, name + ".o")
        objs.append(obj)
        if force or _newer([src] + headers, obj):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall",
                   f"-I{os.path.join(cuda, 'include')}", "-c", src, "-o", obj]
            jobs_list.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(_run, jobs_list))
    if force or jobs_list or not os.path.exists(LIBNAME):
        tmp = LIBNAME + ".tmp"
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart=static", "-ldl", "-lpthread"])
        os.replace(tmp, LIBNAME)
    # command-line drivers (link against the shared library)
    for exe, src_name in CLI_UNITS.items():
        src = os.path.join(CSRC, src_name)
        out = os.path.join(BIN, exe)
        if not os.path.exists(src):
            continue
        if force or _newer([src, LIBNAME] + headers, out):
            _run(["g++", "-O2", "-std=c++17", "-Wall", "-o", out, src, f"-L{LIB}", "-lspherocyl",
                  f"-Wl,-rpath,{LIB}", "-Wl,-rpath,$ORIGIN/../lib"])
    return LIBNAME


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIBNAME)
