"""Build the in-tree CUDA library ``niftyrec_gb300/lib_et_array_interface.so``
for sm_103a (GB300) with nvcc: one object per translation unit, compiled in
parallel, then one shared-library link.  No CMake, no torch extension
machinery: the library has a plain C ABI and depends only on the CUDA runtime.

    python -m niftyrec_gb300.build          # build if stale
    python -m niftyrec_gb300.build --force  # rebuild everything
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lib_et_array_interface.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["et_geometry.cpp", "et_engine.cpp", "et_api.cpp", "et_profile.cpp", "et_general.cu", "et_ygantry.cu",
           "et_yg_project.cu", "et_yg_proj_r01.cu", "et_yg_proj_r23.cu", "et_yg_proj_r45.cu", "et_yg_proj_r67.cu",
           "et_yg_back.cu", "et_yg_dmu.cu", "et_yg_grad.cu", "et_update.cu", "et_noalloc.cu", "et_plan.cpp", "et_fisher.cu", "et_nifti.cpp"]
TOOL = os.path.join(HERE, "rec_spect")  # command-line reconstruction (csrc/rec_spect.cpp)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
              "-I" + CSRC, "-I" + INCLUDE]


def _nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = os.path.join(cuda, "bin", "nvcc")
    return path if os.path.exists(path) else (shutil.which("nvcc") or "nvcc")


def _zlib() -> bool:
    """zlib headers and a linkable library (for .nii.gz)."""
    import glob

    if not os.path.exists("/usr/include/zlib.h"):
        return False
    return bool(glob.glob("/usr/lib*/libz.so") + glob.glob("/usr/lib*/*/libz.so") + glob.glob("/lib*/*/libz.so"))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    if os.path.isdir(INCLUDE):
        hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if _stale(obj, [path, __file__] + _headers()):
        cmd = [_nvcc()] + ARCH + NVCC_FLAGS + (["-DNRGB_ZLIB"] if src == "et_nifti.cpp" and _zlib() else []) + [
            "-c", path, "-o", obj]
        if src.endswith(".cu") and verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every CUDA/C++ source for sm_103a and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if force or _stale(LIB, objs):
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        cmd = [_nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB] + objs + [
            "-Xlinker", "-rpath," + os.path.join(cuda, "lib64")] + (["-lz"] if _zlib() else [])
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    tool_src = os.path.join(CSRC, "rec_spect.cpp")
    if force or _stale(TOOL, [LIB, tool_src] + _headers()):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-I" + INCLUDE, tool_src, "-o", TOOL, "-L" + HERE,
               "-l:lib_et_array_interface.so", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"rec_spect build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
