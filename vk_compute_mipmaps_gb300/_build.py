"""Build recipe for the native library libnvpro_pyramid_cuda.so (sm_103a).

Each translation unit is compiled by nvcc in parallel into _build/, then linked
into the package directory, where vk_compute_mipmaps_gb300 loads it.
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libnvpro_pyramid_cuda.so"
SOURCES = ["api.cpp", "host_io.cpp", "kernels_portable.cu", "kernels_tma.cu", "kernels_adjoint.cu",
           "kernels_general.cu", "kernels_batch.cu", "kernels_stage.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "--expt-relaxed-constexpr", "-I", str(PKG.parent / "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, ptxas_verbose: bool) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
    if ptxas_verbose and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if ptxas_verbose:
        print(res.stderr)
    return obj


def build(ptxas_verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, ptxas_verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(ptxas_verbose="-v" in sys.argv))
