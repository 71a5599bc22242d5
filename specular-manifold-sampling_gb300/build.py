"""Build recipe for libsms_gb300.so (sm_103a only).

Compiles every translation unit under csrc/ with nvcc in parallel and links one
shared library next to this file.  No CMake, one -gencode, a few TUs, so the
build takes well under a minute here and on the GPU host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR / "csrc"
INCLUDE = PKG_DIR.parent / "include"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "libsms_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "--expt-relaxed-constexpr", "-I", str(INCLUDE),
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsms_gb300.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def lib_path() -> Path:
    return PKG_DIR / LIB_NAME


def _up_to_date(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> Path:
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    srcs = sources()
    objs = [BUILD_DIR / (s.name + ".o") for s in srcs]
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(pair):
        src, obj = pair
        if not force and _up_to_date(obj, [src] + headers):
            return ""
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose or ptxas_info:
        for lg in logs:
            if lg:
                sys.stderr.write(lg)
    out = lib_path()
    if force or not _up_to_date(out, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart_static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv)
    print(lib_path())
