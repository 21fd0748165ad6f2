"""Build ``libautojax_gb300.so`` in-tree from ``csrc/*.cu`` for sm_103a with nvcc.

Each translation unit compiles in parallel to an object under ``_build/``;
the objects link into a shared library next to this file.  Nothing is
installed into site-packages, so the library a process loads is always the
in-tree one.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
PROJECT = PKG.parent
CSRC = PROJECT / "csrc"
INCLUDE = PROJECT.parent / "include"
BUILD = PROJECT / "_build"
LIB_NAME = "libautojax_gb300.so"
LIB_PATH = PKG / LIB_NAME
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _flags() -> list[str]:
    return ARCH + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler",
        "-fPIC",
        "-I",
        str(INCLUDE),
        "-I",
        str(CSRC),
        "-DAJ_BUILDING_LIBRARY",
    ]


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def up_to_date() -> bool:
    if not LIB_PATH.exists():
        return False
    t = LIB_PATH.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every CUDA source and link the shared library; returns its path."""
    if not force and up_to_date():
        return LIB_PATH
    nvcc = str(cuda_home() / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    flags = _flags()
    srcs = _sources()

    def compile_one(src: Path) -> Path:
        obj = BUILD / (src.stem + ".o")
        cmd = [nvcc, *flags, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    lib_dir = cuda_home() / "lib64"
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "shared", "-Xlinker", f"-rpath={lib_dir}"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
