"""Build of the native engine ``libtopt_gb300.so`` (CUDA, sm_103a only).

The library is compiled in-tree with nvcc: one object per translation unit,
compiled in parallel, then linked into ``sktopt_gb300/lib/``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
LIBDIR = PKG / "lib"
LIBNAME = "libtopt_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = Path(cuda) / "bin" / "nvcc"
    if p.exists():
        return str(p)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtopt_gb300")


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def library_path() -> Path:
    return LIBDIR / LIBNAME


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA/C++ source of the engine and link the shared library."""
    lib = library_path()
    if not force and not _stale(lib):
        return lib
    nvcc = nvcc_path()
    objdir = PKG.parent / "_build"
    objdir.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}",
              "-diag-suppress", "177"]

    def compile_one(src: Path):
        obj = objdir / (src.stem + ".o")
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, "-lineinfo", *common, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(1, min(os.cpu_count() or 8, len(srcs)))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force=True, verbose=True))
