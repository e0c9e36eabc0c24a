"""In-tree build of the CUDA C-ABI library ``libmpasg.so`` for sm_103a.

Plain ``nvcc`` (no torch headers, no cmake): each translation unit under ``csrc/`` is
compiled in parallel to an object file, then linked into a shared library next to this
file.  A stamp of the sources and flags skips the rebuild when nothing changed.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libmpasg.so"
SOURCES = ("kern_column.cu", "kern_tend.cu", "kern_diag.cu", "kern_transport.cu", "driver.cu", "reorder.cu",
           "kern_adjoint.cu", "kern_transport_adj.cu", "kern_adj_column.cu", "kern_adj_tend.cu", "kern_adj_diag.cu",
           "driver_adj.cu", "kern_digest.cu", "kern_tan_column.cu", "kern_tan_tend.cu", "driver_tan.cu")
ARCH = ("-gencode", "arch=compute_103a,code=sm_103a")


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmpasg.so")


def _flags(extra: tuple[str, ...]) -> list[str]:
    return [*ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            f"-I{INCLUDE}", *extra]


def _stamp(flags: list[str]) -> str:
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)):
        h.update(name.encode())
        h.update((CSRC / name).read_bytes())
    h.update((INCLUDE / "mpasg.h").read_bytes())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def build(force: bool = False, extra_flags: tuple[str, ...] = (), verbose: bool = False) -> pathlib.Path:
    """Compile ``libmpasg.so`` (idempotent); returns its path."""
    nvcc = nvcc_path()
    flags = _flags(tuple(extra_flags))
    stamp = _stamp(flags)
    stamp_file = BUILD / "stamp"
    if not force and LIB.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    BUILD.mkdir(exist_ok=True)

    def compile_one(src: str) -> pathlib.Path:
        obj = BUILD / (pathlib.Path(src).stem + ".o")
        cmd = [nvcc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    stamp_file.write_text(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
