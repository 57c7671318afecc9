"""Build libnlse_sm103.so in-tree with nvcc (sm_103a only).

The translation units compile in parallel; the ptxas register/spill report of
each one is kept next to the objects (``_lib/obj/*.ptxas.txt``).  A stamp
file holding the hash of the sources and flags skips rebuilding when nothing
changed.
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIBDIR = PKG / "_lib"
LIBNAME = "libnlse_sm103.so"

SOURCES = [
    "capi.cu",
    "pointwise.cu",
    "rows_f32_c1.cu",
    "rows_f32_c2.cu",
    "rows_f64_c1.cu",
    "rows_f64_c2.cu",
    "cols_f32.cu",
    "cols_f64.cu",
    "rows_pair16_mid.cu",
    "rows_pair16_last.cu",
    "rows_pair8_mid.cu",
    "rows_pair8_last.cu",
    "cols_pair.cu",
    "rows_deep_mid.cu",
    "rows_deep_last.cu",
    "cols_deep.cu",
    "nonlocal_rows.cu",
    "multi_pair.cu",
    "multi_rows_mid.cu",
    "multi_rows_last.cu",
    "fno.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe is None:
        cand = Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnlse_sm103")
    return exe


def _digest() -> str:
    h = hashlib.sha256()
    h.update(" ".join(ARCH + CFLAGS).encode())
    for p in sorted(list(CSRC.glob("*")) + list(INCLUDE.glob("*.h"))):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    return h.hexdigest()


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    """Compile and link the shared library; returns its path."""
    out = lib_path()
    stamp = LIBDIR / "build.stamp"
    digest = _digest()
    if not force and out.exists() and stamp.exists() and stamp.read_text() == digest:
        return out
    objdir = LIBDIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    exe = nvcc()

    def compile_one(src: str) -> Path:
        obj = objdir / (Path(src).stem + ".o")
        cmd = [exe, *ARCH, *CFLAGS, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        (objdir / (Path(src).stem + ".ptxas.txt")).write_text(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr[-4000:]}")
        if verbose:
            print(f"  compiled {src}")
        return obj

    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    # longest translation units first
    order = sorted(SOURCES, key=lambda s: (not s.startswith(("rows", "multi_rows")), s))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, order))
    tmp = out.with_suffix(".so.tmp")
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, out)
    stamp.write_text(digest)
    return out


if __name__ == "__main__":
    import time

    t = time.time()
    p = build(force=True, verbose=True)
    print(f"built {p} in {time.time() - t:.1f} s")
