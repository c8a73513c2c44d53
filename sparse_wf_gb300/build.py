"""Builds ``libfire.so`` (the C-ABI library of the hot path) in-tree for sm_103a.

Every translation unit is compiled in parallel with nvcc and linked into
``sparse_wf_gb300/libfire.so``.  Rebuilds only when a source is newer than the
library (or ``force=True``).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB = PKG / "libfire.so"
OBJ = ROOT / "_build" / "obj"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-static-global-template-stub=false",
                     "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the FiRE CUDA library cannot be built")
    return path


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = sources() + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    OBJ.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def compile_one(src: Path) -> Path:
        obj = OBJ / (src.stem + ".o")
        cmd = [cc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def jax_ffi_include() -> Path | None:
    """jaxlib's FFI header directory (xla/ffi/api/ffi.h), or None where jax is not installed."""
    try:
        import jax
    except ImportError:
        return None
    inc = Path(jax.ffi.include_dir())
    return inc if (inc / "xla" / "ffi" / "api" / "ffi.h").exists() else None


def build_xla(force: bool = False) -> Path | None:
    """Builds libfire_xla.so (the XLA FFI handlers of xla/fire_xla.cc, linked with libfire.so) where jax is
    installed; returns None (nothing built) where it is not."""
    inc = jax_ffi_include()
    if inc is None:
        return None
    lib = build(force)
    out = PKG / "libfire_xla.so"
    src = PKG / "xla" / "fire_xla.cc"
    if not force and out.exists() and out.stat().st_mtime > max(src.stat().st_mtime, lib.stat().st_mtime):
        return out
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{inc}",
           "-x", "cu", str(src), "-o", str(out), f"-L{PKG}", "-lfire", f"-Xlinker=-rpath,{PKG}", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    t = build(force="--force" in sys.argv, verbose=True)
    print(t)
