"""Builds liblmgpu.so in-tree with nvcc for sm_103a (GB300)."""
from __future__ import annotations

import os
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR.parent / "csrc"
INCLUDE = PKG_DIR.parent.parent / "include"
LIB_PATH = PKG_DIR / "liblmgpu.so"
SOURCES = ["lmgpu_api.cu", "lmgpu_kernels.cu", "lmgpu_fused.cu", "lmgpu_noalloc.cu", "lmgpu_batch.cu", "lmgpu_adjoint.cu",
           "lmgpu_ring.cu", "lmgpu_kpm.cu", "lmgpu_ell.cu", "lmgpu_stream.cu", "lmgpu_eigh.cu",
           "lmgpu_resident.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}"]
# extra nvcc flags for tuning builds (e.g. LMGPU_NVCC_FLAGS=-DLM_FUSED_SITES=2); the default
# build needs none
EXTRA = os.environ.get("LMGPU_NVCC_FLAGS", "").split()


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the lmgpu CUDA library cannot be built")
    return cand


def _newest_source_mtime() -> float:
    files = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max(f.stat().st_mtime for f in files)


def up_to_date() -> bool:
    return LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= _newest_source_mtime()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every translation unit in parallel and link the shared library."""
    if not force and up_to_date():
        return LIB_PATH
    nvcc = nvcc_path()
    with tempfile.TemporaryDirectory(prefix="lmgpu_build_") as tmp:
        objs = []

        def compile_one(src: str) -> str:
            obj = os.path.join(tmp, src.replace(".cu", ".o"))
            cmd = [nvcc, *ARCH, *FLAGS, *EXTRA, "-c", str(CSRC / src), "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose:
                print(r.stdout, r.stderr)
            return obj

        with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
            objs = list(ex.map(compile_one, SOURCES))
        tmp_lib = os.path.join(tmp, "liblmgpu.so")
        cmd = [nvcc, *ARCH, "-shared", *objs, "-o", tmp_lib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
        shutil.move(tmp_lib, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
