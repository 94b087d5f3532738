"""Build libptycho_gb300.so in-tree with nvcc for sm_103a.

Compiles the CUDA translation units of ``csrc/`` in parallel and links them into
``py4dstem_gb300/_lib/libptycho_gb300.so``. Nothing is installed outside the
package directory. Run ``python -m py4dstem_gb300.build``.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_NAME = "libptycho_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

SOURCES = ["ptycho_position_128.cu", "ptycho_position_96.cu", "ptycho_position_64.cu",
           "ptycho_position_96x128.cu", "ptycho_position_128x96.cu",
           "ptycho_position_48.cu", "ptycho_position_32.cu", "ptycho_gd128.cu",
           "ptycho_staged.cu", "ptycho_reduce.cu", "ptycho_preprocess.cu", "ptycho_volume.cu",
           "ptycho_position.cu",
           "ptycho_capi.cu", "nn_conv.cu", "nn_unet.cu", "nn_data.cu"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libptycho_gb300")


def _inputs():
    files = [os.path.join(CSRC, s) for s in SOURCES]
    files += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    files.append(os.path.join(os.path.dirname(PKG_DIR), "include", "ptycho_gb300.h"))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(f) <= t for f in _inputs() if os.path.exists(f))


def _compile(src: str, extra, verbose: bool) -> str:
    nvcc = nvcc_path()
    obj = os.path.join(BUILD_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc, *ARCH_FLAGS, *COMMON_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout.strip() or res.stderr.strip()):
        print(res.stdout + res.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, verbose or ptxas_info), SOURCES))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), *ARCH_FLAGS, "-shared", *objs, "-o", tmp, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(path)
