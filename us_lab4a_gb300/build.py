"""In-tree build of libusgb.so (CUDA, sm_103a) with nvcc.

Each translation unit is compiled to an object in parallel, then linked into
``us_lab4a_gb300/libusgb.so``; objects go to ``us_lab4a_gb300/_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libusgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["usgb_api.cu", "usgb_prep.cu", "usgb_das.cu", "usgb_das_staged.cu", "usgb_das_group.cu",
           "usgb_das_group_f32.cu", "usgb_das_group_f16.cu", "usgb_das_group_bf16.cu", "usgb_post.cu", "usgb_noalloc.cu",
           "usgb_single.cu", "usgb_two_medium.cu", "usgb_h5.cpp"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libusgb")
    return path


def _flags() -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                   "-Xcompiler", "-ffp-contract=off",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _deps() -> list[str]:
    out = [os.path.join(ROOT, "include", "usgb.h")]
    for f in os.listdir(CSRC):
        out.append(os.path.join(CSRC, f))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile (if stale) and return the path of libusgb.so."""
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = _flags() + list(extra or [])

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
