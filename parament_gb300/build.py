"""Builds libparament.so (the GB300 equiprop library) in-tree with nvcc.

Every translation unit under ``csrc/`` is compiled for sm_103a in parallel and
linked into ``parament_gb300/libparament.so``; no CMake, no setuptools.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libparament.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", INCLUDE, "-I", CSRC]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libparament.so")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _lib_matches(arch: str) -> bool:
    """True when the existing libparament.so is an ELF file for this host."""
    machine = {"x86_64": 62, "aarch64": 183}.get(arch)
    try:
        with open(LIB, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    return machine is not None and len(head) == 20 and head[:4] == b"\x7fELF" and \
        int.from_bytes(head[18:20], "little") == machine


def _stale(obj: str, src: str, hdr_mtime: float) -> bool:
    return not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_mtime)


def build(verbose: bool = False, force: bool = False, extra_flags=None) -> str:
    import platform

    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    # Objects from another host architecture (a copied tree) are never reused.
    stamp = os.path.join(BUILD, "host_arch")
    arch = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != arch or \
            (os.path.exists(LIB) and not _lib_matches(arch)):
        force = True
        with open(stamp, "w") as f:
            f.write(arch)
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    srcs = _sources()
    objs = [os.path.join(BUILD, os.path.basename(s) + ".o") for s in srcs]
    flags = FLAGS + list(extra_flags or [])

    def compile_one(src, obj):
        if not force and not _stale(obj, src, hdr_mtime):
            return None
        cmd = [nvcc] + ARCH + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(compile_one, s, o) for s, o in zip(srcs, objs)]
        for f in futs:
            f.result()
    if force or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
