"""In-tree build of libvvlic.so (the CUDA kernels and the C ABI of include/vvlic.h).

Every .cu file under csrc/ is compiled for sm_103a in parallel and linked into
vectorvisualization_gb300/_lib/libvvlic.so.  No torch extension machinery is involved: the
library is a plain C-ABI shared object loaded with ctypes.

    python -m vectorvisualization_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libvvlic.so")
BUILD_DIR = os.path.join(ROOT, "_build", "vvlic")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
# Files whose float arithmetic must round like the reference's CPU code.
NO_FMA = {"preprocess.cu", "noalloc.cu", "illum.cu"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvvlic")


def _sources() -> list[str]:
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand:
            return cand
    raise RuntimeError("no C++ compiler found")


def _hash_sources(h):
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                with open(p, "rb") as fh:
                    h.update(fh.read())
    return h


def _digest(extra: str) -> str:
    return _hash_sources(hashlib.sha256(extra.encode())).hexdigest()


def source_digest() -> str:
    """Digest of the kernel and ABI sources alone (no flags, no machine): identifies the code a
    profile was captured with, so a committed measurement can be matched to the current build."""
    return _hash_sources(hashlib.sha256()).hexdigest()[:16]


def build(force: bool = False, verbose: bool = False, jobs: int | None = None, extra: list[str] | None = None,
          variant: str | None = None) -> str:
    """Compile libvvlic.so if its sources changed; returns the library path.

    `extra` nvcc flags default to $VVLIC_NVCC_EXTRA (e.g. -DVVLIC_MIN_BLOCKS=8 to trade
    registers for occupancy).  A `variant` name builds into _lib/<variant>/ and _build/<variant>/
    instead, leaving the default library alone (e.g. the VVLIC_BOUNDS_CHECK build)."""
    nvcc = _nvcc()
    out_dir = OUT_DIR if not variant else os.path.join(OUT_DIR, variant)
    build_dir = BUILD_DIR if not variant else os.path.join(os.path.dirname(BUILD_DIR), variant)
    lib = os.path.join(out_dir, "libvvlic.so")
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(out_dir, exist_ok=True)
    stamp = os.path.join(out_dir, "libvvlic.stamp")
    if extra is None:
        extra = os.environ.get("VVLIC_NVCC_EXTRA", "").split()
    digest = _digest(" ".join(ARCH + COMMON + extra) + os.uname().machine)
    if not force and os.path.exists(lib) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return lib

    def compile_one(src: str) -> str:
        obj = os.path.join(build_dir, os.path.splitext(src)[0] + ".o")
        if src.endswith(".cpp"):  # host-only C++ (file formats): the plain C++ compiler
            cmd = [_cxx(), "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-c",
                   os.path.join(CSRC, src), "-o", obj]
        else:
            cmd = [nvcc, *ARCH, *COMMON, *extra, "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
        if src in NO_FMA:
            cmd[1:1] = ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = _sources()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return lib


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    args = ap.parse_args(argv)
    print(build(force=args.force, verbose=args.verbose))
    return 0


if __name__ == "__main__":
    sys.exit(main())
