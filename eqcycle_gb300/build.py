"""Build libeqc.so (the CUDA C ABI of include/eqc.h) in-tree with nvcc for sm_103a.

    python -m eqcycle_gb300.build [--force]

Sources are compiled in parallel into eqcycle_gb300/_build/ and linked into
eqcycle_gb300/libeqc.so.  Only the GB300 target (sm_103a) is generated.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libeqc.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
# Translation units whose arithmetic mirrors the reference's operation order exactly
# (friction Newton, state evolution): no FMA contraction.
NO_FMAD = {"stepper.cu", "setup.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libeqc")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _compile(src: str, obj: str, extra=()) -> str:
    cmd = [nvcc()] + ARCH + COMMON + list(extra)
    if os.path.basename(src) in NO_FMAD:
        cmd += ["-fmad=false"]
    cmd += ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def elf_matches_host(path: str) -> bool:
    """True when the ELF file at path targets this machine (x86-64 vs aarch64)."""
    try:
        with open(path, "rb") as f:
            hdr = f.read(20)
    except OSError:
        return False
    if len(hdr) < 20 or hdr[:4] != b"\x7fELF":
        return False
    mach = int.from_bytes(hdr[18:20], "little")
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return want is None or mach == want


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "machine")
    mach = platform.machine()
    if not os.path.exists(stamp) or open(stamp).read().strip() != mach or \
            (os.path.exists(LIB) and not elf_matches_host(LIB)):
        force = True
    with open(stamp, "w") as f:
        f.write(mach)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    hdr_time = max((os.path.getmtime(h) for h in _headers()), default=0.0)
    jobs = []
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_time):
            jobs.append((s, o))
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(_compile, s, o, extra): s for s, o in jobs}
            for f in cf.as_completed(futs):
                msg = f.result()
                if verbose and msg:
                    print(f"--- {os.path.basename(futs[f])}\n{msg}", file=sys.stderr)
    if jobs or not os.path.exists(LIB) or force:
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
