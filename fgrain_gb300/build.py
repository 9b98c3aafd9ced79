"""Builds libfgrain_cuda.so in-tree for sm_103a (GB300).

Each .cu translation unit (csrc/) is compiled in parallel with nvcc and each host-only .cpp
translation unit (host/) with the host C++ compiler, then all are linked into one shared library
next to this file.  Object files go to fgrain_gb300/_build/.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
HOST = HERE / "host"
INCLUDE = HERE.parent / "include"
OUT = HERE / "libfgrain_cuda.so"
BUILD = HERE / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "--extended-lambda",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off"]


def cxx() -> str:
    return os.environ.get("CXX") or "g++"


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(HOST.glob("*.cpp"))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    objs = []
    jobs = []
    for src in sources():
        obj = BUILD / (src.stem + (".o" if src.suffix == ".cu" else ".host.o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            if src.suffix == ".cu":
                cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            else:
                cmd = [cxx(), *HOST_FLAGS, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failed = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if r.returncode != 0:
                failed.append((cmd, r.stderr))
            elif verbose and r.stderr.strip():
                print(r.stderr, file=sys.stderr)
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + e for c, e in failed)
        raise RuntimeError("compile failed:\n" + msg)
    if force or jobs or _stale(OUT, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(OUT), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
