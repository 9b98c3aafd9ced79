"""Builds the CPU oracle (TEST INFRASTRUCTURE) into oracle/build/liboracle.so.

g++ -O3 with OpenMP; -ffp-contract=off keeps every double operation individually rounded (GCC on
aarch64 would otherwise fuse multiply-adds), so the oracle rounds exactly like the reference's
Rust code and like the device's FP64 predicates.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "build" / "liboracle.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    srcs = [HERE / "fg_oracle.cpp", HERE / "fg_oracle_film.cpp", HERE / "fg_oracle_fast.cpp"]
    deps = srcs + [HERE / "fg_oracle.h", HERE / "philox.h"]
    if not force and OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", *map(str, srcs), "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
