"""Build recipe for the C oracle (test infrastructure): oracle/_build/libmsm_oracle.so.

    python oracle/build.py

Plain gcc with OpenMP; no architecture-specific flags, so it builds the same on x86_64 and
aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmsm_oracle.so")
SRC = os.path.join(HERE, "cpu_msm.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = f"{LIB}.{os.getpid()}.tmp"  # one file per builder; the rename below is atomic
    cmd = [os.environ.get("CC", "gcc"), "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", SRC,
           "-o", tmp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
