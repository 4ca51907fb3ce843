"""Build recipe for the C oracle (test infrastructure): oracle/_build/libmsm_oracle.so (the MSM
oracle cpu_msm.c and the NTT oracle cpu_ntt.c).

    python oracle/build.py

Plain gcc with OpenMP; no architecture-specific flags, so it builds the same on x86_64 and
aarch64 hosts.

build_ref() also compiles the one piece of the reference that builds from its own files: the NTT
host's field header zprize/ntt/host/gf.h, included from where it lies in a checkout of the
reference (HARDCAML_ZPRIZE_REF, default /root/reference) by oracle/ref_gf_probe.cpp, into
oracle/_ref/ref_gf_probe.  It is skipped when no checkout is present.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmsm_oracle.so")
SRCS = [os.path.join(HERE, "cpu_msm.c"), os.path.join(HERE, "cpu_ntt.c")]
REF_OUT = os.path.join(HERE, "_ref")
REF_PROBE = os.path.join(REF_OUT, "ref_gf_probe")


def build(force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(x) for x in SRCS):
        return LIB
    tmp = f"{LIB}.{os.getpid()}.tmp"  # one file per builder; the rename below is atomic
    cmd = [os.environ.get("CC", "gcc"), "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", *SRCS,
           "-o", tmp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_ref() -> str:
    """Compile oracle/ref_gf_probe.cpp against the reference's gf.h; returns the binary's path,
    or "" when no reference checkout is present."""
    ref = os.environ.get("HARDCAML_ZPRIZE_REF", "/root/reference")
    hdr_dir = os.path.join(ref, "zprize", "ntt", "host")
    if not os.path.exists(os.path.join(hdr_dir, "gf.h")):
        return ""
    os.makedirs(REF_OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_gf_probe.cpp")
    tmp = f"{REF_PROBE}.{os.getpid()}.tmp"
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-I", hdr_dir, src, "-o", tmp]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"reference field probe build failed:\n{p.stdout}\n{p.stderr}")
    os.replace(tmp, REF_PROBE)
    return REF_PROBE


if __name__ == "__main__":
    print(build(force=True))
