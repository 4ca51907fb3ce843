"""The divstep inversion (csrc/fq_divstep.cuh) is plain integer C++ shared by host and device;
this compiles it for the host with g++ and checks it against Python's modular inverse on edge
values and random values below q.  The device build of the same code is checked through
msm_field_selftest in the GPU suite."""
import os
import random
import shutil
import struct
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "hardcaml_zprize_gb300", "csrc", "fq_divstep.cuh")

DRIVER = r"""
#include <cstdio>
#include <cstdint>
#include "%s"
int main() {
  const uint32_t q[12] = {%s};
  uint32_t a[12], out[12];
  while (fread(a, 4, 12, stdin) == 12) {
    const bool ok = ds_inverse(a, q, out);
    fwrite(&ok, 1, 1, stdout);
    fwrite(out, 4, 12, stdout);
  }
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_divstep_inverse_matches_python(ref, tmp_path):
    Q = ref.Q
    qwords = ", ".join("0x%08xu" % ((Q >> (32 * i)) & 0xFFFFFFFF) for i in range(12))
    src = tmp_path / "ds.cpp"
    src.write_text(DRIVER % (HDR, qwords))
    exe = tmp_path / "ds"
    subprocess.run(["g++", "-O2", "-std=c++17", str(src), "-o", str(exe)], check=True)
    rng = random.Random(11)
    vals = [0, 1, 2, 3, Q - 1, Q - 2, (Q - 1) // 2, 2**32, 2**376, Q - 2**32, ref.MONT_R % Q]
    vals += [rng.randrange(Q) for _ in range(3000)]
    inp = b"".join(struct.pack("<12I", *[(v >> (32 * i)) & 0xFFFFFFFF for i in range(12)]) for v in vals)
    out = subprocess.run([str(exe)], input=inp, capture_output=True, check=True).stdout
    assert len(out) == 49 * len(vals)
    for k, v in enumerate(vals):
        rec = out[49 * k:49 * (k + 1)]
        got = sum(w << (32 * i) for i, w in enumerate(struct.unpack("<12I", rec[1:])))
        assert rec[0] == 1
        assert got == (pow(v, -1, Q) if v else 0), f"value {k}"
