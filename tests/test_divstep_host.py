"""The divstep inversion (csrc/fq_divstep.cuh) is plain integer C++ shared by host and device;
this compiles it for the host with g++ and checks it against Python's modular inverse on edge
values and random values below q, both the one-thread form and the four-lane schedule of
fq_inv_quad run lane after lane (every value must give the same inverse both ways).  The device build of the same code is checked through
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
// the four-lane schedule of fq_inv_quad, one lane after another: each batch's four
// combinations through ds_combine_any with the lanes' operands
static bool by_lanes(const uint32_t (&a)[12], const uint32_t (&q12)[12], uint32_t (&out)[12]) {
  uint32_t f[DS_LIMBS] = {}, g[DS_LIMBS] = {}, d[DS_LIMBS] = {}, e[DS_LIMBS] = {}, q[DS_LIMBS] = {};
  uint32_t nz = 0;
  for (int i = 0; i < 12; i++) { f[i] = q[i] = q12[i]; g[i] = a[i]; nz |= a[i]; out[i] = 0; }
  e[0] = 1;
  if (!nz) return true;
  int delta = 1;
  for (int batch = 0; batch < 64; batch++) {
    int32_t u, v, qq, r;
    delta = ds_batch30(delta, f[0], g[0], u, v, qq, r);
    uint32_t res[4][DS_LIMBS];
    for (int l = 0; l < 4; l++)
      ds_combine_any(res[l], (l & 1) ? qq : u, l < 2 ? f : d, (l & 1) ? r : v, l < 2 ? g : e, q, l >= 2);
    uint32_t gz = 0;
    for (int i = 0; i < DS_LIMBS; i++) { f[i] = res[0][i]; g[i] = res[1][i]; d[i] = res[2][i]; e[i] = res[3][i]; gz |= g[i]; }
    if (!gz) {
      if (ds_is_neg(f)) {
        int64_t acc = 0;
        for (int i = 0; i < DS_LIMBS; i++) { acc += (int64_t)q[i] - (int64_t)d[i]; d[i] = (uint32_t)acc; acc >>= 32; }
      }
      for (int i = 0; i < 12; i++) out[i] = d[i];
      return true;
    }
  }
  return false;
}
int main() {
  const uint32_t q[12] = {%s};
  uint32_t a[12], out[12], out2[12];
  while (fread(a, 4, 12, stdin) == 12) {
    const bool ok = ds_inverse(a, q, out) && by_lanes(a, q, out2);
    bool same = true;
    for (int i = 0; i < 12; i++) same &= out[i] == out2[i];
    const bool all = ok && same;
    fwrite(&all, 1, 1, stdout);
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
