// Probe of the reference's own field header (zprize/ntt/host/gf.h), compiled from the file where
// it lies by oracle/build.py into oracle/_ref/ (test infrastructure; nothing of it ships).
// Reads pairs (a, b) of little-endian u64 from stdin and writes a*b, a+b, a-b as the reference's
// GF class computes them; with the argument "omega" it writes the 33 roots of its OMEGA table.
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "gf.h"

int main(int argc, char **argv) {
  if (argc > 1 && strcmp(argv[1], "omega") == 0) {
    for (int i = 0; i < 33; i++) {
      const uint64_t v = OMEGA[i].to_uint64();
      fwrite(&v, 8, 1, stdout);
    }
    return 0;
  }
  uint64_t ab[2];
  while (fread(ab, 8, 2, stdin) == 2) {
    GF a(ab[0]), b(ab[1]);
    const uint64_t r[3] = {(a * b).to_uint64(), (a + b).to_uint64(), (a - b).to_uint64()};
    fwrite(r, 8, 3, stdout);
  }
  return 0;
}
