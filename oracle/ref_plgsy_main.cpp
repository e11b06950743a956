// Driver for the reference's own PLASMA generator — TEST INFRASTRUCTURE ONLY.
// Compiled by oracle/build.py against examples/potrf/core_plgsy.h where it lies in the reference
// checkout (never copied here); the binary goes to oracle/_ref/ and is used only to pin the
// oracle's restatement (orc_plgsy_tiles) and to write golden fixtures.
// It walks the lower tiles exactly as examples/potrf/plgsy.h:8-34 does (tempmm/tempnn ragged
// sizes, ldam = NB, global offsets I*NB, J*NB) and writes them in the oracle's slot order.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <vector>
#include "core_plgsy.h"

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s N NB bump seed out.bin\n", argv[0]);
    return 2;
  }
  const int N = std::atoi(argv[1]), NB = std::atoi(argv[2]);
  const double bump = std::atof(argv[3]);
  const unsigned long long seed = std::strtoull(argv[4], nullptr, 10);
  const int NT = (N + NB - 1) / NB;
  const long nslots = (long)NT * (NT + 1) / 2;
  std::vector<double> tiles((size_t)nslots * NB * NB, 0.0);
  for (int J = 0; J < NT; ++J)
    for (int I = J; I < NT; ++I) {
      const long slot = (long)J * NT - (long)J * (J - 1) / 2 + (I - J);
      double* a = tiles.data() + slot * (long)NB * NB;
      const int tempmm = (I == NT - 1) ? N - I * NB : NB;
      const int tempnn = (J == NT - 1) ? N - J * NB : NB;
      CORE_plgsy<double>(bump, tempmm, tempnn, a, NB, N, I * NB, J * NB, seed);
    }
  FILE* f = std::fopen(argv[5], "wb");
  if (!f) return 1;
  std::fwrite(tiles.data(), sizeof(double), tiles.size(), f);
  std::fclose(f);
  return 0;
}
