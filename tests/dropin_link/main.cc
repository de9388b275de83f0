// A caller of the reference library, unchanged: it declares ts::zquatev the
// way the reference's header does (zquatev.h:54), is compiled without any
// header of this project, and is linked against libzquatev_gb300.so instead of
// the reference. It reads D (column-major ld2 x n2 complex doubles) from a
// file, calls ts::zquatev, and writes the info, eig[0..n2-1] and D back.
//
//   usage: dropin_main <n2> <ld2> <in.bin> <out.bin>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace ts {
int zquatev(const int n2, std::complex<double>* const D, const int ld2, double* const eig);
}

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s n2 ld2 in.bin out.bin\n", argv[0]);
    return 2;
  }
  const int n2 = std::atoi(argv[1]), ld2 = std::atoi(argv[2]);
  std::vector<std::complex<double>> D((size_t)ld2 * n2);
  std::vector<double> eig(n2, 7.25);
  FILE* f = std::fopen(argv[3], "rb");
  if (!f || std::fread(D.data(), sizeof(D[0]), D.size(), f) != D.size()) return 3;
  std::fclose(f);
  const int info = ts::zquatev(n2, D.data(), ld2, eig.data());
  FILE* g = std::fopen(argv[4], "wb");
  if (!g) return 4;
  std::fwrite(&info, sizeof(int), 1, g);
  std::fwrite(eig.data(), sizeof(double), eig.size(), g);
  std::fwrite(D.data(), sizeof(D[0]), D.size(), g);
  std::fclose(g);
  return info == 0 ? 0 : 1;
}
