// Runs SPH::Domain::AddBoxLength of include/persiansph/Domain.h for one box
// given on the command line and writes int64 n, x[3n], mass[n] (raw binary).
// args: dim tag V0 V1 V2 Lx Ly Lz r rho h type rotation random fixed out.bin
#include <cstdio>
#include <cstdlib>

#include "Domain.h"

int main(int argc, char** argv) try {
  if (argc != 17) {
    std::printf("usage: %s dim tag V0 V1 V2 Lx Ly Lz r rho h type rotation random fixed out.bin\n", argv[0]);
    return 2;
  }
  auto d = [&](int k) { return std::atof(argv[k]); };
  SPH::Domain dom;
  dom.Dimension = std::atoi(argv[1]);
  dom.AddBoxLength(std::atoi(argv[2]), Vec3_t(d(3), d(4), d(5)), d(6), d(7), d(8), d(9), d(10), d(11),
                   std::atoi(argv[12]), std::atoi(argv[13]), std::atoi(argv[14]) != 0, std::atoi(argv[15]) != 0);
  FILE* f = std::fopen(argv[16], "wb");
  const int64_t n = (int64_t)dom.Particles.Size();
  std::fwrite(&n, sizeof n, 1, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(dom.Particles[a]->x.data(), sizeof(double), 3, f);
  for (size_t a = 0; a < dom.Particles.Size(); a++) std::fwrite(&dom.Particles[a]->Mass, sizeof(double), 1, f);
  std::fclose(f);
  return 0;
}
MECHSYS_CATCH
