// Test driver, not product code: prints the crystal surface behind an `ft`
// stiffness kernel (cell, basis, neighbour list up to a cutoff) for
// tests/test_surfaces.py.  Usage: surface_neighbors "<kernel arguments>" rcut
#include <cstdio>
#include <sstream>
#include <string>
#include <vector>

#include "stiffness.h"

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  std::istringstream is(argv[1]);
  std::vector<std::string> tok;
  for (std::string t; is >> t;) tok.push_back(t);
  size_t pos = 0;
  gfmd::StiffnessKernel *k = gfmd::StiffnessKernel::create(tok, pos);
  gfmd::CrystalSurface s = k->surface();
  s.compute_neighbor_list(std::stod(argv[2]));
  std::printf("cell");
  for (double c : s.cell) std::printf(" %.17g", c);
  std::printf("\npos");
  for (double p : s.pos) std::printf(" %.17g", p);
  std::printf("\n");
  for (const gfmd::LatticeNeighbor &n : s.neigh)
    std::printf("n %d %d %d %d %d %.17g %.17g %.17g %.17g %d\n", n.i, n.j, n.x, n.y, n.ab, n.r[0], n.r[1], n.r[2],
                n.rnorm, n.shell);
  delete k;
  return 0;
}
