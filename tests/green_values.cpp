// Test driver, not product code: prints the surface Green's function of the
// `nonperiodic` stiffness style (displacement under a unit force spread over
// one grid cell) for tests/test_green.py.
// Usage: green_values "<kernel arguments>" dx dy, then "i j" pairs on stdin;
// prints the 9 entries G[3 a + b] per pair.
#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "stiffness.h"

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  std::istringstream is(argv[1]);
  std::vector<std::string> tok;
  for (std::string t; is >> t;) tok.push_back(t);
  size_t pos = 0;
  gfmd::StiffnessKernel *k = gfmd::StiffnessKernel::create(tok, pos);
  const double dx = std::stod(argv[2]), dy = std::stod(argv[3]);
  int i, j;
  while (std::cin >> i >> j) {
    double G[9];
    k->nonperiodic_green(i, j, dx, dy, G);
    for (int a = 0; a < 9; a++) std::printf(a ? " %.17g" : "%.17g", G[a]);
    std::printf("\n");
  }
  delete k;
  return 0;
}
