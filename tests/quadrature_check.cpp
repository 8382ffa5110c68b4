// Prints the library's quadrature rules (wavebem_gb300/csrc/quadrature_rules.h)
// for tests/test_quadrature_rules.py: "G n" then n lines "x w" for the
// Gauss-Legendre rules, "S n v" then 2 n^2 lines "x y w" for the
// vertex-singular rules, n = 1..8, v = 0..3.
#include <cstdio>
#include "quadrature_rules.h"

int main() {
  std::vector<double> x, y, w;
  for (int n = 1; n <= 8; ++n) {
    wbem::quad::gauss_legendre01(n, x, w);
    std::printf("G %d\n", n);
    for (int i = 0; i < n; ++i) std::printf("%.17g %.17g\n", x[i], w[i]);
  }
  for (int n = 1; n <= 8; ++n)
    for (int v = 0; v < 4; ++v) {
      wbem::quad::vertex_singular_points(n, v, x, y, w);
      std::printf("S %d %d\n", n, v);
      for (size_t k = 0; k < x.size(); ++k) std::printf("%.17g %.17g %.17g\n", x[k], y[k], w[k]);
    }
  return 0;
}
