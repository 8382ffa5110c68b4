// Host construction of the library's quadrature rules (plain C++, no CUDA):
// the Gauss-Legendre rule on [0, 1] and the vertex-singular rule of the unit
// square. build_quadrature (wbem_api.cu) turns them into the constant-memory
// tables; tests/quadrature_check.cpp prints them for the CPU comparison with
// the oracle's rules.
#pragma once
#include <cmath>
#include <vector>

namespace wbem {
namespace quad {

// Gauss-Legendre points and weights on [0,1] (Newton on the Legendre
// recurrence), ascending.
inline void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.resize(n);
  w.resize(n);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int i = 0; i < n; ++i) {
    long double z = cosl(pi * (i + 0.75L) / (n + 0.5L)), dp = 1;
    for (int it = 0; it < 100; ++it) {
      // P_n(z) and P_{n-1}(z) by the three-term recurrence
      long double pn = (n == 0) ? 1 : z, pm = 1;
      for (int k = 2; k <= n; ++k) {
        long double pk = ((2 * k - 1) * z * pn - (k - 1) * pm) / k;
        pm = pn;
        pn = pk;
      }
      dp = n * (z * pn - pm) / (z * z - 1);
      long double dz = pn / dp;
      z -= dz;
      if (fabsl(dz) < 1e-20L) break;
    }
    x[i] = (double)((1 - z) / 2);
    w[i] = (double)(1 / ((1 - z * z) * dp * dp));
  }
}

// Vertex-singular rule with n x n points on each of the two triangles of the
// unit square that meet at vertex v (0: (0,0), 1: (1,0), 2: (0,1), 3: (1,1)):
// the polar map x = u, y = u tan(pi t / 4) of the triangle below the
// diagonal, the 1/R weight folded into the weights (w carries the Jacobian
// (pi/4) R / cos(pi t / 4)), the other triangle its mirror x <-> y, the
// vertex-0 rule rotated onto vertex v. Point k = half n^2 + a + n b, with a
// the index along u and b along t; the weight is the same for both halves.
inline void vertex_singular_points(int n, int v, std::vector<double>& px, std::vector<double>& py,
                                   std::vector<double>& pw) {
  std::vector<double> sx, sw;
  gauss_legendre01(n, sx, sw);
  const int m = n * n;
  px.assign(2 * m, 0.0);
  py.assign(2 * m, 0.0);
  pw.assign(2 * m, 0.0);
  const double pi4 = 0.78539816339744830962;
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < n; ++a) {
      const int q = a + n * b;
      const double u = sx[a], th = pi4 * sx[b];
      const double x = u, y = u * std::tan(th);
      const double wq = sw[a] * sw[b] * pi4 / std::cos(th) * std::sqrt(x * x + y * y);
      const double pts[2][2] = {{x, y}, {y, x}};
      for (int half = 0; half < 2; ++half) {
        const double X0 = pts[half][0], Y0 = pts[half][1];
        double Xr = X0, Yr = Y0;
        if (v == 1) { Xr = 1 - Y0; Yr = X0; }
        if (v == 2) { Xr = Y0; Yr = 1 - X0; }
        if (v == 3) { Xr = 1 - X0; Yr = 1 - Y0; }
        px[half * m + q] = Xr;
        py[half * m + q] = Yr;
        pw[half * m + q] = wq;
      }
    }
}

}  // namespace quad
}  // namespace wbem
