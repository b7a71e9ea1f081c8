// gb_rules.h -- host construction of the conical product rules over a
// triangle that the double-float quadrature uses for far triangle pairs
// (gb_quad_df.cuh uploads them).  Plain C++, no CUDA: the CPU tests compile
// it directly.
//
// The element's reference triangle has vertices V0 = (1, 0),
// V1 = (-1/2, sqrt(3)/2), V2 = (-1/2, -sqrt(3)/2) in the parameters (z, e)
// (the reference's linear triangle map, circumradius 1 about the centroid).
// It is the image of the unit square under (s, t) -> V0 + s (V1 - V0) +
// s t (V2 - V1), whose Jacobian is proportional to s (Stroud's conical
// product): Gauss-Jacobi nodes for the weight s in s, Gauss-Legendre in t;
// n x n points integrate polynomials of degree 2n - 1 in (z, e) exactly.
// The weights are scaled to the total of the reference's three
// sub-quadrangle rule (12), so the two rules share every other factor.
#pragma once
#include <cmath>

// Gauss-Jacobi nodes and weights on [-1, 1] for the weight (1 + x) (Jacobi
// alpha = 0, beta = 1), n <= 16: Newton on P_n from its three-term
// recurrence, with the roots already found divided out;
// w_i = 4 / ((1 - x_i^2) P_n'(x_i)^2)
static inline void gb_gauss_jacobi01(int n, double* xo, double* wo) {
  auto jac = [n](long double x, long double* dp) {
    const long double a = 0.0L, b = 1.0L;
    long double pm = 1.0L, p = ((a + b + 2.0L) * x + (a - b)) / 2.0L;
    for (int m = 2; m <= n; m++) {
      const long double c1 = 2.0L * m * (m + a + b) * (2.0L * m + a + b - 2.0L);
      const long double c2 = (2.0L * m + a + b - 1.0L) * (a * a - b * b);
      const long double c3 = (2.0L * m + a + b - 2.0L) * (2.0L * m + a + b - 1.0L) * (2.0L * m + a + b);
      const long double c4 = 2.0L * (m + a - 1.0L) * (m + b - 1.0L) * (2.0L * m + a + b);
      const long double pn = ((c2 + c3 * x) * p - c4 * pm) / c1;
      pm = p;
      p = pn;
    }
    *dp = (n * ((a - b) - (2.0L * n + a + b) * x) * p + 2.0L * (n + a) * (n + b) * pm) / ((2.0L * n + a + b) * (1.0L - x * x));
    return p;
  };
  long double r[16];
  for (int k = 0; k < n; k++) {
    long double x = std::cos(3.14159265358979323846264338327950288L * (k + 0.75L) / (n + 0.5L));
    for (int it = 0; it < 100; it++) {
      long double dp = 0.0L;
      const long double p = jac(x, &dp);
      long double sdef = 0.0L;
      for (int j = 0; j < k; j++) sdef += 1.0L / (x - r[j]);
      const long double dx = p / (dp - p * sdef);
      x -= dx;
      if (std::fabs(dx) < 1e-19L) break;
    }
    r[k] = x;
  }
  for (int k = 0; k < n; k++) {
    long double dp = 0.0L;
    jac(r[k], &dp);
    xo[k] = (double)r[k];
    wo[k] = (double)(4.0L / ((1.0L - r[k] * r[k]) * dp * dp));
  }
}

// The n x n conical rule (n <= 8): points (z, e) and weights, point i n + j
// from the i-th Gauss-Jacobi node s_i and the j-th of the given n-point
// Gauss-Legendre rule (xl, wl on [-1, 1]) as t_j = (1 + xl_j) / 2:
// z = 1 - 3 s / 2, e = sqrt(3) s (1/2 - t), weight 24 (wj_i / 4) (wl_j / 2)
// (int_0^1 f(s) s ds = sum wj_i / 4 f(s_i) with s_i = (1 + xj_i) / 2).
static inline void gb_conical_rule(int n, const double* xl, const double* wl, double* z, double* e, double* w) {
  double xj[16], wj[16];
  gb_gauss_jacobi01(n, xj, wj);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      const double sv = 0.5 * (1.0 + xj[i]), tv = 0.5 * (1.0 + xl[j]);
      z[i * n + j] = 1.0 - 1.5 * sv;
      e[i * n + j] = std::sqrt(3.0) * sv * (0.5 - tv);
      w[i * n + j] = 24.0 * (0.25 * wj[i]) * (0.5 * wl[j]);
    }
}
