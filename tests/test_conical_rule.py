"""CPU: the conical product rules of the double-float quadrature (host
construction in csrc/gb_rules.h, compiled here with g++): Gauss-Jacobi nodes
and weights against scipy, and exactness of the n x n rule over the
element's reference triangle for every monomial z^a e^b with a + b <= 2n - 1
against the reference's three sub-quadrangle map with a 40-point rule."""
import os
import subprocess

import numpy as np
import pytest
from numpy.polynomial.legendre import leggauss

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bem3_emf_b2_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "gb_rules.h"
int main(int argc, char** argv) {
  const int n = atoi(argv[1]);
  double xl[16], wl[16], xj[16], wj[16], z[64], e[64], w[64];
  for (int i = 0; i < n; i++) { xl[i] = atof(argv[2 + i]); wl[i] = atof(argv[2 + n + i]); }
  gb_gauss_jacobi01(n, xj, wj);
  for (int i = 0; i < n; i++) printf("J %.17g %.17g\n", xj[i], wj[i]);
  gb_conical_rule(n, xl, wl, z, e, w);
  for (int q = 0; q < n * n; q++) printf("P %.17g %.17g %.17g\n", z[q], e[q], w[q]);
  return 0;
}
"""


def _subquad(n):
    x, w = leggauss(n)
    X, Y = [a.ravel() for a in np.meshgrid(x, x, indexing="ij")]
    W = np.outer(w, w).ravel() * (1 + 0.25 * X + 0.25 * Y)
    s3 = np.sqrt(3.0)
    zs = [0.125 * (3 + 2 * X + 2 * Y + X * Y), 0.0625 * (-3 + X - 5 * Y - X * Y), 0.0625 * (-3 - 5 * X + Y - X * Y)]
    es = [0.125 * s3 * (-X + Y), 0.0625 * s3 * (3 + 3 * X + Y + X * Y), 0.0625 * s3 * (-3 - X - 3 * Y - X * Y)]
    return np.concatenate(zs), np.concatenate(es), np.concatenate([W] * 3)


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("rules")
    src = d / "rules.cpp"
    src.write_text(DRIVER)
    exe = str(d / "rules")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("n", [5, 6, 7, 8])
def test_conical_rule(driver, n):
    from scipy.special import roots_jacobi
    xl, wl = leggauss(n)
    out = subprocess.run([driver, str(n)] + ["%.17g" % v for v in xl] + ["%.17g" % v for v in wl],
                         check=True, capture_output=True, text=True).stdout.split("\n")
    J = np.array([[float(t) for t in l.split()[1:]] for l in out if l.startswith("J")])
    P = np.array([[float(t) for t in l.split()[1:]] for l in out if l.startswith("P")])
    xr, wr = roots_jacobi(n, 0.0, 1.0)
    o = np.argsort(J[:, 0])
    assert np.max(np.abs(J[o, 0] - np.sort(xr))) < 1e-14
    assert np.max(np.abs(J[o, 1] - wr[np.argsort(xr)])) < 1e-14
    z, e, w = P.T
    assert abs(w.sum() - 12.0) < 1e-13
    zr, er, wr2 = _subquad(40)
    worst = 0.0
    for a in range(2 * n):
        for b in range(2 * n - a):
            ref = np.sum(wr2 * zr ** a * er ** b)
            got = np.sum(w * z ** a * e ** b)
            worst = max(worst, abs(got - ref) / max(1.0, abs(ref)))
    assert worst < 1e-13, worst
