"""Mie series of a homogeneous dielectric sphere in a plane wave (Bohren and
Huffman, "Absorption and Scattering of Light by Small Particles", 1983,
sec. 4.4 and 4.5): coefficients a_n, b_n from Riccati-Bessel functions,
extinction and scattering cross sections and the radiation-pressure cross
section C_pr = C_ext - g C_sca.  Test helper: an analytic check of the
sphere scenes, independent of the reference's code."""
import numpy as np
from scipy import special


def coefficients(m, x):
    """a_n, b_n (n = 1..nmax) for relative index m and size parameter x."""
    nmax = int(x + 4.0 * x ** (1.0 / 3.0) + 2.0) + 10
    n = np.arange(1, nmax + 1)
    mx = m * x
    jx, djx = special.spherical_jn(n, x), special.spherical_jn(n, x, derivative=True)
    yx, dyx = special.spherical_yn(n, x), special.spherical_yn(n, x, derivative=True)
    jm, djm = special.spherical_jn(n, mx), special.spherical_jn(n, mx, derivative=True)
    psi_x, dpsi_x = x * jx, jx + x * djx
    xi_x, dxi_x = x * (jx + 1j * yx), (jx + 1j * yx) + x * (djx + 1j * dyx)
    psi_m, dpsi_m = mx * jm, jm + mx * djm
    a = (m * psi_m * dpsi_x - psi_x * dpsi_m) / (m * psi_m * dxi_x - xi_x * dpsi_m)
    b = (psi_m * dpsi_x - m * psi_x * dpsi_m) / (psi_m * dxi_x - m * xi_x * dpsi_m)
    return n, a, b


def cross_sections(n_sphere, n_host, radius, lambda0):
    """(C_ext, C_sca, C_pr) in units of lambda0^2."""
    k = 2.0 * np.pi * n_host / lambda0
    n, a, b = coefficients(n_sphere / n_host, k * radius)
    c = 2.0 * np.pi / k ** 2
    cext = c * np.sum((2 * n + 1) * np.real(a + b))
    csca = c * np.sum((2 * n + 1) * (np.abs(a) ** 2 + np.abs(b) ** 2))
    g1 = np.sum(n[:-1] * (n[:-1] + 2) / (n[:-1] + 1) * np.real(a[:-1] * np.conj(a[1:]) + b[:-1] * np.conj(b[1:])))
    g2 = np.sum((2 * n + 1) / (n * (n + 1)) * np.real(a * np.conj(b)))
    gcsca = 2.0 * c * (g1 + g2)
    return cext, csca, cext - gcsca


def radiation_force_z(n_sphere, n_host, radius, lambda0, power=1.0):
    """Force along the propagation direction on the sphere, in the units of the
    reference's force (power per unit area of the beam times n_host times
    C_pr, the speed of light being 1 in those units)."""
    return n_host * power * cross_sections(n_sphere, n_host, radius, lambda0)[2]
