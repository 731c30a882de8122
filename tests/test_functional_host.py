"""The device functional code (functionals.cuh, compiled here for the host)
against the oracle's dual-number derivatives -- checks the hand-derived
vrho / vsigma without a GPU."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle

HARNESS = r"""
#define GB300_HD
#include "functionals.cuh"
extern "C" void dev_xc(int kind, double xs, double cs, double kappa, double mu, int gga, long n,
                       const double* rho, const double* sigma, double* eps, double* vr, double* vs) {
  gb300::XCFunctionalDesc f{kind, xs, cs, kappa, mu, gga};
  for (long i = 0; i < n; ++i) gb300::xc_eval_unpol(f, rho[i], sigma[i], eps[i], vr[i], vs[i]);
}
"""


@pytest.fixture(scope="module")
def devxc():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    inc = os.path.join(root, "gauxc_gb300", "csrc", "device")
    d = tempfile.mkdtemp()
    src = os.path.join(d, "h.cpp")
    so = os.path.join(d, "h.so")
    open(src, "w").write(HARNESS)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", inc, src, "-o", so],
                   check=True)
    return ctypes.CDLL(so)


@pytest.mark.parametrize("name", ["SVWN5", "PBE", "REVPBE", "PBE0"])
def test_device_functional_matches_oracle(devxc, name):
    rng = np.random.default_rng(7)
    # densities over the range the grids see, reduced gradients s in [0, 8]
    rho = np.concatenate([10 ** rng.uniform(-10, 3, 4000), [0.0, 1e-16, 1e-13, 2e-12]])
    s = rng.uniform(0.0, 8.0, len(rho))
    sigma = s * s * 4.0 * (3 * np.pi ** 2) ** (2 / 3) * rho ** (8 / 3)
    sigma[-4:] = 0.0
    kind, xs, cs, kappa, mu, gga = oracle.FUNCTIONALS[name]
    eps, vr, vs = (np.zeros_like(rho) for _ in range(3))
    dp = ctypes.POINTER(ctypes.c_double)
    devxc.dev_xc(kind, ctypes.c_double(xs), ctypes.c_double(cs), ctypes.c_double(kappa),
                 ctypes.c_double(mu), gga, ctypes.c_long(len(rho)), rho.ctypes.data_as(dp),
                 sigma.ctypes.data_as(dp), eps.ctypes.data_as(dp), vr.ctypes.data_as(dp),
                 vs.ctypes.data_as(dp))
    e2, v2, s2 = oracle.functional(name, rho, sigma)
    np.testing.assert_allclose(eps, e2, rtol=2e-13, atol=1e-300)
    np.testing.assert_allclose(vr, v2, rtol=1e-11, atol=1e-300)
    if gga:
        # below rho ~ 1e-10 vsigma is the difference of ~1e14-sized exchange and
        # correlation terms; only the regular range is compared
        m = rho > 1e-10
        np.testing.assert_allclose(vs[m], s2[m], rtol=1e-9, atol=1e-300)


HARNESS_POL = r"""
#define GB300_HD
#include "functionals_pol.cuh"
extern "C" void dev_xc_pol(int kind, double xs, double cs, double kappa, double mu, int gga,
                           long n, const double* rho, const double* sigma, double* eps,
                           double* vr, double* vs) {
  gb300::XCFunctionalDesc f{kind, xs, cs, kappa, mu, gga};
  for (long i = 0; i < n; ++i)
    gb300::xc_eval_pol(f, rho[2 * i], rho[2 * i + 1], sigma[3 * i], sigma[3 * i + 1],
                       sigma[3 * i + 2], eps[i], vr + 2 * i, vs + 3 * i);
}
"""


@pytest.fixture(scope="module")
def devxc_pol():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    inc = os.path.join(root, "gauxc_gb300", "csrc", "device")
    d = tempfile.mkdtemp()
    src = os.path.join(d, "hp.cpp")
    so = os.path.join(d, "hp.so")
    open(src, "w").write(HARNESS_POL)
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", inc, src, "-o", so],
                   check=True)
    return ctypes.CDLL(so)


@pytest.mark.parametrize("name", ["SVWN5", "PBE", "REVPBE", "PBE0"])
def test_device_polarized_functional_matches_oracle(devxc_pol, name):
    """functionals_pol.cuh (host build) against the oracle's polarized
    functionals over spin polarizations from closed shell to fully polarized."""
    rng = np.random.default_rng(9)
    n = 3000
    rho = 10 ** rng.uniform(-9, 3, n)
    zeta = np.concatenate([rng.uniform(-1, 1, n - 4), [0.0, 1.0, -1.0, 0.999999]])
    ra, rb = 0.5 * rho * (1 + zeta), 0.5 * rho * (1 - zeta)
    c = 4.0 * (3 * np.pi ** 2) ** (2 / 3)
    saa = rng.uniform(0, 4, n) ** 2 * c * (2 * ra) ** (8 / 3) / 4
    sbb = rng.uniform(0, 4, n) ** 2 * c * (2 * rb) ** (8 / 3) / 4
    sab = rng.uniform(-1, 1, n) * np.sqrt(saa * sbb)
    R = np.ascontiguousarray(np.stack([ra, rb], 1))
    S = np.ascontiguousarray(np.stack([saa, sab, sbb], 1))
    kind, xs, cs, kappa, mu, gga = oracle.FUNCTIONALS[name]
    eps, vr, vs = np.zeros(n), np.zeros((n, 2)), np.zeros((n, 3))
    dp = ctypes.POINTER(ctypes.c_double)
    devxc_pol.dev_xc_pol(kind, ctypes.c_double(xs), ctypes.c_double(cs), ctypes.c_double(kappa),
                         ctypes.c_double(mu), gga, ctypes.c_long(n), R.ctypes.data_as(dp),
                         S.ctypes.data_as(dp), eps.ctypes.data_as(dp), vr.ctypes.data_as(dp),
                         vs.ctypes.data_as(dp))
    e2, v2, s2 = oracle.functional_pol(name, R, S if gga else None)
    np.testing.assert_allclose(eps, e2, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(vr, v2, rtol=1e-10, atol=1e-300)
    if gga:
        m = rho > 1e-8
        np.testing.assert_allclose(vs[m], s2[m], rtol=1e-9, atol=1e-300)
