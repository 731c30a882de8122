// Spin-polarized LDA / GGA kernels (UKS), FP64, with first derivatives by
// forward-mode dual numbers over the five inputs (rho_a, rho_b, sigma_aa,
// sigma_ab, sigma_bb).  The reference obtains these from ExchCXX's polarized
// eval_exc_vxc (same call sites as the unpolarized kernels).  Formulas:
//   Slater exchange   spin scaling e_x[a, b] = (e_x[2 rho_a] + e_x[2 rho_b]) / 2
//   VWN correlation   RPA-fit paramagnetic (P) and ferromagnetic (F) forms of
//                     Vosko, Wilk, Nusair (1980) joined by the exchange-like
//                     interpolation e = e_P + f(zeta) (e_F - e_P),
//                     f(z) = ((1 + z)^(4/3) + (1 - z)^(4/3) - 2) / (2^(4/3) - 2);
//                     this form reproduces the reference's UKS SVWN5 golden
//                     (cytosine cc-pVDZ; the unpolarized limit is vwn5_c)
//   PBE exchange      spin scaling of pbe_x: (e_x[2 rho_a, 4 s_aa] + e_x[2 rho_b, 4 s_bb]) / 2
//   PBE correlation   PW92 e_c(rs, zeta) (Perdew, Wang 1992, the three fits with
//                     the A values of pw92_c) plus H(rs, zeta, t) of PBE 1996,
//                     phi = ((1 + z)^(2/3) + (1 - z)^(2/3)) / 2,
//                     t^2 = (s_aa + 2 s_ab + s_bb) / (4 phi^2 ks^2 rho^2)
// Cutoffs follow the unpolarized kernels: nothing for rho_a + rho_b at or
// below 1e-15 (PBE correlation 1e-12), a spin channel's exchange vanishes at
// rho_s <= 5e-16, and |zeta| is held at or below 1 - 1e-12.
#pragma once
#include <cmath>

#include "functionals.cuh"

namespace gb300 {

namespace pol {

struct D5 {
  double v, d[5];
};
GB300_HD inline D5 c5(double v) { return D5{v, {0., 0., 0., 0., 0.}}; }
GB300_HD inline D5 v5(double v, int i) {
  D5 r = c5(v);
  r.d[i] = 1.;
  return r;
}
GB300_HD inline D5 operator+(D5 a, const D5& b) {
  a.v += b.v;
  for (int i = 0; i < 5; ++i) a.d[i] += b.d[i];
  return a;
}
GB300_HD inline D5 operator-(D5 a, const D5& b) {
  a.v -= b.v;
  for (int i = 0; i < 5; ++i) a.d[i] -= b.d[i];
  return a;
}
GB300_HD inline D5 operator*(const D5& a, const D5& b) {
  D5 r{a.v * b.v, {}};
  for (int i = 0; i < 5; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
GB300_HD inline D5 operator/(const D5& a, const D5& b) {
  const double q = 1. / b.v;
  D5 r{a.v * q, {}};
  for (int i = 0; i < 5; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * q;
  return r;
}
GB300_HD inline D5 operator*(double c, D5 a) {
  a.v *= c;
  for (int i = 0; i < 5; ++i) a.d[i] *= c;
  return a;
}
GB300_HD inline D5 operator*(const D5& a, double c) { return c * a; }
GB300_HD inline D5 operator+(D5 a, double c) {
  a.v += c;
  return a;
}
GB300_HD inline D5 operator+(double c, const D5& a) { return a + c; }
GB300_HD inline D5 operator-(D5 a, double c) {
  a.v -= c;
  return a;
}
GB300_HD inline D5 operator-(double c, const D5& a) { return c5(c) - a; }
GB300_HD inline D5 operator/(const D5& a, double c) { return (1. / c) * a; }
GB300_HD inline D5 operator/(double c, const D5& a) { return c5(c) / a; }
// f(a) with f(a.v) = fv and f'(a.v) = df
GB300_HD inline D5 apply(const D5& a, double fv, double df) {
  D5 r{fv, {}};
  for (int i = 0; i < 5; ++i) r.d[i] = df * a.d[i];
  return r;
}
GB300_HD inline D5 log5(const D5& a) { return apply(a, log(a.v), 1. / a.v); }
GB300_HD inline D5 exp5(const D5& a) {
  const double e = exp(a.v);
  return apply(a, e, e);
}
GB300_HD inline D5 sqrt5(const D5& a) {
  const double q = sqrt(a.v);
  return apply(a, q, 0.5 / q);
}
GB300_HD inline D5 atan5(const D5& a) { return apply(a, atan(a.v), 1. / (1. + a.v * a.v)); }
GB300_HD inline D5 pow5(const D5& a, double p) {
  const double q = pow(a.v, p);
  return apply(a, q, p * q / a.v);
}
GB300_HD inline D5 cbrt5(const D5& a) {
  const double q = cbrt(a.v);
  return apply(a, q, q / (3. * a.v));
}

// one VWN fit at x = sqrt(rs)
GB300_HD inline D5 vwn_fit(const D5& x, double A, double b, double c, double x0) {
  const double Q = sqrt(4. * c - b * b);
  const double X0 = x0 * x0 + b * x0 + c;
  const D5 X = x * x + b * x + c;
  const D5 at = atan5(Q / (2. * x + b));
  return A * (log5(x * x / X) + (2. * b / Q) * at -
              (b * x0 / X0) * (log5((x - x0) * (x - x0) / X) + (2. * (b + 2. * x0) / Q) * at));
}

// one PW92 fit G(rs) (p = 1)
GB300_HD inline D5 pw92_fit(const D5& rs, double A, double a1, double b1, double b2, double b3,
                            double b4) {
  const D5 s = sqrt5(rs);
  const D5 den = 2. * A * (b1 * s + b2 * rs + b3 * rs * s + b4 * rs * rs);
  return -2. * A * (1. + a1 * rs) * log5(1. + 1. / den);
}

GB300_HD inline D5 zeta_of(const D5& ra, const D5& rb) {
  D5 z = (ra - rb) / (ra + rb);
  const double lim = 1. - 1e-12;
  if (z.v > lim) z = c5(lim);
  if (z.v < -lim) z = c5(-lim);
  return z;
}

GB300_HD inline D5 fzeta(const D5& z) {
  const double den = 0.5198420997897464;  // 2^(4/3) - 2
  return (pow5(1. + z, 4. / 3.) + pow5(1. - z, 4. / 3.) - 2.) / den;
}

// per-volume energy densities
GB300_HD inline D5 slater(const D5& ra, const D5& rb) {
  const double Cx = -0.73855876638202240588;  // -(3/4)(3/pi)^(1/3)
  D5 e = c5(0.);
  if (ra.v > 0.5 * kRhoTolX) {
    const D5 r2 = 2. * ra;
    e = e + 0.5 * Cx * (r2 * cbrt5(r2));
  }
  if (rb.v > 0.5 * kRhoTolX) {
    const D5 r2 = 2. * rb;
    e = e + 0.5 * Cx * (r2 * cbrt5(r2));
  }
  return e;
}

GB300_HD inline D5 vwn(const D5& ra, const D5& rb) {
  const D5 rho = ra + rb;
  const D5 rs = cbrt5(3. / (4. * kPi) / rho);
  const D5 x = sqrt5(rs);
  const D5 eP = vwn_fit(x, 0.0310907, 13.0720, 42.7198, -0.409286);
  const D5 eF = vwn_fit(x, 0.01554535, 20.1231, 101.578, -0.743294);
  return rho * (eP + fzeta(zeta_of(ra, rb)) * (eF - eP));
}

GB300_HD inline D5 pbe_x_spin(const D5& r2, const D5& s4, double kappa, double mu) {
  // unpolarized PBE exchange energy density at density r2, sigma s4
  const double Cx = -0.73855876638202240588;
  const double c2 = 4.0 * 9.5707800006273119;  // 4 (3 pi^2)^(2/3)
  const D5 r13 = cbrt5(r2);
  const D5 r43 = r2 * r13;
  const D5 s2 = s4 / (c2 * r43 * r43);
  const D5 F = 1. + kappa - kappa * kappa / (kappa + mu * s2);
  return Cx * r43 * F;
}

GB300_HD inline D5 pbe_x(const D5& ra, const D5& rb, const D5& saa, const D5& sbb, double kappa,
                         double mu) {
  D5 e = c5(0.);
  if (ra.v > 0.5 * kRhoTolX) e = e + 0.5 * pbe_x_spin(2. * ra, 4. * saa, kappa, mu);
  if (rb.v > 0.5 * kRhoTolX) e = e + 0.5 * pbe_x_spin(2. * rb, 4. * sbb, kappa, mu);
  return e;
}

GB300_HD inline D5 pbe_c(const D5& ra, const D5& rb, const D5& saa, const D5& sab,
                         const D5& sbb) {
  const double beta = 0.06672455060314922;
  const double gamma = 0.031090690869654895;  // (1 - ln 2)/pi^2
  const double fz20 = 1.709920934161365617563962776245;
  const D5 rho = ra + rb;
  const D5 rs = cbrt5(3. / (4. * kPi) / rho);
  const D5 z = zeta_of(ra, rb);
  const D5 e0 = pw92_fit(rs, 0.0310907, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294);
  const D5 e1 = pw92_fit(rs, 0.01554535, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517);
  const D5 mac = pw92_fit(rs, 0.0168869, 0.11125, 10.357, 3.6231, 0.88026, 0.49671);
  const D5 f = fzeta(z);
  const D5 z2 = z * z;
  const D5 z4 = z2 * z2;
  const D5 ec = e0 - mac * f * (1. - z4) / fz20 + (e1 - e0) * f * z4;
  const D5 phi = 0.5 * (pow5(1. + z, 2. / 3.) + pow5(1. - z, 2. / 3.));
  const D5 phi3 = phi * phi * phi;
  const D5 kf = cbrt5(3. * kPi * kPi * rho);
  const D5 ks2 = 4. * kf / kPi;
  const D5 t2 = (saa + 2. * sab + sbb) / (4. * phi * phi * ks2 * rho * rho);
  const D5 A = (beta / gamma) / (exp5(-1. * ec / (gamma * phi3)) - 1.);
  const D5 At2 = A * t2;
  const D5 H =
      gamma * phi3 * log5(1. + (beta / gamma) * t2 * (1. + At2) / (1. + At2 + At2 * At2));
  return rho * (ec + H);
}

}  // namespace pol

// Polarized functional at one point: eps per particle, vrho[2] (a, b),
// vsigma[3] (aa, ab, bb).
GB300_HD inline void xc_eval_pol(const XCFunctionalDesc& f, double rho_a, double rho_b,
                                 double s_aa, double s_ab, double s_bb, double& eps,
                                 double* vrho, double* vsigma) {
  using namespace pol;
  const D5 ra = v5(rho_a, 0), rb = v5(rho_b, 1), saa = v5(s_aa, 2), sab = v5(s_ab, 3),
           sbb = v5(s_bb, 4);
  const double rho = rho_a + rho_b;
  D5 e = c5(0.);
  if (f.kind == kXC_SVWN5) {
    if (rho > kRhoTolX) e = e + f.x_scale * slater(ra, rb);
    if (rho > kRhoTolVWN) e = e + f.c_scale * vwn(ra, rb);
  } else {
    if (rho > kRhoTolX) e = e + f.x_scale * pbe_x(ra, rb, saa, sbb, f.kappa, f.mu);
    if (rho > kRhoTolPBEc) e = e + f.c_scale * pbe_c(ra, rb, saa, sab, sbb);
  }
  eps = (rho > 0. && e.v != 0.) ? e.v / rho : 0.;
  vrho[0] = e.d[0];
  vrho[1] = e.d[1];
  vsigma[0] = e.d[2];
  vsigma[1] = e.d[3];
  vsigma[2] = e.d[4];
}

}  // namespace gb300
