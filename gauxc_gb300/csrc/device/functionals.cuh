// Spin-unpolarized LDA / GGA exchange-correlation kernels, FP64.
//
// Inputs are the total density rho and sigma = |grad rho|^2.  Outputs are the
// energy per particle eps, vrho = d(rho eps)/d rho and vsigma = d(rho eps)/d sigma,
// the quantities the reference obtains from ExchCXX (unpolarized
// eval_exc_vxc, called from src/xc_integrator/local_work_driver/device/
// scheme1_base.cxx:1358-1431).  Formulas are from the original papers:
//   Slater exchange         : eps_x = -(3/4) (3 rho/pi)^(1/3)
//   VWN correlation         : Vosko, Wilk, Nusair, Can. J. Phys. 58, 1200 (1980),
//                             paramagnetic interpolation formula, RPA-fit parameters
//   PW92 correlation        : Perdew, Wang, PRB 45, 13244 (1992), unpolarized G(rs)
//   PBE exchange/correlation: Perdew, Burke, Ernzerhof, PRL 77, 3865 (1996)
// Derivatives are written out analytically below.
//
// Density cutoffs (a project choice; the third-party kernels' own small-density
// behaviour is not part of the reference tree): a kernel contributes nothing
// where rho <= its threshold -- 1e-15 for Slater, VWN5 and PBE exchange,
// 1e-12 for PBE correlation.
#pragma once
#include <cmath>

#ifndef GB300_HD
#define GB300_HD __host__ __device__
#endif

namespace gb300 {

enum XCKind : int { kXC_SVWN5 = 0, kXC_PBE = 1 };

struct XCFunctionalDesc {
  int kind;        // XCKind
  double x_scale;  // exchange scale (0.75 for PBE0, 1 otherwise)
  double c_scale;  // correlation scale
  double kappa;    // PBE exchange kappa
  double mu;       // PBE exchange mu
  int is_gga;
  int polarized = 0;  // spin-polarized (UKS) functional
};

constexpr double kRhoTolX = 1e-15;
constexpr double kRhoTolVWN = 1e-15;
constexpr double kRhoTolPBEc = 1e-12;
constexpr double kPi = 3.14159265358979323846;

// rho*eps_x = Cx rho^(4/3), Cx = -(3/4)(3/pi)^(1/3)
GB300_HD inline void slater_x(double rho, double& e, double& vr) {
  const double Cx = -0.73855876638202240588;  // -(3/4)(3/pi)^(1/3)
  const double r13 = cbrt(rho);
  e = Cx * r13;                  // per particle
  vr = (4.0 / 3.0) * Cx * r13;
}

// VWN paramagnetic correlation: x = sqrt(rs), X(x) = x^2 + b x + c,
// Q = sqrt(4c - b^2).  The reference's SVWN5 kernel uses the RPA-fit
// parameter set below (its benzene SVWN5 goldens are reproduced with it to
// 1e-12; the Ceperley-Alder fit differs by 0.8 Eh there).
GB300_HD inline void vwn5_c(double rho, double& e, double& vr) {
  const double A = 0.0310907, b = 13.0720, c = 42.7198, x0 = -0.409286;
  const double Q = sqrt(4.0 * c - b * b);
  const double X0 = x0 * x0 + b * x0 + c;
  const double rs = cbrt(3.0 / (4.0 * kPi * rho));
  const double x = sqrt(rs);
  const double X = x * x + b * x + c;
  const double tx = 2.0 * x + b;
  const double at = atan(Q / tx);
  const double bx0 = b * x0 / X0;
  const double ec = A * (log(x * x / X) + (2.0 * b / Q) * at -
                         bx0 * (log((x - x0) * (x - x0) / X) + (2.0 * (b + 2.0 * x0) / Q) * at));
  const double den = tx * tx + Q * Q;
  const double dedx = A * (2.0 / x - tx / X - 4.0 * b / den -
                           bx0 * (2.0 / (x - x0) - tx / X - 4.0 * (b + 2.0 * x0) / den));
  e = ec;
  vr = ec - (x / 6.0) * dedx;
}

// PW92 unpolarized correlation (parameter set used by PBE correlation).
GB300_HD inline void pw92_c(double rs, double& ec, double& dec_drs) {
  const double A = 0.0310907, a1 = 0.21370, b1 = 7.5957, b2 = 3.5876, b3 = 1.6382, b4 = 0.49294;
  const double srs = sqrt(rs);
  const double Q1 = 2.0 * A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs);
  const double Q1p = A * (b1 / srs + 2.0 * b2 + 3.0 * b3 * srs + 4.0 * b4 * rs);
  const double lg = log(1.0 + 1.0 / Q1);
  ec = -2.0 * A * (1.0 + a1 * rs) * lg;
  dec_drs = -2.0 * A * a1 * lg + 2.0 * A * (1.0 + a1 * rs) * Q1p / (Q1 * Q1 + Q1);
}

// PBE exchange: rho eps = Cx rho^(4/3) F(s^2), s^2 = sigma / (4 (3 pi^2)^(2/3) rho^(8/3))
GB300_HD inline void pbe_x(double rho, double sigma, double kappa, double mu, double& e,
                           double& vr, double& vs) {
  const double Cx = -0.73855876638202240588;
  const double c2 = 4.0 * 9.5707800006273119;  // 4 (3 pi^2)^(2/3)
  const double r13 = cbrt(rho);
  const double r43 = rho * r13;
  const double r83 = r43 * r43;
  const double s2 = sigma / (c2 * r83);
  const double den = kappa + mu * s2;
  const double F = 1.0 + kappa - kappa * kappa / den;
  const double Fp = kappa * kappa * mu / (den * den);  // dF/ds2
  e = Cx * r13 * F;
  vr = (4.0 / 3.0) * Cx * r13 * F - (8.0 / 3.0) * Cx * r13 * s2 * Fp;
  vs = Cx * Fp / (c2 * r43);
}

// PBE correlation (phi = 1): eps = ec(rs) + H(ec, t^2),
// t^2 = sigma pi / (16 (3 pi^2)^(1/3) rho^(7/3)).
GB300_HD inline void pbe_c(double rho, double sigma, double& e, double& vr, double& vs) {
  const double beta = 0.06672455060314922;
  const double gamma = 0.031090690869654895;  // (1 - ln 2)/pi^2
  const double y = beta / gamma;
  const double rs = cbrt(3.0 / (4.0 * kPi * rho));
  double ec, decdrs;
  pw92_c(rs, ec, decdrs);
  const double ct = kPi / (16.0 * 3.0936677262801359);  // pi / (16 (3 pi^2)^(1/3))
  const double r13 = cbrt(rho);
  const double r73 = rho * rho * r13;
  const double dt2ds = ct / r73;
  const double t2 = sigma * dt2ds;
  const double E = exp(-ec / gamma);
  const double A = y / (E - 1.0);
  const double At2 = A * t2;
  const double N = 1.0 + At2;
  const double D = 1.0 + At2 + At2 * At2;
  const double Phi = y * t2 * N / D;
  const double H = gamma * log(1.0 + Phi);
  const double g1 = gamma / (1.0 + Phi);
  const double D2 = D * D;
  // dPhi/dt2 = y (N D + t2 A D - t2 N (A + 2 A^2 t2)) / D^2
  const double dPhi_dt2 = y * (N * D + t2 * A * D - t2 * N * (A + 2.0 * A * At2)) / D2;
  // dPhi/dA = y t2 (t2 D - N (t2 + 2 A t2^2)) / D^2
  const double dPhi_dA = y * t2 * (t2 * D - N * (t2 + 2.0 * At2 * t2)) / D2;
  const double dH_dt2 = g1 * dPhi_dt2;
  const double dH_dA = g1 * dPhi_dA;
  const double dA_dec = A * A * E / (y * gamma);
  e = ec + H;
  vr = ec + H - (rs / 3.0) * decdrs * (1.0 + dH_dA * dA_dec) - (7.0 / 3.0) * t2 * dH_dt2;
  vs = rho * dH_dt2 * dt2ds;
}

// Full functional at one point.
GB300_HD inline void xc_eval_unpol(const XCFunctionalDesc& f, double rho, double sigma,
                                   double& eps, double& vrho, double& vsigma) {
  eps = 0.;
  vrho = 0.;
  vsigma = 0.;
  if (f.kind == kXC_SVWN5) {
    double e, v;
    if (rho > kRhoTolX) {
      slater_x(rho, e, v);
      eps += f.x_scale * e;
      vrho += f.x_scale * v;
    }
    if (rho > kRhoTolVWN) {
      vwn5_c(rho, e, v);
      eps += f.c_scale * e;
      vrho += f.c_scale * v;
    }
  } else {
    double e, v, s;
    if (rho > kRhoTolX) {
      pbe_x(rho, sigma, f.kappa, f.mu, e, v, s);
      eps += f.x_scale * e;
      vrho += f.x_scale * v;
      vsigma += f.x_scale * s;
    }
    if (rho > kRhoTolPBEc) {
      pbe_c(rho, sigma, e, v, s);
      eps += f.c_scale * e;
      vrho += f.c_scale * v;
      vsigma += f.c_scale * s;
    }
  }
}

}  // namespace gb300
