// Shell normalization, shell cutoff radii, basis offsets and molecular metadata.
#include "core.hpp"

#include <cmath>
#include <limits>
#include <numeric>

namespace gb300 {

namespace {
// (2l-1)!!, with (-1)!! = 1
double odd_double_factorial(int l) {
  double r = 1.;
  for (int k = 2 * l - 1; k > 1; k -= 2) r *= k;
  return r;
}

// R(r) = r^l sum_i |c_i| exp(-a_i r^2)   (gau_rad_eval.hpp:20-28)
double radial_abs(int l, int n, const double* a, const double* absc, double r) {
  double s = 0.;
  const double r2 = r * r;
  for (int i = 0; i < n; ++i) s += absc[i] * std::exp(-a[i] * r2);
  return std::pow(r, l) * s;
}
}  // namespace

// Normalization of a contracted shell (include/gauxc/shell.hpp:72-109):
// primitive factors N_i = sqrt( 2^l (2a_i)^(l+3/2) / (pi^(3/2) (2l-1)!!) ),
// then one overall factor so that the contracted radial self-overlap is 1.
void Shell::normalize() {
  if (l > 15) throw error("Shell::normalize: l > 15");
  const double sqrt_pi3 = 5.56832799683170784528481798212;
  const double df = std::pow(2, l) / sqrt_pi3 / odd_double_factorial(l);
  for (int i = 0; i < nprim; ++i) {
    if (alpha[i] < 0.) throw error("negative exponent");
    if (alpha[i] != 0.) {
      const double ta = 2 * alpha[i];
      coeff[i] *= std::sqrt(df * (std::pow(ta, l + 1) * std::sqrt(ta)));
    }
  }
  double s = 0.;
  for (int i = 0; i < nprim; ++i)
    for (int j = 0; j <= i; ++j) {
      const double g = alpha[i] + alpha[j];
      s += (i == j ? 1 : 2) * coeff[i] * coeff[j] / (df * (std::pow(g, l + 1) * std::sqrt(g)));
    }
  const double f = 1. / std::sqrt(s);
  for (int i = 0; i < nprim; ++i) coeff[i] *= f;
}

// Cutoff radius: start at the largest primitive estimate
// sqrt((-ln tol + ln(a)/2)/a) and walk in steps of 0.01 bohr until the
// absolute radial envelope crosses `tol` (gau_rad_eval.hpp:32-71).
void Shell::compute_cutoff() {
  if (tol <= 0.) {
    cutoff_radius = std::numeric_limits<double>::infinity();
    return;
  }
  const double log_tol = -std::log(tol);
  double r = 0.;
  for (int i = 0; i < nprim; ++i) {
    const double pc = std::sqrt((log_tol + std::log(alpha[i]) / 2.) / alpha[i]);
    r = std::max(r, pc);
  }
  double absc[kMaxPrim];
  for (int i = 0; i < nprim; ++i) absc[i] = std::abs(coeff[i]);
  double v = radial_abs(l, nprim, alpha, absc, r);
  const double step = 0.01;
  if (v > tol) {
    while (v > tol) {
      r = r + step;
      v = radial_abs(l, nprim, alpha, absc, r);
    }
  } else {
    while (v < tol) {
      r = r - step;
      v = radial_abs(l, nprim, alpha, absc, r);
    }
    r = r + step;
  }
  cutoff_radius = r;
}

void BasisSet::finalize() {
  shell_offs.resize(shells.size());
  nbf = 0;
  max_l = 0;
  for (size_t i = 0; i < shells.size(); ++i) {
    shell_offs[i] = nbf;
    nbf += shells[i].size();
    max_l = std::max(max_l, (int)shells[i].l);
  }
}

MolMeta::MolMeta(const Molecule& mol) : natoms(mol.size()) {
  rab.assign(natoms * natoms, 0.);
  for (size_t i = 0; i < natoms; ++i) {
    for (size_t j = 0; j < i; ++j) {
      const double dx = mol[i].x - mol[j].x;
      const double dy = mol[i].y - mol[j].y;
      const double dz = mol[i].z - mol[j].z;
      const double d = std::sqrt(dx * dx + dy * dy + dz * dz);
      rab[i + j * natoms] = d;
      rab[j + i * natoms] = d;
    }
  }
  dist_nearest.assign(natoms, std::numeric_limits<double>::infinity());
  for (size_t i = 0; i < natoms; ++i)
    for (size_t j = 0; j < natoms; ++j)
      if (i != j && rab[i * natoms + j] < dist_nearest[i]) dist_nearest[i] = rab[i * natoms + j];
}

}  // namespace gb300
