"""Generate ``collocation_angular.inc``: angular factors of Gaussian shells, l <= 4.

For a shell with radial part R(r) = sum_k c_k exp(-a_k r^2), every basis
function is phi = R(r) * S(x, y, z) with S a homogeneous polynomial:

  * pure shells: real regular solid harmonics in Racah normalization, ordered
    m = -l..l (Helgaker, Jorgensen, Olsen, "Molecular Electronic-Structure
    Theory", eqs. 6.4.47-6.4.50).  l = 1 gives (y, z, x); l = 2 gives
    (sqrt3 xy, sqrt3 yz, (2z^2-x^2-y^2)/2, sqrt3 xz, sqrt3/2 (x^2-y^2)),
    matching the component order of the reference's device collocation
    (src/xc_integrator/local_work_driver/device/cuda/kernels/collocation/
    collocation_angular_spherical_unnorm.hpp).
  * cartesian shells: monomials x^a y^b z^c, a descending then b descending.

The gradient uses grad phi = S grad R + R grad S with grad R = r_vec * R1,
R1 = -2 sum_k a_k c_k exp(-a_k r^2).

Emitted functions (usable on host and device):
  ang_eval_<p|c>_<l>(x, y, z, R, out, stride)
  ang_grad_<p|c>_<l>(x, y, z, R, R1, f, fx, fy, fz, stride)

Run: python gen_collocation.py > collocation_angular.inc
"""
from math import comb, factorial
import sympy as sp

LMAX = 4
x, y, z = sp.symbols("x y z", real=True)


def solid_harmonic(l, m):
    am = abs(m)
    odd = 0 if m >= 0 else 1          # 2*v_m
    N = sp.sqrt(sp.Rational(2 * factorial(l + am) * factorial(l - am), 2 if m == 0 else 1)) \
        / (2 ** am * factorial(l))
    expr = 0
    for t in range((l - am) // 2 + 1):
        for u in range(t + 1):
            for two_v in range(odd, am + 1, 2):
                sign = (-1) ** (t + (two_v - odd) // 2)
                c = sp.Rational(sign) * sp.Rational(1, 4) ** t * comb(l, t) * comb(l - t, am + t) \
                    * comb(t, u) * comb(am, two_v)
                px = 2 * t + am - 2 * u - two_v
                py = 2 * u + two_v
                pz = l - 2 * t - am
                expr += c * x ** px * y ** py * z ** pz
    return sp.expand(N * expr)


def cart_list(l):
    out = []
    for a in range(l, -1, -1):
        for b in range(l - a, -1, -1):
            out.append(x ** a * y ** b * z ** (l - a - b))
    return out


def cexpr(e):
    """Straight-line C for a polynomial in x, y, z with numeric coefficients."""
    e = sp.expand(e)
    if e == 0:
        return "T(0)"
    terms = []
    for (a, b, c), coef in sp.Poly(e, x, y, z).terms():
        mono = "*".join(["x"] * a + ["y"] * b + ["z"] * c)
        cv = float(sp.N(coef, 30))
        lit = "T(%.17g)" % cv
        terms.append(lit + ("*" + mono if mono else ""))
    return " + ".join(terms)


def emit(kind, l, polys):
    tag = f"{kind}_{l}"
    # O: T* or any type whose operator[] takes a stored value (a value sink)
    print(f"template <typename T, typename O> GB300_HD inline void ang_eval_{tag}"
          f"(T x, T y, T z, T R, O out, int64_t s) {{")
    for i, p in enumerate(polys):
        print(f"  out[{i}*s] = R*({cexpr(p)});")
    print("}")
    print(f"template <typename T, typename O> GB300_HD inline void ang_grad_{tag}"
          f"(T x, T y, T z, T R, T R1, O f, O fx, O fy, O fz, int64_t s) {{")
    for i, p in enumerate(polys):
        dx, dy, dz = sp.diff(p, x), sp.diff(p, y), sp.diff(p, z)
        print(f"  {{ const T S = {cexpr(p)};")
        print(f"    f[{i}*s] = R*S;")
        print(f"    fx[{i}*s] = R1*x*S + R*({cexpr(dx)});")
        print(f"    fy[{i}*s] = R1*y*S + R*({cexpr(dy)});")
        print(f"    fz[{i}*s] = R1*z*S + R*({cexpr(dz)}); }}")
    print("}")


def main():
    print("// Generated by gen_collocation.py -- angular factors of Gaussian shells.")
    print("#pragma once")
    print("#include <cstdint>")
    print("#ifndef GB300_HD")
    print("#define GB300_HD __host__ __device__")
    print("#endif")
    for l in range(LMAX + 1):
        emit("p", l, [solid_harmonic(l, m) for m in range(-l, l + 1)])
        emit("c", l, cart_list(l))


if __name__ == "__main__":
    main()
