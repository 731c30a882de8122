"""Generate ``lebedev_orbits.inc``: Lebedev-Laikov sphere rules as symmetry orbits.

The published Lebedev-Laikov rules are octahedrally symmetric; every rule is a
union of orbits of six kinds (a1, a2, a3, b_k, c_k, d_k in Lebedev's notation).
This script reads the tabulated rules from ``scipy.integrate.lebedev_rule``,
identifies each orbit by the sorted absolute values of its coordinates and
stores one representative + weight per orbit.  ``molgrid.cxx`` expands the
orbits back into points with all sign/permutation images, in a fixed order.

Weights are stored as they come from the table (they sum to 4*pi).

Run from this directory:  python gen_lebedev.py > lebedev_orbits.inc
"""
import numpy as np
from scipy.integrate import lebedev_rule

ORDERS = [3, 5, 7, 9, 11, 13, 15, 17, 19, 21, 23, 25, 27, 29, 31, 35, 41,
          47, 53, 59, 65]


def orbits(order):
    x, w = lebedev_rule(order)
    x = x.T
    seen = {}
    for p, wt in zip(x, w):
        a = np.sort(np.abs(p))[::-1]
        key = tuple(np.round(a, 12))
        if key not in seen:
            seen[key] = [a, wt, 0]
        seen[key][2] += 1
    out = []
    for key, (a, wt, cnt) in seen.items():
        out.append((a, wt, cnt))
    out.sort(key=lambda t: (-t[2], tuple(t[0])))
    return x.shape[0], out


def main():
    print("// Generated by gen_lebedev.py from the tabulated Lebedev-Laikov rules.")
    print("// {order, npts, norbits, offset into kLebedevOrbitData}")
    rows, data = [], []
    for o in ORDERS:
        npts, orb = orbits(o)
        rows.append((o, npts, len(orb), len(data)))
        tot = 0
        for a, wt, cnt in orb:
            data.append((a[0], a[1], a[2], wt, cnt))
            tot += cnt
        assert tot == npts, (o, tot, npts)
    print("static const int kLebedevRules[][4] = {")
    for r in rows:
        print("  {%d, %d, %d, %d}," % r)
    print("};")
    print("// {|c0| >= |c1| >= |c2|, weight, orbit size}")
    print("static const double kLebedevOrbitData[][5] = {")
    for a0, a1, a2, wt, cnt in data:
        print("  {%.17g, %.17g, %.17g, %.17g, %d}," % (a0, a1, a2, wt, cnt))
    print("};")


if __name__ == "__main__":
    main()
