"""Python restatement of shell cutoff radii, micro-batch screening and task
merging -- TEST INFRASTRUCTURE ONLY (the checker for the library's task list).

Follows:
  include/gauxc/util/gau_rad_eval.hpp:32-71     (cutoff radius walk)
  include/gauxc/util/geometry.hpp:36-49         (cube_sphere_intersect)
  src/load_balancer/host/petite_replicated_load_balancer.cxx:31-65
  src/load_balancer/host/replicated_host_load_balancer.cxx:22-193
Scalar math uses Python floats (C doubles through libm), so results are
bit-comparable with the C++ implementation.
"""
import math


def rad_eval(l, alpha, abscoeff, r):
    s = 0.0
    r2 = r * r
    for a, c in zip(alpha, abscoeff):
        s += c * math.exp(-a * r2)
    return math.pow(r, l) * s


def cutoff_radius(l, alpha, coeff, tol):
    if tol <= 0.0:
        return math.inf
    log_tol = -math.log(tol)
    r = 0.0
    for a in alpha:
        r = max(r, math.sqrt((log_tol + math.log(a) / 2.0) / a))
    ac = [abs(c) for c in coeff]
    v = rad_eval(l, alpha, ac, r)
    step = 0.01
    if v > tol:
        while v > tol:
            r = r + step
            v = rad_eval(l, alpha, ac, r)
    else:
        while v < tol:
            r = r - step
            v = rad_eval(l, alpha, ac, r)
        r = r + step
    return r


def cube_sphere_intersect(lo, up, c, rad):
    d = rad * rad
    for i in range(3):
        r = 0.0
        if c[i] < lo[i]:
            r = lo[i] - c[i]
        elif c[i] > up[i]:
            r = c[i] - up[i]
        d -= r * r
        if d < 0.0:
            return False
    return True


def screen(lo, up, origins, radii):
    return [s for s in range(len(radii)) if cube_sphere_intersect(lo, up, origins[s], radii[s])]


def make_tasks(atoms, atomic_grids, origins, radii, sizes, dist_nearest):
    """atoms: [(Z,x,y,z)]; atomic_grids: Z -> (points[n,3], weights[n], batches[nb,2]).
    Returns merged tasks sorted by (iParent, shell_list) as dicts."""
    cand = []
    for iat, (Z, x, y, z) in enumerate(atoms):
        pts, w, br = atomic_grids[Z]
        c = (x, y, z)
        for b0, b1 in br:
            if b1 == b0:
                continue
            P = [(p[0] + c[0], p[1] + c[1], p[2] + c[2]) for p in pts[b0:b1]]
            lo = [min(p[a] for p in P) for a in range(3)]
            up = [max(p[a] for p in P) for a in range(3)]
            sl = screen(lo, up, origins, radii)
            if not sl:
                continue
            cand.append(dict(iParent=iat, points=P, weights=list(w[b0:b1]), shell_list=sl,
                             nbe=sum(sizes[s] for s in sl), dist_nearest=dist_nearest[iat]))
    cand.sort(key=lambda t: (t["iParent"], t["shell_list"]))
    merged = []
    for t in cand:
        if merged and merged[-1]["iParent"] == t["iParent"] and merged[-1]["shell_list"] == t["shell_list"]:
            merged[-1]["points"] += t["points"]
            merged[-1]["weights"] += t["weights"]
        else:
            merged.append(t)
    for t in merged:
        t["npts"] = len(t["weights"])
    return merged


def dist_nearest(atoms):
    out = []
    for i, a in enumerate(atoms):
        d = math.inf
        for j, b in enumerate(atoms):
            if i != j:
                dx, dy, dz = a[1] - b[1], a[2] - b[2], a[3] - b[3]
                d = min(d, math.sqrt(dx * dx + dy * dy + dz * dz))
        out.append(d)
    return out
