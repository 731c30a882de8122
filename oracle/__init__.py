"""CPU oracle for the GB300 XC integrator -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker / baseline; the
``gauxc_gb300`` library never uses it.

``oracle.cpp`` restates the reference's FP64 host integrator (see its header
for the file:line list); ``screening.py`` restates shell cutoff radii, the
cube/sphere screen and task merging.  The restatement is pinned against the
reference's golden vectors in ``tests/golden`` (benzene SVWN5 / PBE0 EXC and
VXC, benzene SSF weights, water collocation).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "liboracle.so")

_lib = None


def build():
    """Compile oracle.cpp (g++, OpenMP) into oracle/build/liboracle.so."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp,
                    "-ldl"], check=True)
    os.replace(tmp, LIB)
    return LIB


def blas_library():
    """Path of the OpenBLAS that scipy bundles (the only CPU BLAS on these
    machines), or None."""
    import glob
    try:
        import scipy
    except ImportError:
        return None
    base = os.path.dirname(os.path.dirname(os.path.abspath(scipy.__file__)))
    for pat in ("scipy.libs/libscipy_openblas*.so*", "scipy/.libs/libscipy_openblas*.so*",
                "scipy.libs/libopenblas*.so*"):
        hits = sorted(glob.glob(os.path.join(base, pat)))
        if hits:
            return hits[0]
    return None


def lib():
    """The oracle library; its contractions use scipy's OpenBLAS when present."""
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.oracle_use_blas.restype = ctypes.c_int
        L.oracle_use_blas.argtypes = [ctypes.c_char_p]
        L.oracle_blas_active.restype = ctypes.c_int
        path = blas_library()
        if path:
            L.oracle_use_blas(path.encode())
        _lib = L
    return _lib


def blas_active():
    """True when the contractions run on a BLAS (dgemm / dsyr2k)."""
    return bool(lib().oracle_blas_active())


def _p(a, ct=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ct)) if a is not None else None


def _i32(a):
    return _p(a, ctypes.c_int32)


def _i64(a):
    return _p(a, ctypes.c_int64)


def normalize_shell(l, alpha, coeff):
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    c = np.ascontiguousarray(coeff, dtype=np.float64).copy()
    lib().oracle_normalize_shell(ctypes.c_int(l), ctypes.c_int(len(alpha)), _p(alpha), _p(c))
    return c


def ssf_weights(points, iparent, dist_nearest, coords, weights, nthreads=0):
    pts = np.ascontiguousarray(points, dtype=np.float64)
    w = np.ascontiguousarray(weights, dtype=np.float64).copy()
    ip = np.ascontiguousarray(iparent, dtype=np.int32)
    dn = np.ascontiguousarray(dist_nearest, dtype=np.float64)
    co = np.ascontiguousarray(coords, dtype=np.float64)
    lib().oracle_ssf_weights(ctypes.c_int64(len(w)), ctypes.c_int(len(co) // 3 if co.ndim == 1 else co.shape[0]),
                             _p(pts), _i32(ip), _p(dn), _p(co), _p(w), ctypes.c_int(nthreads))
    return w


class Basis:
    """Shell arrays in the layout oracle.cpp expects (coefficients normalized)."""

    def __init__(self, l, pure, nprim, alpha, coeff, origin):
        self.l = np.ascontiguousarray(l, dtype=np.int32)
        self.pure = np.ascontiguousarray(pure, dtype=np.int32)
        self.nprim = np.ascontiguousarray(nprim, dtype=np.int32)
        n = len(self.l)
        self.alpha = np.zeros((n, 32))
        self.coeff = np.zeros((n, 32))
        a = np.asarray(alpha)
        c = np.asarray(coeff)
        self.alpha[:, :a.shape[1]] = a
        self.coeff[:, :c.shape[1]] = c
        self.origin = np.ascontiguousarray(origin, dtype=np.float64).reshape(n, 3)
        self.sizes = np.where(self.pure != 0, 2 * self.l + 1, (self.l + 1) * (self.l + 2) // 2)
        self.nbf = int(self.sizes.sum())

    def args(self):
        return (ctypes.c_int(len(self.l)), _i32(self.l), _i32(self.pure), _i32(self.nprim),
                _p(self.alpha), _p(self.coeff), _p(self.origin))


def collocation(basis, points, shell_list, grad=False):
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    sl = np.ascontiguousarray(shell_list, dtype=np.int32)
    nbe = int(basis.sizes[sl].sum())
    n = len(pts)
    out = [np.zeros(n * nbe) for _ in range(4 if grad else 1)]
    ptrs = [_p(o) for o in out] + [None] * (4 - len(out))
    lib().oracle_collocation(*basis.args(), ctypes.c_int(n), _p(pts), ctypes.c_int(len(sl)),
                             _i32(sl), ctypes.c_int(1 if grad else 0), *ptrs)
    return [o.reshape(n, nbe) for o in out]


FUNCTIONALS = {
    # name: (kind, x_scale, c_scale, kappa, mu, gga)
    "SVWN5": (0, 1.0, 1.0, 0.804, 0.2195149727645171, 0),
    "PBE": (1, 1.0, 1.0, 0.804, 0.2195149727645171, 1),
    "REVPBE": (1, 1.0, 1.0, 1.245, 0.2195149727645171, 1),
    "PBE0": (1, 0.75, 1.0, 0.804, 0.2195149727645171, 1),
}


def functional(name, rho, sigma=None):
    kind, xs, cs, kappa, mu, _ = FUNCTIONALS[name.upper()]
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    sg = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64)
    eps, vr, vs = np.zeros_like(rho), np.zeros_like(rho), np.zeros_like(rho)
    lib().oracle_functional(ctypes.c_int(kind), ctypes.c_double(xs), ctypes.c_double(cs),
                            ctypes.c_double(kappa), ctypes.c_double(mu), ctypes.c_int64(len(rho)),
                            _p(rho), _p(sg), _p(eps), _p(vr), _p(vs))
    return eps, vr, vs


def eval_exc_vxc(basis, tasks, P, func, want_vxc=True, nthreads=0):
    """tasks: list of (points[n,3], weights[n], shell_list).  Returns (EXC, VXC, N_el)."""
    kind, xs, cs, kappa, mu, gga = FUNCTIONALS[func.upper()]
    pt_off = np.zeros(len(tasks) + 1, np.int64)
    sh_off = np.zeros(len(tasks) + 1, np.int64)
    for i, (p, w, s) in enumerate(tasks):
        pt_off[i + 1] = pt_off[i] + len(w)
        sh_off[i + 1] = sh_off[i] + len(s)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(t[0]).reshape(-1, 3) for t in tasks]) if tasks else np.zeros((0, 3)))
    wts = np.ascontiguousarray(np.concatenate([t[1] for t in tasks]) if tasks else np.zeros(0))
    sl = np.ascontiguousarray(np.concatenate([t[2] for t in tasks]).astype(np.int32) if tasks else np.zeros(0, np.int32))
    nbf = basis.nbf
    Pm = np.asfortranarray(P, dtype=np.float64)
    V = np.zeros((nbf, nbf), order="F") if want_vxc else None
    en = np.zeros(2)
    lib().oracle_eval_exc_vxc(*basis.args(), ctypes.c_int(nbf), ctypes.c_int(len(tasks)),
                              _i64(pt_off), _p(pts), _p(wts), _i64(sh_off), _i32(sl),
                              ctypes.c_int(kind), ctypes.c_double(xs), ctypes.c_double(cs),
                              ctypes.c_double(kappa), ctypes.c_double(mu), ctypes.c_int(gga),
                              Pm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              V.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if V is not None else None,
                              _p(en), ctypes.c_int(nthreads))
    return en[0], V, en[1]


def functional_pol(name, rho, sigma=None):
    """Polarized functional: rho[n, 2] (alpha, beta), sigma[n, 3] (aa, ab, bb).
    Returns eps[n], vrho[n, 2], vsigma[n, 3]."""
    kind, xs, cs, kappa, mu, _ = FUNCTIONALS[name.upper()]
    rho = np.ascontiguousarray(rho, dtype=np.float64).reshape(-1, 2)
    n = len(rho)
    sg = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1, 3)
    eps, vr, vs = np.zeros(n), np.zeros((n, 2)), np.zeros((n, 3))
    lib().oracle_functional_pol(ctypes.c_int(kind), ctypes.c_double(xs), ctypes.c_double(cs),
                                ctypes.c_double(kappa), ctypes.c_double(mu), ctypes.c_int64(n),
                                _p(rho), _p(sg), _p(eps), _p(vr), _p(vs))
    return eps, vr, vs


def eval_exc_vxc_uks(basis, tasks, Ps, Pz, func, want_vxc=True, nthreads=0):
    """UKS: Ps = Pa + Pb, Pz = Pa - Pb.  Returns (EXC, VXCs, VXCz, N_el)."""
    kind, xs, cs, kappa, mu, gga = FUNCTIONALS[func.upper()]
    pt_off = np.zeros(len(tasks) + 1, np.int64)
    sh_off = np.zeros(len(tasks) + 1, np.int64)
    for i, (p, w, s) in enumerate(tasks):
        pt_off[i + 1] = pt_off[i] + len(w)
        sh_off[i + 1] = sh_off[i] + len(s)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(t[0]).reshape(-1, 3) for t in tasks]))
    wts = np.ascontiguousarray(np.concatenate([t[1] for t in tasks]))
    sl = np.ascontiguousarray(np.concatenate([t[2] for t in tasks]).astype(np.int32))
    nbf = basis.nbf
    A = np.asfortranarray(Ps, dtype=np.float64)
    Bz = np.asfortranarray(Pz, dtype=np.float64)
    Vs = np.zeros((nbf, nbf), order="F") if want_vxc else None
    Vz = np.zeros((nbf, nbf), order="F") if want_vxc else None
    en = np.zeros(2)
    dp = ctypes.POINTER(ctypes.c_double)
    lib().oracle_eval_exc_vxc_uks(*basis.args(), ctypes.c_int(nbf), ctypes.c_int(len(tasks)),
                                  _i64(pt_off), _p(pts), _p(wts), _i64(sh_off), _i32(sl),
                                  ctypes.c_int(kind), ctypes.c_double(xs), ctypes.c_double(cs),
                                  ctypes.c_double(kappa), ctypes.c_double(mu), ctypes.c_int(gga),
                                  A.ctypes.data_as(dp), Bz.ctypes.data_as(dp),
                                  Vs.ctypes.data_as(dp) if Vs is not None else None,
                                  Vz.ctypes.data_as(dp) if Vz is not None else None,
                                  _p(en), ctypes.c_int(nthreads))
    return en[0], Vs, Vz, en[1]
