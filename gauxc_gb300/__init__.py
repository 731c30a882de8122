"""GB300 device XC integrator with GauXC's integrator API.

Python mirror of the reference C++ front end for the device EXC/VXC path
(include/gauxc/xc_integrator/integrator_factory.hpp:24-111,
include/gauxc/xc_integrator.hpp:30-94): build a Molecule, a BasisSet and a
MolGrid, get a LoadBalancer from a LoadBalancerFactory, apply SSF weights
with a MolecularWeights instance, then call
``XCIntegratorFactory(...).get_instance(func, lb).eval_exc_vxc(P)``.

Everything goes through the C ABI of ``lib/libgauxc_gb300.so`` (declared in
``include/gauxc_gb300.h``); importing this package fails if the native library
has not been built (``python -m gauxc_gb300.build``).
"""
import ctypes
import enum
import os

import numpy as np

from ._capi import (GauXCAtom, GauXCIntegrator, GauXCShell, GauXCStatus,
                    MolecularWeightsSettingsC, check, load_library)

__all__ = [
    "ExecutionSpace", "PruningScheme", "RadialQuad", "AtomicGridSizeDefault", "XCWeightAlg",
    "Molecule", "Shell", "BasisSet", "MolGrid", "MolGridFactory", "RuntimeEnvironment",
    "DeviceRuntimeEnvironment", "LoadBalancer", "LoadBalancerFactory",
    "MolecularWeightsSettings", "MolecularWeights", "MolecularWeightsFactory",
    "functional_type", "XCIntegrator", "XCIntegratorFactory", "IntegratorBatch", "lib",
    "LocalDeviceWorkDriver", "XCDeviceData",
    "device_count",
    "ssf_weights", "collocation", "set_device", "measure_fp64_peak", "host_register",
    "host_unregister",
]

class _LazyLibrary:
    """Loads the native library on first use (so the build module can be imported
    before the library exists); any missing library or symbol raises then."""

    _cdll = None

    def __getattr__(self, name):
        if _LazyLibrary._cdll is None:
            _LazyLibrary._cdll = load_library()
        return getattr(_LazyLibrary._cdll, name)


_L = _LazyLibrary()


def lib():
    _L.gauxc_gb300_version  # force the load
    return _LazyLibrary._cdll


def device_count():
    return int(_L.gauxc_gb300_device_count())


def set_device(dev):
    _call(_L.gauxc_gb300_set_device, int(dev))


def tensor_core_selftest(n=256, k=256):
    """Worst relative error of the tensor-core emulated-FP64 GEMM on random data."""
    return float(_call(_L.gauxc_gb300_tensor_core_selftest, int(n), int(k)))


def ff_exp_selftest(n=1 << 20):
    """Largest relative error of the collocation's float-float exp against FP64."""
    return float(_call(_L.gauxc_gb300_ff_exp_selftest, int(n)))


def host_register(a):
    """Page-locks the memory of numpy array `a` in place (for P / VXC buffers
    reused every SCF iteration); True when it registered it."""
    return bool(_call(_L.gauxc_gb300_host_register, ctypes.c_void_p(a.ctypes.data),
                      ctypes.c_size_t(a.nbytes)))


def host_unregister(a):
    """Undoes host_register."""
    _call(_L.gauxc_gb300_host_unregister, ctypes.c_void_p(a.ctypes.data))


def measure_fp64_peak():
    """Measured FP64 FMA throughput of the current GPU, TFLOP/s."""
    return float(_call(_L.gauxc_gb300_measure_fp64_peak))


class ExecutionSpace(enum.IntEnum):
    Host = 0
    Device = 1


class PruningScheme(enum.IntEnum):
    Unpruned = 0
    Robust = 1
    Treutler = 2


class RadialQuad(enum.IntEnum):
    Becke = 0
    MuraKnowles = 1
    MurrayHandyLaming = 2
    TreutlerAhlrichs = 3


class AtomicGridSizeDefault(enum.IntEnum):
    FineGrid = 0
    UltraFineGrid = 1
    SuperFineGrid = 2
    GM3 = 3
    GM5 = 4


class XCWeightAlg(enum.IntEnum):
    NOTPARTITIONED = 0
    Becke = 1
    SSF = 2
    LKO = 3


class _Handle:
    _delete = None

    def __init__(self, h):
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.ptr and self._delete is not None and _L is not None:
            st = GauXCStatus()
            getattr(_L, self._delete)(ctypes.byref(st), ctypes.byref(h))
            _L.gauxc_status_delete(ctypes.byref(st))


def _call(fn, *args):
    st = GauXCStatus()
    r = fn(ctypes.byref(st), *args)
    check(st, _L)
    return r


# ------------------------------------------------------------------ molecule / basis
class Molecule(_Handle):
    """Atoms with coordinates in bohr: list of (Z, x, y, z)."""
    _delete = "gauxc_molecule_delete"

    def __init__(self, atoms):
        atoms = list(atoms)
        arr = (GauXCAtom * max(len(atoms), 1))()
        for i, (Z, x, y, z) in enumerate(atoms):
            arr[i] = GauXCAtom(int(Z), float(x), float(y), float(z))
        super().__init__(_call(_L.gauxc_molecule_new_from_atoms, arr, ctypes.c_size_t(len(atoms))))
        self.atoms = [(int(a[0]), float(a[1]), float(a[2]), float(a[3])) for a in atoms]

    def natoms(self):
        return int(_call(_L.gauxc_molecule_natoms, self._h))

    def coords(self):
        return np.array([[a[1], a[2], a[3]] for a in self.atoms])


class Shell:
    """One contracted shell: exponents, coefficients, origin, l, pure."""

    def __init__(self, l, exponents, coefficients, origin, pure=True, tolerance=1e-10):
        self.l = int(l)
        self.exponents = np.asarray(exponents, dtype=np.float64)
        self.coefficients = np.asarray(coefficients, dtype=np.float64)
        self.origin = np.asarray(origin, dtype=np.float64)
        self.pure = bool(pure)
        self.tolerance = float(tolerance)

    def size(self):
        return 2 * self.l + 1 if self.pure else (self.l + 1) * (self.l + 2) // 2


class BasisSet(_Handle):
    _delete = "gauxc_basisset_delete"

    def __init__(self, shells, normalize=True):
        shells = list(shells)
        arr = (GauXCShell * max(len(shells), 1))()
        for i, s in enumerate(shells):
            c = GauXCShell()
            c.l = s.l
            c.pure = s.pure
            c.nprim = len(s.exponents)
            for k in range(len(s.exponents)):
                c.exponents[k] = s.exponents[k]
                c.coefficients[k] = s.coefficients[k]
            for a in range(3):
                c.origin[a] = s.origin[a]
            c.shell_tolerance = s.tolerance
            arr[i] = c
        super().__init__(_call(_L.gauxc_basisset_new_from_shells, arr,
                               ctypes.c_size_t(len(shells)), ctypes.c_bool(normalize)))

    def nshells(self):
        return int(_call(_L.gauxc_gb300_basisset_nshells, self._h))

    def nbf(self):
        return int(_call(_L.gauxc_gb300_basisset_nbf, self._h))

    def shell(self, i):
        """(l, pure, exponents, coefficients (normalized), origin, tolerance, cutoff_radius)."""
        c = GauXCShell()
        r = ctypes.c_double()
        _call(_L.gauxc_gb300_basisset_get_shell, self._h, ctypes.c_size_t(i), ctypes.byref(c),
              ctypes.byref(r))
        n = c.nprim
        return (c.l, bool(c.pure), np.array(c.exponents[:n]), np.array(c.coefficients[:n]),
                np.array(c.origin[:]), c.shell_tolerance, r.value)

    def set_shell_tolerance(self, tol):
        _call(_L.gauxc_gb300_basisset_set_tolerance, self._h, ctypes.c_double(tol))

    def arrays(self):
        """Shell arrays (l, pure, nprim, alpha[n,32], coeff[n,32], origin[n,3], cutoff[n])."""
        n = self.nshells()
        l = np.zeros(n, np.int32)
        pure = np.zeros(n, np.int32)
        nprim = np.zeros(n, np.int32)
        alpha = np.zeros((n, 32))
        coeff = np.zeros((n, 32))
        origin = np.zeros((n, 3))
        cut = np.zeros(n)
        for i in range(n):
            li, pi, a, c, o, _, r = self.shell(i)
            l[i], pure[i], nprim[i] = li, int(pi), len(a)
            alpha[i, :len(a)] = a
            coeff[i, :len(c)] = c
            origin[i] = o
            cut[i] = r
        return l, pure, nprim, alpha, coeff, origin, cut


# ------------------------------------------------------------------ grids
class MolGrid(_Handle):
    _delete = "gauxc_molgrid_delete"

    def atomic_grid(self, Z):
        """(points[n,3], weights[n], batch_ranges[nb,2]) of element Z, origin-centred."""
        n = ctypes.c_int64()
        nb = ctypes.c_int64()
        _call(_L.gauxc_gb300_molgrid_atomic_grid, self._h, ctypes.c_int64(Z), ctypes.byref(n),
              ctypes.byref(nb), None, None, None)
        pts = np.zeros((n.value, 3))
        w = np.zeros(n.value)
        br = np.zeros((nb.value, 2), np.int64)
        _call(_L.gauxc_gb300_molgrid_atomic_grid, self._h, ctypes.c_int64(Z), None, None,
              pts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              br.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
        return pts, w, br


class MolGridFactory:
    @staticmethod
    def create_default_molgrid(mol, pruning_scheme, batch_size, radial_quad, grid_size):
        h = _call(_L.gauxc_molgrid_new_default, mol._h, int(pruning_scheme),
                  ctypes.c_int64(int(batch_size)), int(radial_quad), int(grid_size))
        g = MolGrid(h)
        g._mol = mol
        return g


# ------------------------------------------------------------------ runtime
class RuntimeEnvironment(_Handle):
    _delete = "gauxc_runtime_environment_delete"

    def __init__(self, h=None):
        super().__init__(h if h is not None else _call(_L.gauxc_runtime_environment_new))

    def comm_rank(self):
        return int(_call(_L.gauxc_runtime_environment_comm_rank, self._h))

    def comm_size(self):
        return int(_call(_L.gauxc_runtime_environment_comm_size, self._h))


class DeviceRuntimeEnvironment(RuntimeEnvironment):
    """fill_fraction of free device memory, or a caller-owned device buffer (ptr, nbytes)."""

    def __init__(self, fill_fraction=0.9, mem=None):
        if mem is not None:
            ptr, nbytes = mem
            h = _call(_L.gauxc_device_runtime_environment_new_mem, ctypes.c_void_p(ptr),
                      ctypes.c_size_t(nbytes))
        else:
            h = _call(_L.gauxc_device_runtime_environment_new, ctypes.c_double(fill_fraction))
        super().__init__(h)


# ------------------------------------------------------------------ load balancer
class LoadBalancer(_Handle):
    _delete = "gauxc_load_balancer_delete"

    def ntasks(self):
        return int(_call(_L.gauxc_gb300_load_balancer_ntasks, self._h))

    def task_info(self, i):
        info = (ctypes.c_int32 * 4)()
        dn = ctypes.c_double()
        _call(_L.gauxc_gb300_load_balancer_task_info, self._h, ctypes.c_size_t(i), info,
              ctypes.byref(dn))
        return dict(iParent=info[0], npts=info[1], nbe=info[2], nshells=info[3],
                    dist_nearest=dn.value)

    def task(self, i):
        inf = self.task_info(i)
        pts = np.zeros((inf["npts"], 3))
        w = np.zeros(inf["npts"])
        sl = np.zeros(inf["nshells"], np.int32)
        _call(_L.gauxc_gb300_load_balancer_task_data, self._h, ctypes.c_size_t(i),
              pts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              sl.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        inf.update(points=pts, weights=w, shell_list=sl)
        return inf

    def get_tasks(self):
        return [self.task(i) for i in range(self.ntasks())]

    def weights_modified(self):
        return bool(_call(_L.gauxc_gb300_load_balancer_weights_modified, self._h))

    def subset(self, task_indices):
        """A load balancer over the listed tasks (copies, current weights)."""
        idx = np.ascontiguousarray(task_indices, dtype=np.int64)
        lb = LoadBalancer(_call(_L.gauxc_gb300_load_balancer_subset, self._h,
                                idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                ctypes.c_size_t(len(idx))))
        lb._keep = self._keep
        return lb


class LoadBalancerFactory(_Handle):
    _delete = "gauxc_load_balancer_factory_delete"

    def __init__(self, ex, kernel_name="Default"):
        super().__init__(_call(_L.gauxc_load_balancer_factory_new, int(ex), kernel_name.encode()))

    def get_instance(self, rt, mol, mg, basis):
        lb = LoadBalancer(_call(_L.gauxc_load_balancer_factory_get_instance, self._h, rt._h,
                                mol._h, mg._h, basis._h))
        lb._keep = (rt, mol, mg, basis)
        return lb


# ------------------------------------------------------------------ weights
class MolecularWeightsSettings:
    def __init__(self, weight_alg=XCWeightAlg.SSF, becke_size_adjustment=False):
        self.weight_alg = weight_alg
        self.becke_size_adjustment = becke_size_adjustment


class MolecularWeights(_Handle):
    _delete = "gauxc_molecular_weights_delete"

    def modify_weights(self, lb):
        _call(_L.gauxc_molecular_weights_modify_weights, self._h, lb._h)


class MolecularWeightsFactory(_Handle):
    _delete = "gauxc_molecular_weights_factory_delete"

    def __init__(self, ex, lwd_kernel="Default", settings=None):
        settings = settings or MolecularWeightsSettings()
        s = MolecularWeightsSettingsC(int(settings.weight_alg), bool(settings.becke_size_adjustment))
        super().__init__(_call(_L.gauxc_molecular_weights_factory_new, int(ex), lwd_kernel.encode(), s))

    def get_instance(self):
        return MolecularWeights(_call(_L.gauxc_molecular_weights_factory_get_instance, self._h))


# ------------------------------------------------------------------ functional / integrator
class functional_type(_Handle):
    """XC functional by name: SVWN5, PBE, revPBE, PBE0; polarized=True for UKS."""
    _delete = "gauxc_functional_delete"

    def __init__(self, name, polarized=False):
        super().__init__(_call(_L.gauxc_functional_from_string, name.encode(),
                               ctypes.c_bool(polarized)))
        self.name = name


class XCIntegrator(_Handle):
    _delete = "gauxc_integrator_delete"

    def _nbf(self):
        return self._lb._keep[3].nbf()

    def eval_exc_vxc(self, P):
        """Returns (EXC, VXC) for the alpha density P (RKS)."""
        P = np.asfortranarray(P, dtype=np.float64)
        n = self._nbf()
        VXC = np.zeros((n, n), order="F")
        exc = ctypes.c_double()
        _call(_L.gauxc_integrator_eval_exc_vxc_rks, self._h, ctypes.c_int64(P.shape[0]),
              ctypes.c_int64(P.shape[1]), P.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              ctypes.c_int64(P.shape[0]), ctypes.byref(exc),
              VXC.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_int64(n))
        return exc.value, VXC

    def eval_exc_vxc_uks(self, Ps, Pz):
        """UKS: Ps = P_alpha + P_beta, Pz = P_alpha - P_beta (polarized
        functional).  Returns (EXC, VXC_s, VXC_z)."""
        Ps = np.asfortranarray(Ps, dtype=np.float64)
        Pz = np.asfortranarray(Pz, dtype=np.float64)
        n = self._nbf()
        Vs = np.zeros((n, n), order="F")
        Vz = np.zeros((n, n), order="F")
        exc = ctypes.c_double()
        dp = ctypes.POINTER(ctypes.c_double)
        _call(_L.gauxc_integrator_eval_exc_vxc_uks, self._h, ctypes.c_int64(Ps.shape[0]),
              ctypes.c_int64(Ps.shape[1]), Ps.ctypes.data_as(dp), ctypes.c_int64(Ps.shape[0]),
              Pz.ctypes.data_as(dp), ctypes.c_int64(Pz.shape[0]), ctypes.byref(exc),
              Vs.ctypes.data_as(dp), ctypes.c_int64(n), Vz.ctypes.data_as(dp), ctypes.c_int64(n))
        return exc.value, Vs, Vz

    def eval_exc_uks(self, Ps, Pz):
        Ps = np.asfortranarray(Ps, dtype=np.float64)
        Pz = np.asfortranarray(Pz, dtype=np.float64)
        exc = ctypes.c_double()
        dp = ctypes.POINTER(ctypes.c_double)
        _call(_L.gauxc_integrator_eval_exc_uks, self._h, ctypes.c_int64(Ps.shape[0]),
              ctypes.c_int64(Ps.shape[1]), Ps.ctypes.data_as(dp), ctypes.c_int64(Ps.shape[0]),
              Pz.ctypes.data_as(dp), ctypes.c_int64(Pz.shape[0]), ctypes.byref(exc))
        return exc.value

    def eval_exc(self, P):
        P = np.asfortranarray(P, dtype=np.float64)
        exc = ctypes.c_double()
        _call(_L.gauxc_integrator_eval_exc_rks, self._h, ctypes.c_int64(P.shape[0]),
              ctypes.c_int64(P.shape[1]), P.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              ctypes.c_int64(P.shape[0]), ctypes.byref(exc))
        return exc.value

    def integrate_den(self, P):
        P = np.asfortranarray(P, dtype=np.float64)
        den = ctypes.c_double()
        _call(_L.gauxc_integrator_integrate_den, self._h, ctypes.c_int64(P.shape[0]),
              ctypes.c_int64(P.shape[1]), P.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
              ctypes.c_int64(P.shape[0]), ctypes.byref(den))
        return den.value

    def last_nel(self):
        return float(_call(_L.gauxc_gb300_integrator_last_nel, self._h))

    def timings(self):
        out = (ctypes.c_double * 8)()
        _call(_L.gauxc_gb300_integrator_timings, self._h, out, 8)
        return dict(zip(["h2d_ms", "compute_ms", "d2h_ms", "wall_ms", "plan_ms", "plan_merge_ms",
                         "plan_layout_ms", "plan_lists_ms"], list(out)))

    def set_profiling(self, on=True):
        _call(_L.gauxc_gb300_integrator_set_profiling, self._h, ctypes.c_bool(on))

    def set_pipeline_check(self, wait_ms=1000.0, withhold=False):
        """Bound of the tensor-core pipeline waits (ms) of the following calls;
        withhold=True makes the GEMM producers issue no copy, so the calls fail
        with the pipeline error after wait_ms (check of the error path)."""
        _call(_L.gauxc_gb300_integrator_set_pipeline_check, self._h, ctypes.c_double(wait_ms),
              ctypes.c_bool(withhold))

    def kernel_times(self):
        out = (ctypes.c_double * 14)()
        _call(_L.gauxc_gb300_integrator_kernel_times, self._h, out, 14)
        names = ["collocation", "density", "zmat", "vxc", "other", "phi_digits", "p_digits"]
        return {n: dict(ms=out[2 * i], launches=int(out[2 * i + 1])) for i, n in enumerate(names)}

    def plan_stats(self):
        out = (ctypes.c_double * 18)()
        _call(_L.gauxc_gb300_integrator_plan_stats, self._h, out, 18)
        keys = ["ntasks", "npts", "npts_pad", "nbatches", "sum_npts_nbe", "sum_npts_nbe2",
                "sum_pad_npts_nbe2", "scratch_bytes", "gpu_launches", "tensor_flops_x",
                "tensor_flops_v"]
        st = dict(zip(keys, list(out)))
        names = ["collocation", "density", "zmat", "vxc", "other", "phi_digits", "p_digits"]
        st["kernel_bytes"] = {n: out[11 + i] for i, n in enumerate(names)}
        return st


    def set_plan_params(self, pb_max_pts=384, nu2_weight=100.0, scratch_gb=0.0):
        """Plan parameters (point-block size and merge weight of "GB300-Mixed",
        work-space cap in GB, 0 = from free memory); the plan is rebuilt on the
        next call."""
        _call(_L.gauxc_gb300_integrator_set_plan_params, self._h, int(pb_max_pts),
              float(nu2_weight), float(scratch_gb))

    def autotune(self, P):
        """Times the candidate plans on P, keeps the fastest.
        Returns (compute_ms, dict(pb_max_pts=..., nu2_weight=...))."""
        P = np.asfortranarray(P, dtype=np.float64)
        pts, w = ctypes.c_int(), ctypes.c_double()
        ms = _call(_L.gauxc_gb300_integrator_autotune, self._h, ctypes.c_int64(P.shape[0]),
                   ctypes.c_int64(P.shape[1]), P.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                   ctypes.c_int64(P.shape[0]), ctypes.byref(pts), ctypes.byref(w))
        return float(ms), dict(pb_max_pts=pts.value, nu2_weight=w.value)


class IntegratorBatch(_Handle):
    """Many integrators evaluated by one CUDA-graph launch per call.

    The first call with a given set of arrays runs the members one by one and
    captures the graph; later calls with the same arrays replay it.  The
    arrays are page-locked in place while the batch uses them, so keep them
    (and reuse them across SCF iterations)."""
    _delete = "gauxc_gb300_batch_delete"

    def __init__(self, integrators):
        self.members = list(integrators)
        arr = (GauXCIntegrator * len(self.members))(*[m._h for m in self.members])
        super().__init__(_call(_L.gauxc_gb300_batch_new, arr, ctypes.c_int32(len(self.members))))

    def eval_exc_vxc(self, Ps, VXCs):
        """EXC of every member into a numpy array; VXC[i] written in place
        (Fortran-ordered float64 arrays, nbf_i x nbf_i; None = EXC only)."""
        n = len(self.members)
        dp = ctypes.POINTER(ctypes.c_double)
        for P in Ps:
            if not (P.dtype == np.float64 and P.flags.f_contiguous):
                raise ValueError("batch density matrices must be Fortran-ordered float64")
        pp = (dp * n)(*[P.ctypes.data_as(dp) for P in Ps])
        ldp = (ctypes.c_int64 * n)(*[P.shape[0] for P in Ps])
        vv = (dp * n)(*[V.ctypes.data_as(dp) if V is not None else dp() for V in VXCs])
        ldv = (ctypes.c_int64 * n)(*[V.shape[0] if V is not None else 0 for V in VXCs])
        exc = np.zeros(n)
        _call(_L.gauxc_gb300_batch_eval_exc_vxc_rks, self._h, pp, ldp, vv, ldv,
              exc.ctypes.data_as(dp))
        return exc

    def timings(self):
        out = (ctypes.c_double * 5)()
        _call(_L.gauxc_gb300_batch_timings, self._h, out, 5)
        return dict(zip(["compute_ms", "wall_ms", "graph_launch", "members", "gpu_launches"],
                        list(out)))


class XCIntegratorFactory:
    def __init__(self, ex, input_type="Replicated", integrator_kernel="Default",
                 lwd_kernel="Default", reduction_kernel="Default"):
        self.args = (int(ex), input_type.encode(), integrator_kernel.encode(),
                     lwd_kernel.encode(), reduction_kernel.encode())

    def get_instance(self, func, lb):
        ex, it, ik, lk, rk = self.args
        h = _call(_L.gauxc_integrator_new, func._h, lb._h, ex, it, ik, lk, rk)
        integ = XCIntegrator(h)
        integ._lb = lb
        integ._func = func
        return integ


# ------------------------------------------------------------------ stage-level work driver
class XCDeviceData(_Handle):
    """Device data of the stage-level work driver: tasks [begin, end) of a
    weighted load balancer with every intermediate on the device."""
    _delete = "gauxc_gb300_lwd_device_data_delete"


class LocalDeviceWorkDriver:
    """The reference's LocalDeviceWorkDriver stages
    (src/xc_integrator/local_work_driver/device/local_device_work_driver.hpp:62-127),
    FP64, one call per stage on an XCDeviceData."""

    def create_device_data(self, lb, task_begin=0, task_end=None):
        end = lb.ntasks() if task_end is None else task_end
        d = XCDeviceData(_call(_L.gauxc_gb300_lwd_device_data_new, lb._h,
                               ctypes.c_int64(task_begin), ctypes.c_int64(end)))
        d._lb = lb
        d._nbf = lb._keep[3].nbf()
        return d

    def eval_collocation(self, d):
        _call(_L.gauxc_gb300_lwd_eval_collocation, d._h, ctypes.c_bool(False))

    def eval_collocation_gradient(self, d):
        _call(_L.gauxc_gb300_lwd_eval_collocation, d._h, ctypes.c_bool(True))

    def eval_xmat(self, fac, d, P):
        P = np.asfortranarray(P, dtype=np.float64)
        _call(_L.gauxc_gb300_lwd_eval_xmat, d._h, ctypes.c_double(fac),
              P.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_int64(P.shape[0]))

    def eval_vvars_lda(self, d):
        _call(_L.gauxc_gb300_lwd_eval_vvars, d._h, ctypes.c_bool(False))

    def eval_vvars_gga(self, d):
        _call(_L.gauxc_gb300_lwd_eval_vvars, d._h, ctypes.c_bool(True))

    def eval_uvars_gga(self, d):
        _call(_L.gauxc_gb300_lwd_eval_uvars, d._h)

    def eval_kern_exc_vxc_lda(self, func, d):
        _call(_L.gauxc_gb300_lwd_eval_kern_exc_vxc, d._h, func._h)

    eval_kern_exc_vxc_gga = eval_kern_exc_vxc_lda

    def inc_exc(self, d):
        _call(_L.gauxc_gb300_lwd_inc_exc, d._h)

    def inc_nel(self, d):
        _call(_L.gauxc_gb300_lwd_inc_nel, d._h)

    def eval_zmat_lda_vxc(self, d):
        _call(_L.gauxc_gb300_lwd_eval_zmat_vxc, d._h, ctypes.c_bool(False))

    def eval_zmat_gga_vxc(self, d):
        _call(_L.gauxc_gb300_lwd_eval_zmat_vxc, d._h, ctypes.c_bool(True))

    def inc_vxc(self, d):
        _call(_L.gauxc_gb300_lwd_inc_vxc, d._h)

    def symmetrize_vxc(self, d):
        V = np.zeros((d._nbf, d._nbf), order="F")
        _call(_L.gauxc_gb300_lwd_symmetrize_vxc, d._h,
              V.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_int64(d._nbf))
        return V

    def results(self, d):
        """(EXC, N_el) accumulated by inc_exc / inc_nel."""
        e, n = ctypes.c_double(), ctypes.c_double()
        _call(_L.gauxc_gb300_lwd_results, d._h, ctypes.byref(e), ctypes.byref(n))
        return e.value, n.value


# ------------------------------------------------------------------ stage entry points
def ssf_weights(points, iparent, dist_nearest, coords, weights):
    """SSF partition weights on the device (returns the modified weights)."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    w = np.ascontiguousarray(weights, dtype=np.float64).copy()
    ip = np.ascontiguousarray(iparent, dtype=np.int32)
    dn = np.ascontiguousarray(dist_nearest, dtype=np.float64)
    co = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
    dp = ctypes.POINTER(ctypes.c_double)
    _call(_L.gauxc_gb300_ssf_weights, ctypes.c_int64(len(w)), ctypes.c_int32(len(co)),
          pts.ctypes.data_as(dp), ip.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
          dn.ctypes.data_as(dp), co.ctypes.data_as(dp), w.ctypes.data_as(dp))
    return w


def collocation(basis, points, shell_list, grad=False):
    """phi (and grad phi) on the device, host layout [npts, nbe]."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    sl = np.ascontiguousarray(shell_list, dtype=np.int32)
    sizes = [basis.shell(int(s))[0] for s in sl]
    pure = [basis.shell(int(s))[1] for s in sl]
    nbe = sum(2 * l + 1 if p else (l + 1) * (l + 2) // 2 for l, p in zip(sizes, pure))
    outs = [np.zeros((len(pts), nbe)) for _ in range(4 if grad else 1)]
    dp = ctypes.POINTER(ctypes.c_double)
    ptrs = [o.ctypes.data_as(dp) for o in outs] + [None] * (4 - len(outs))
    _call(_L.gauxc_gb300_collocation, basis._h, ctypes.c_int64(len(pts)), pts.ctypes.data_as(dp),
          ctypes.c_int32(len(sl)), sl.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), *ptrs)
    return outs
