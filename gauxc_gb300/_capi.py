"""ctypes declarations of the C ABI in include/gauxc_gb300.h."""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgauxc_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gauxc_gb300.h")


class GauXCStatus(ctypes.Structure):
    _fields_ = [("code", ctypes.c_int), ("message", ctypes.c_void_p)]


class GauXCHeader(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int)]


def _handle(name, extra=()):
    return type(name, (ctypes.Structure,),
                {"_fields_": [("hdr", GauXCHeader), ("ptr", ctypes.c_void_p)] + list(extra)})


GauXCMolecule = _handle("GauXCMolecule")
GauXCBasisSet = _handle("GauXCBasisSet")
GauXCMolGrid = _handle("GauXCMolGrid")
GauXCRuntimeEnvironment = _handle("GauXCRuntimeEnvironment", [("device_ptr", ctypes.c_void_p)])
GauXCLoadBalancer = _handle("GauXCLoadBalancer")
GauXCLoadBalancerFactory = _handle("GauXCLoadBalancerFactory")
GauXCMolecularWeights = _handle("GauXCMolecularWeights")
GauXCMolecularWeightsFactory = _handle("GauXCMolecularWeightsFactory")
GauXCFunctional = _handle("GauXCFunctional")
GauXCIntegrator = _handle("GauXCIntegrator")
GauXCGB300Batch = _handle("GauXCGB300Batch")
GauXCGB300DeviceData = _handle("GauXCGB300DeviceData")


class GauXCAtom(ctypes.Structure):
    _fields_ = [("Z", ctypes.c_int64), ("x", ctypes.c_double), ("y", ctypes.c_double),
                ("z", ctypes.c_double)]


class GauXCShell(ctypes.Structure):
    _fields_ = [("l", ctypes.c_int32), ("pure", ctypes.c_bool), ("nprim", ctypes.c_int32),
                ("exponents", ctypes.c_double * 32), ("coefficients", ctypes.c_double * 32),
                ("origin", ctypes.c_double * 3), ("shell_tolerance", ctypes.c_double)]


class MolecularWeightsSettingsC(ctypes.Structure):
    _fields_ = [("weight_alg", ctypes.c_int), ("becke_size_adjustment", ctypes.c_bool)]


S = ctypes.POINTER(GauXCStatus)
P = ctypes.POINTER
dbl, i32, i64, sz, cstr, vp, b = (ctypes.c_double, ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t,
                                  ctypes.c_char_p, ctypes.c_void_p, ctypes.c_bool)
I = ctypes.c_int

PROTOTYPES = {
    "gauxc_status_delete": (None, [S]),
    "gauxc_object_delete": (None, [S, P(vp)]),
    "gauxc_molecule_new": (GauXCMolecule, [S]),
    "gauxc_molecule_new_from_atoms": (GauXCMolecule, [S, P(GauXCAtom), sz]),
    "gauxc_molecule_delete": (None, [S, P(GauXCMolecule)]),
    "gauxc_molecule_natoms": (sz, [S, GauXCMolecule]),
    "gauxc_basisset_new": (GauXCBasisSet, [S]),
    "gauxc_basisset_new_from_shells": (GauXCBasisSet, [S, P(GauXCShell), sz, b]),
    "gauxc_basisset_delete": (None, [S, P(GauXCBasisSet)]),
    "gauxc_molgrid_new_default": (GauXCMolGrid, [S, GauXCMolecule, I, i64, I, I]),
    "gauxc_molgrid_delete": (None, [S, P(GauXCMolGrid)]),
    "gauxc_runtime_environment_new": (GauXCRuntimeEnvironment, [S]),
    "gauxc_device_runtime_environment_new": (GauXCRuntimeEnvironment, [S, dbl]),
    "gauxc_device_runtime_environment_new_mem": (GauXCRuntimeEnvironment, [S, vp, sz]),
    "gauxc_runtime_environment_delete": (None, [S, P(GauXCRuntimeEnvironment)]),
    "gauxc_runtime_environment_comm_rank": (I, [S, GauXCRuntimeEnvironment]),
    "gauxc_runtime_environment_comm_size": (I, [S, GauXCRuntimeEnvironment]),
    "gauxc_load_balancer_factory_new": (GauXCLoadBalancerFactory, [S, I, cstr]),
    "gauxc_load_balancer_factory_delete": (None, [S, P(GauXCLoadBalancerFactory)]),
    "gauxc_load_balancer_factory_get_instance": (
        GauXCLoadBalancer,
        [S, GauXCLoadBalancerFactory, GauXCRuntimeEnvironment, GauXCMolecule, GauXCMolGrid,
         GauXCBasisSet]),
    "gauxc_load_balancer_delete": (None, [S, P(GauXCLoadBalancer)]),
    "gauxc_molecular_weights_factory_new": (GauXCMolecularWeightsFactory,
                                            [S, I, cstr, MolecularWeightsSettingsC]),
    "gauxc_molecular_weights_factory_delete": (None, [S, P(GauXCMolecularWeightsFactory)]),
    "gauxc_molecular_weights_factory_get_instance": (GauXCMolecularWeights,
                                                     [S, GauXCMolecularWeightsFactory]),
    "gauxc_molecular_weights_modify_weights": (None, [S, GauXCMolecularWeights, GauXCLoadBalancer]),
    "gauxc_molecular_weights_delete": (None, [S, P(GauXCMolecularWeights)]),
    "gauxc_functional_from_string": (GauXCFunctional, [S, cstr, b]),
    "gauxc_functional_from_enum": (GauXCFunctional, [S, I, b]),
    "gauxc_functional_delete": (None, [S, P(GauXCFunctional)]),
    "gauxc_integrator_new": (GauXCIntegrator,
                             [S, GauXCFunctional, GauXCLoadBalancer, I, cstr, cstr, cstr, cstr]),
    "gauxc_integrator_delete": (None, [S, P(GauXCIntegrator)]),
    "gauxc_integrator_integrate_den": (None, [S, GauXCIntegrator, i64, i64, P(dbl), i64, P(dbl)]),
    "gauxc_integrator_eval_exc_rks": (None, [S, GauXCIntegrator, i64, i64, P(dbl), i64, P(dbl)]),
    "gauxc_integrator_eval_exc_vxc_rks": (None, [S, GauXCIntegrator, i64, i64, P(dbl), i64,
                                                 P(dbl), P(dbl), i64]),
    "gauxc_integrator_eval_exc_uks": (None, [S, GauXCIntegrator, i64, i64, P(dbl), i64, P(dbl),
                                             i64, P(dbl)]),
    "gauxc_integrator_eval_exc_vxc_uks": (None, [S, GauXCIntegrator, i64, i64, P(dbl), i64,
                                                 P(dbl), i64, P(dbl), P(dbl), i64, P(dbl), i64]),
    "gauxc_gb300_lwd_device_data_new": (GauXCGB300DeviceData, [S, GauXCLoadBalancer, i64, i64]),
    "gauxc_gb300_lwd_device_data_delete": (None, [S, P(GauXCGB300DeviceData)]),
    "gauxc_gb300_lwd_eval_collocation": (None, [S, GauXCGB300DeviceData, b]),
    "gauxc_gb300_lwd_eval_xmat": (None, [S, GauXCGB300DeviceData, dbl, P(dbl), i64]),
    "gauxc_gb300_lwd_eval_vvars": (None, [S, GauXCGB300DeviceData, b]),
    "gauxc_gb300_lwd_eval_uvars": (None, [S, GauXCGB300DeviceData]),
    "gauxc_gb300_lwd_eval_kern_exc_vxc": (None, [S, GauXCGB300DeviceData, GauXCFunctional]),
    "gauxc_gb300_lwd_inc_exc": (None, [S, GauXCGB300DeviceData]),
    "gauxc_gb300_lwd_inc_nel": (None, [S, GauXCGB300DeviceData]),
    "gauxc_gb300_lwd_eval_zmat_vxc": (None, [S, GauXCGB300DeviceData, b]),
    "gauxc_gb300_lwd_inc_vxc": (None, [S, GauXCGB300DeviceData]),
    "gauxc_gb300_lwd_symmetrize_vxc": (None, [S, GauXCGB300DeviceData, P(dbl), i64]),
    "gauxc_gb300_lwd_results": (None, [S, GauXCGB300DeviceData, P(dbl), P(dbl)]),
    "gauxc_gb300_version": (ctypes.c_char_p, []),
    "gauxc_gb300_device_count": (I, []),
    "gauxc_gb300_basisset_nshells": (sz, [S, GauXCBasisSet]),
    "gauxc_gb300_basisset_nbf": (i32, [S, GauXCBasisSet]),
    "gauxc_gb300_basisset_get_shell": (None, [S, GauXCBasisSet, sz, P(GauXCShell), P(dbl)]),
    "gauxc_gb300_basisset_set_tolerance": (None, [S, GauXCBasisSet, dbl]),
    "gauxc_gb300_molgrid_atomic_grid": (None, [S, GauXCMolGrid, i64, P(i64), P(i64), P(dbl),
                                               P(dbl), P(i64)]),
    "gauxc_gb300_load_balancer_ntasks": (sz, [S, GauXCLoadBalancer]),
    "gauxc_gb300_load_balancer_task_info": (None, [S, GauXCLoadBalancer, sz, P(i32), P(dbl)]),
    "gauxc_gb300_load_balancer_task_data": (None, [S, GauXCLoadBalancer, sz, P(dbl), P(dbl),
                                                   P(i32)]),
    "gauxc_gb300_load_balancer_weights_modified": (b, [S, GauXCLoadBalancer]),
    "gauxc_gb300_load_balancer_subset": (GauXCLoadBalancer, [S, GauXCLoadBalancer, P(i64), sz]),
    "gauxc_gb300_integrator_last_nel": (dbl, [S, GauXCIntegrator]),
    "gauxc_gb300_integrator_timings": (I, [S, GauXCIntegrator, P(dbl), I]),
    "gauxc_gb300_integrator_plan_stats": (I, [S, GauXCIntegrator, P(dbl), I]),
    "gauxc_gb300_integrator_set_plan_params": (None, [S, GauXCIntegrator, I, dbl, dbl]),
    "gauxc_gb300_integrator_autotune": (dbl, [S, GauXCIntegrator, i64, i64, P(dbl), i64, P(I),
                                               P(dbl)]),
    "gauxc_gb300_batch_new": (GauXCGB300Batch, [S, P(GauXCIntegrator), i32]),
    "gauxc_gb300_batch_eval_exc_vxc_rks": (None, [S, GauXCGB300Batch, P(P(dbl)), P(i64),
                                                  P(P(dbl)), P(i64), P(dbl)]),
    "gauxc_gb300_batch_timings": (I, [S, GauXCGB300Batch, P(dbl), I]),
    "gauxc_gb300_batch_delete": (None, [S, P(GauXCGB300Batch)]),
    "gauxc_gb300_integrator_set_profiling": (None, [S, GauXCIntegrator, b]),
    "gauxc_gb300_integrator_set_pipeline_check": (None, [S, GauXCIntegrator, dbl, b]),
    "gauxc_gb300_integrator_kernel_times": (I, [S, GauXCIntegrator, P(dbl), I]),
    "gauxc_gb300_measure_fp64_peak": (dbl, [S]),
    "gauxc_gb300_host_register": (ctypes.c_int, [S, ctypes.c_void_p, ctypes.c_size_t]),
    "gauxc_gb300_host_unregister": (None, [S, ctypes.c_void_p]),
    "gauxc_gb300_set_device": (None, [S, I]),
    "gauxc_gb300_tensor_core_selftest": (dbl, [S, I, I]),
    "gauxc_gb300_ff_exp_selftest": (dbl, [S, I]),
    "gauxc_gb300_ssf_weights": (None, [S, i64, i32, P(dbl), P(i32), P(dbl), P(dbl), P(dbl)]),
    "gauxc_gb300_ssf_weights_noalloc": (None, [S, i64, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
    "gauxc_gb300_collocation": (None, [S, GauXCBasisSet, i64, P(dbl), i32, P(i32), P(dbl),
                                       P(dbl), P(dbl), P(dbl)]),
}


class GauXCError(RuntimeError):
    pass


def header_symbols():
    """Function names declared in include/gauxc_gb300.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = set()
    for m in re.finditer(r"\b(gauxc_\w+)\s*\(", txt):
        names.add(m.group(1))
    return sorted(names)


def load_library(path=LIB_PATH):
    if not os.path.exists(path):
        raise ImportError(f"native library {path} is missing; build it with "
                          f"'python -m gauxc_gb300.build'")
    L = ctypes.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def check(st, L):
    if st.code != 0:
        msg = ctypes.string_at(st.message).decode() if st.message else "error"
        L.gauxc_status_delete(ctypes.byref(st))
        raise GauXCError(msg)
    if st.message:
        L.gauxc_status_delete(ctypes.byref(st))
