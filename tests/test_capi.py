"""C ABI: library loads, exports every declared symbol, reports errors
through GauXCStatus like the reference C API (src/c-api/c_status.hpp)."""
import ctypes

import numpy as np
import pytest

from gauxc_gb300 import _capi


def test_every_header_symbol_is_exported(g):
    L = g.lib()
    names = _capi.header_symbols()
    assert len(names) >= 45
    for n in names:
        assert hasattr(L, n), n
        assert n in _capi.PROTOTYPES, n


def test_version_and_device_count(g):
    assert g.lib().gauxc_gb300_version().startswith(b"gauxc_gb300")
    assert g.device_count() >= 0


def test_invalid_handle_sets_status(g):
    L = g.lib()
    st = _capi.GauXCStatus()
    bad = _capi.GauXCMolecule()
    n = L.gauxc_molecule_natoms(ctypes.byref(st), bad)
    assert n == 0 and st.code == 1
    assert b"Invalid Molecule handle" in ctypes.string_at(st.message)
    L.gauxc_status_delete(ctypes.byref(st))
    assert st.code == 0 and not st.message


def test_status_reset_on_success(g):
    L = g.lib()
    st = _capi.GauXCStatus()
    L.gauxc_molecule_natoms(ctypes.byref(st), _capi.GauXCMolecule())
    assert st.code == 1
    m = L.gauxc_molecule_new(ctypes.byref(st))
    assert st.code == 0 and not st.message
    L.gauxc_molecule_delete(ctypes.byref(st), ctypes.byref(m))
    assert not m.ptr


def test_factory_errors(g):
    from gauxc_gb300._capi import GauXCError
    with pytest.raises(GauXCError, match="SSF"):
        g.MolecularWeightsFactory(g.ExecutionSpace.Device, "Default",
                                  g.MolecularWeightsSettings(g.XCWeightAlg.Becke))
    with pytest.raises(GauXCError, match="device only"):
        g.MolecularWeightsFactory(g.ExecutionSpace.Host)
    with pytest.raises(GauXCError, match="not supported"):
        g.functional_type("B3LYP")
    with pytest.raises(GauXCError, match="not supported"):
        g.LoadBalancerFactory(g.ExecutionSpace.Device, "Replicated-FillIn")
    with pytest.raises(GauXCError, match="fill_fraction"):
        g.DeviceRuntimeEnvironment(1.5)


def _tiny_system(g, ex=None):
    mol = g.Molecule([(1, 0.0, 0.0, 0.0), (1, 0.0, 0.0, 1.4)])
    basis = g.BasisSet([g.Shell(0, [1.0], [1.0], (0.0, 0.0, 0.0)),
                        g.Shell(0, [1.0], [1.0], (0.0, 0.0, 1.4))])
    mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme.Unpruned, 128,
                                                 g.RadialQuad.MuraKnowles,
                                                 g.AtomicGridSizeDefault.FineGrid)
    lb = g.LoadBalancerFactory(ex if ex is not None else g.ExecutionSpace.Host,
                               "Default").get_instance(g.DeviceRuntimeEnvironment(0.5), mol, mg,
                                                       basis)
    return mol, basis, lb


def test_integrator_precondition_errors(g):
    from gauxc_gb300._capi import GauXCError
    mol, basis, lb = _tiny_system(g)
    func = g.functional_type("SVWN5")
    with pytest.raises(GauXCError, match="Local work kernel not supported"):
        g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", "Scheme1-MAGMA").get_instance(func, lb)
    with pytest.raises(GauXCError, match="Device execution space only"):
        g.XCIntegratorFactory(g.ExecutionSpace.Host).get_instance(func, lb)
    integ = g.XCIntegratorFactory(g.ExecutionSpace.Device).get_instance(func, lb)
    with pytest.raises(GauXCError, match="Same Dimension"):
        integ.eval_exc_vxc(np.eye(3))
    with pytest.raises(GauXCError, match="Square"):
        integ.eval_exc_vxc(np.zeros((2, 3)))
    with pytest.raises(GauXCError, match="Weights Have Not Been Modified"):
        integ.eval_exc_vxc(np.eye(2))


def test_device_paths_fail_loudly_without_gpu(g):
    if g.device_count() > 0:
        pytest.skip("a GPU is present")
    from gauxc_gb300._capi import GauXCError
    mol, basis, lb = _tiny_system(g)
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    with pytest.raises(GauXCError, match="no CUDA device"):
        mw.modify_weights(lb)
    with pytest.raises(GauXCError, match="no CUDA device"):
        _tiny_system(g, g.ExecutionSpace.Device)  # the Device load balancer screens on the GPU
    with pytest.raises(GauXCError, match="Weights Have Not Been Modified|no CUDA device"):
        g.LocalDeviceWorkDriver().create_device_data(lb)
    with pytest.raises(GauXCError, match="no CUDA device"):
        g.collocation(basis, np.zeros((4, 3)), [0, 1])


def test_pipeline_check_arguments(g):
    from gauxc_gb300 import workloads as W
    from gauxc_gb300._capi import GauXCError
    s = W.config(0)["systems"][0]
    mol, basis, mg, lb = W.build_system(s, device=False)
    integ = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default",
                                  "GB300-Mixed", "Default").get_instance(
                                      g.functional_type(s["functional"]), lb)
    integ.set_pipeline_check(wait_ms=2.0, withhold=True)
    integ.set_pipeline_check()
    for bad in (0.0, -1.0, 1e9):
        with pytest.raises(GauXCError, match="pipeline wait bound"):
            integ.set_pipeline_check(wait_ms=bad)


def test_load_balancer_subset_copies_tasks(g):
    from gauxc_gb300 import workloads as W
    from gauxc_gb300._capi import GauXCError
    s = W.config(5)["systems"][0]
    mol, basis, mg, lb = W.build_system(s, device=False)
    n = lb.ntasks()
    idx = [n - 1, 0, n // 2]
    sub = lb.subset(idx)
    assert sub.ntasks() == 3 and sub.weights_modified() == lb.weights_modified()
    for k, i in enumerate(idx):
        a, b = lb.task(i), sub.task(k)
        assert a["iParent"] == b["iParent"] and a["nbe"] == b["nbe"]
        assert np.array_equal(a["points"], b["points"])
        assert np.array_equal(a["weights"], b["weights"])
        assert np.array_equal(a["shell_list"], b["shell_list"])
    assert lb.subset([]).ntasks() == 0
    with pytest.raises(GauXCError, match="out of range"):
        lb.subset([n])


def test_null_status_raises_like_the_reference(g):
    """With a null GauXCStatus* a failure is thrown as a C++ exception
    (src/c-api/c_status.hpp:31-44); the compiled C++ walk-through in
    test_native_clients.py catches it.  From ctypes only the success path can
    pass a null status: it must return normally."""
    L = g.lib()
    m = L.gauxc_molecule_new(None)
    assert m.ptr
    assert L.gauxc_molecule_natoms(None, m) == 0
    L.gauxc_molecule_delete(None, ctypes.byref(m))
    assert not m.ptr


def test_spin_mismatch_errors(g):
    from gauxc_gb300 import workloads as W
    from gauxc_gb300._capi import GauXCError
    s = W.config(0)["systems"][0]
    mol, basis, mg, lb = W.build_system(s, device=False)
    f = g.XCIntegratorFactory(g.ExecutionSpace.Device)
    rks = f.get_instance(g.functional_type("SVWN5"), lb)
    uks = f.get_instance(g.functional_type("SVWN5", True), lb)
    P = s["P"]
    with pytest.raises(GauXCError, match="requires a polarized functional"):
        rks.eval_exc_vxc_uks(P, P)
    with pytest.raises(GauXCError, match="requires an unpolarized functional"):
        uks.eval_exc_vxc(P)
    with pytest.raises(GauXCError, match="Invalid LDP"):
        uks.eval_exc_vxc_uks(P, np.zeros((3, 3)))
    with pytest.raises(GauXCError, match="Same Dimension"):
        uks.eval_exc_vxc_uks(np.zeros((3, 3)), np.zeros((3, 3)))
