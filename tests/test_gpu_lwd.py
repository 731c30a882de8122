"""The stage-level work driver (needs a GB300): the reference's
LocalDeviceWorkDriver stages composed in the reference integrator's order
(incore_replicated_xc_device_integrator_exc_vxc.hpp:283-404) must give the
oracle's EXC / VXC / N_el at the FP64 gates (1e-10), and the fused integrator's
result; device data over two halves of the task list add up to the whole."""
import numpy as np
import pytest

import oracle
from helpers import benzene_system, oracle_basis, oracle_ssf_tasks

pytestmark = pytest.mark.gpu


def _stages(g, lb, func, P, gga, t0=0, t1=None):
    lwd = g.LocalDeviceWorkDriver()
    d = lwd.create_device_data(lb, t0, t1)
    if gga:
        lwd.eval_collocation_gradient(d)
    else:
        lwd.eval_collocation(d)
    lwd.eval_xmat(2.0, d, P)  # RKS: P is the alpha density
    if gga:
        lwd.eval_vvars_gga(d)
        lwd.eval_uvars_gga(d)
        lwd.eval_kern_exc_vxc_gga(func, d)
    else:
        lwd.eval_vvars_lda(d)
        lwd.eval_kern_exc_vxc_lda(func, d)
    lwd.inc_exc(d)
    lwd.inc_nel(d)
    if gga:
        lwd.eval_zmat_gga_vxc(d)
    else:
        lwd.eval_zmat_lda_vxc(d)
    lwd.inc_vxc(d)
    V = lwd.symmetrize_vxc(d)
    e, n = lwd.results(d)
    return e, V, n


@pytest.mark.parametrize("fname,func,gga", [("benzene_svwn5.npz", "SVWN5", False),
                                            ("benzene_pbe0.npz", "PBE0", True)])
def test_stages_match_oracle_and_integrator(g, fname, func, gga):
    d, mol, basis, mg, lb = benzene_system(g, fname, grid="FineGrid")
    tasks0 = lb.get_tasks()
    g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
    f = g.functional_type(func)
    e, V, n = _stages(g, lb, f, d["P"], gga)
    eo, Vo, no = oracle.eval_exc_vxc(oracle_basis(basis), oracle_ssf_tasks(tasks0, mol.coords()),
                                     d["P"], func)
    print(f"\n[parity] stage driver benzene {func}: |dEXC| {abs(e - eo):.2e} "
          f"max|dVXC| {np.abs(V - Vo).max():.2e} |dN_el| {abs(n - no):.2e}")
    assert abs(e - eo) <= 1e-10 and np.abs(V - Vo).max() <= 1e-10 and abs(n - no) <= 1e-10
    ei, Vi = g.XCIntegratorFactory(g.ExecutionSpace.Device).get_instance(f, lb).eval_exc_vxc(d["P"])
    assert abs(e - ei) <= 1e-11 and np.abs(V - Vi).max() <= 1e-11
    # two device-data objects over the halves of the task list
    h = lb.ntasks() // 2
    e1, V1, n1 = _stages(g, lb, f, d["P"], gga, 0, h)
    e2, V2, n2 = _stages(g, lb, f, d["P"], gga, h, lb.ntasks())
    assert abs(e1 + e2 - e) <= 1e-11 and np.abs(V1 + V2 - V).max() <= 1e-11


def test_stage_order_errors(g):
    from gauxc_gb300._capi import GauXCError
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", grid="FineGrid")
    lwd = g.LocalDeviceWorkDriver()
    with pytest.raises(GauXCError, match="Weights Have Not Been Modified"):
        lwd.create_device_data(lb)
    g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
    with pytest.raises(GauXCError, match="task range"):
        lwd.create_device_data(lb, 0, lb.ntasks() + 1)
    dd = lwd.create_device_data(lb, 0, 4)
    lwd.eval_collocation(dd)
    with pytest.raises(GauXCError, match="gradient"):
        lwd.eval_vvars_gga(dd)
    with pytest.raises(GauXCError, match="unpolarized"):
        lwd.eval_kern_exc_vxc_lda(g.functional_type("SVWN5", True), dd)
