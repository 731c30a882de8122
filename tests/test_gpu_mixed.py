"""Mixed-precision (tensor-core, split-mantissa) path against FP64 (needs a GB300).

Gates for the mixed path: |dEXC| <= 1e-8 Eh and max |dVXC_ij| <= 1e-8 against
the FP64 oracle / the FP64 device path on the same inputs.
"""
import numpy as np
import pytest

import oracle
from helpers import benzene_system, oracle_basis, oracle_ssf_tasks

pytestmark = pytest.mark.gpu

TOL_EXC = 1e-8
TOL_VXC = 1e-8


@pytest.mark.parametrize("n,k", [(128, 64), (256, 256), (384, 192)])
def test_tensor_core_gemm_selftest(g, n, k):
    # symmetric VXC GEMM, 6 digits x 7 bits, pairs up to level 7: about 2^-42
    # relative per product term
    assert g.tensor_core_selftest(n, k) <= 1e-11


def test_float_float_exp_selftest(g):
    # table-driven exp of the collocation (Tang's method, 2^(j/32) table,
    # degree-5 polynomial on |r| <= ln2/64): about 2^-46 relative; the
    # float-float input itself carries 2^-48 of |x| <= 50
    assert g.ff_exp_selftest() <= 1e-13


def _integrator(g, lb, func, lwd):
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    if not lb.weights_modified():
        mw.modify_weights(lb)
    return g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                 "Default").get_instance(g.functional_type(func), lb)


@pytest.mark.parametrize("fname,func", [("benzene_svwn5.npz", "SVWN5"),
                                        ("benzene_pbe0.npz", "PBE0")])
def test_mixed_matches_oracle(g, fname, func):
    d, mol, basis, mg, lb = benzene_system(g, fname, grid="FineGrid")
    tasks0 = lb.get_tasks()
    integ = _integrator(g, lb, func, "GB300-Mixed")
    exc, vxc = integ.eval_exc_vxc(d["P"])
    eo, Vo, no = oracle.eval_exc_vxc(oracle_basis(basis), oracle_ssf_tasks(tasks0, mol.coords()),
                                     d["P"], func)
    print(f"\n[parity] benzene {func} mixed: |dEXC| {abs(exc - eo):.2e} "
          f"max|dVXC| {np.abs(vxc - Vo).max():.2e}")
    assert abs(exc - eo) <= TOL_EXC
    assert np.abs(vxc - Vo).max() <= TOL_VXC
    assert abs(integ.last_nel() - no) <= 1e-8
    exc2, vxc2 = integ.eval_exc_vxc(d["P"])
    assert abs(exc2 - exc) <= 1e-12


def test_mixed_matches_fp64_device_water_cluster(g):
    from gauxc_gb300 import workloads as W
    s = W.config(5)["systems"][0]
    mol, basis, mg, lb = W.build_system(s)
    i64 = _integrator(g, lb, s["functional"], "GB300-FP64")
    imx = _integrator(g, lb, s["functional"], "GB300-Mixed")
    e64, v64 = i64.eval_exc_vxc(s["P"])
    emx, vmx = imx.eval_exc_vxc(s["P"])
    assert abs(emx - e64) <= TOL_EXC
    assert np.abs(vmx - v64).max() <= TOL_VXC
