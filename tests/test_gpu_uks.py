"""UKS (spin-polarized) EXC / VXC on the device (needs a GB300).

* cytosine doublet, SVWN5, cc-pVDZ, UltraFine grid with Robust pruning, tol =
  eps: the reference's UKS golden (tests/xc_integrator.cxx:455-458) and the
  oracle on the same task list;
* closed shell through UKS (Ps = 2 P, Pz = 0) equals RKS;
* an open-shell PBE density (4 waters) against the oracle.
Gates: FP64 path 1e-10 (EXC, every VXC element), mixed path 1e-8; against
the golden the reference's own tolerances (EXC rel 1.2e-5 -- here 5e-9 Eh --
and ||dVXC||_F / nbf < 1e-10).
"""
import numpy as np
import pytest

import oracle
from helpers import benzene_system, oracle_basis, oracle_ssf_tasks

pytestmark = pytest.mark.gpu

GATES = {"GB300-FP64": 1e-10, "GB300-Mixed": 1e-8}
_CACHE = {}


def _integ(g, lb, func, lwd, polarized=True):
    return g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                 "Default").get_instance(g.functional_type(func, polarized), lb)


def _cytosine(g):
    if "cyt" not in _CACHE:
        d, mol, basis, mg, lb = benzene_system(g, "cytosine_svwn5_uks.npz", prune="Robust")
        tasks0 = lb.get_tasks()
        g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
        ref = oracle.eval_exc_vxc_uks(oracle_basis(basis), oracle_ssf_tasks(tasks0, mol.coords()),
                                      d["Ps"], d["Pz"], "SVWN5")
        _CACHE["cyt"] = (d, lb, ref)
    return _CACHE["cyt"]


@pytest.mark.parametrize("lwd", ["GB300-FP64", "GB300-Mixed"])
def test_uks_svwn5_cytosine(g, lwd):
    d, lb, (eo, Vso, Vzo, no) = _cytosine(g)
    integ = _integ(g, lb, "SVWN5", lwd)
    exc, Vs, Vz = integ.eval_exc_vxc_uks(d["Ps"], d["Pz"])
    tol = GATES[lwd]
    nbf = len(Vs)
    print(f"\n[parity] UKS cytosine SVWN5 {lwd}: vs oracle |dEXC| {abs(exc - eo):.2e} "
          f"max|dVXC_s| {np.abs(Vs - Vso).max():.2e} max|dVXC_z| {np.abs(Vz - Vzo).max():.2e}; "
          f"vs golden |dEXC| {abs(exc - d['EXC'][0]):.2e} "
          f"|dVXC_s|/nbf {np.linalg.norm(Vs - d['VXCs']) / nbf:.2e} "
          f"|dVXC_z|/nbf {np.linalg.norm(Vz - d['VXCz']) / nbf:.2e}")
    assert abs(exc - eo) <= tol
    assert np.abs(Vs - Vso).max() <= tol and np.abs(Vz - Vzo).max() <= tol
    assert abs(integ.last_nel() - no) <= tol
    nbf = len(Vs)
    assert abs(exc - d["EXC"][0]) <= 5e-9
    assert np.linalg.norm(Vs - d["VXCs"]) / nbf <= 1e-10
    assert np.linalg.norm(Vz - d["VXCz"]) / nbf <= 1e-10
    assert abs(integ.eval_exc_uks(d["Ps"], d["Pz"]) - exc) <= 1e-12
    # a second call reproduces the first
    exc2, Vs2, Vz2 = integ.eval_exc_vxc_uks(d["Ps"], d["Pz"])
    assert abs(exc2 - exc) <= 1e-12 and np.abs(Vs2 - Vs).max() <= 1e-12


def _waters(g):
    if "w" not in _CACHE:
        from gauxc_gb300 import workloads as W
        s = W.config(5)["systems"][0]
        mol, basis, mg, lb = W.build_system(s)
        tasks0 = lb.get_tasks()
        g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
        rng = np.random.default_rng(17)
        n = s["nbf"]
        Ca = rng.standard_normal((n, 11)) / np.sqrt(n)
        Cb = Ca[:, :9] + 0.05 * rng.standard_normal((n, 9)) / np.sqrt(n)
        Pa, Pb = Ca @ Ca.T, Cb @ Cb.T
        Ps, Pz = np.asfortranarray(Pa + Pb), np.asfortranarray(Pa - Pb)
        ob = oracle_basis(basis)
        ot = oracle_ssf_tasks(tasks0, mol.coords())
        _CACHE["w"] = (s, lb, Ps, Pz, oracle.eval_exc_vxc_uks(ob, ot, Ps, Pz, "PBE"),
                       oracle.eval_exc_vxc(ob, ot, s["P"], "PBE"))
    return _CACHE["w"]


@pytest.mark.parametrize("lwd", ["GB300-FP64", "GB300-Mixed"])
def test_uks_pbe_open_shell(g, lwd):
    s, lb, Ps, Pz, (eo, Vso, Vzo, no), _ = _waters(g)
    exc, Vs, Vz = _integ(g, lb, "PBE", lwd).eval_exc_vxc_uks(Ps, Pz)
    tol = GATES[lwd]
    print(f"\n[parity] UKS 4 waters PBE open shell {lwd}: |dEXC| {abs(exc - eo):.2e} "
          f"max|dVXC_s| {np.abs(Vs - Vso).max():.2e} max|dVXC_z| {np.abs(Vz - Vzo).max():.2e}")
    assert abs(exc - eo) <= tol
    assert np.abs(Vs - Vso).max() <= tol and np.abs(Vz - Vzo).max() <= tol


@pytest.mark.parametrize("lwd", ["GB300-FP64", "GB300-Mixed"])
def test_uks_closed_shell_equals_rks(g, lwd):
    s, lb, _, _, _, (e_rks, V_rks, _) = _waters(g)
    P = s["P"]
    exc, Vs, Vz = _integ(g, lb, "PBE", lwd).eval_exc_vxc_uks(2 * P, np.zeros_like(P))
    tol = GATES[lwd]
    assert abs(exc - e_rks) <= tol
    assert np.abs(Vs - V_rks).max() <= tol
    assert np.abs(Vz).max() <= tol
