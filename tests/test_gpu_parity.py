"""Device path against the oracle and the reference goldens (needs a GB300).

Gates (the target tolerances of the plain FP64 path):
  |dEXC| <= 1e-10 Eh and max |dVXC_ij| <= 1e-10 against the FP64 oracle,
  SSF weights and collocation to ~1e-13 relative, task maps bit-exact.
"""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import golden
from helpers import benzene_system, flat_points, oracle_basis, oracle_exc_vxc, oracle_ssf_tasks

pytestmark = pytest.mark.gpu

TOL_EXC = 1e-10
TOL_VXC = 1e-10


def test_ssf_device_matches_golden(g):
    d = golden("benzene_weights_ssf.npz")
    w = g.ssf_weights(d["points"], d["iparent"], d["dist_nearest"], d["xyz"], d["w_unm"])
    ref = d["w_mod"]
    assert np.all(np.abs(w - ref) <= 1e-12 * np.abs(ref) + 1e-300)


def test_ssf_device_matches_oracle_on_tasks(g):
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", grid="FineGrid")
    pts, w, ip, dn = flat_points(lb.get_tasks())
    wd = g.ssf_weights(pts, ip, dn, mol.coords(), w)
    wo = oracle.ssf_weights(pts, ip, dn, mol.coords(), w)
    # the device kernel truncates each cell product at 1e-13 on its own
    # (cuda_ssf_1d.cu) while the host algorithm updates cell pairs
    # (weights.cxx); the two agree to ~1e-12 of the unmodified weight
    assert np.all(np.abs(wd - wo) <= 5e-12 * np.abs(w))


def test_collocation_device_matches_golden(g):
    raw = golden("ccpvdz_raw.npz")
    c = golden("water_collocation.npz")
    shells = []
    for Z, x in zip(c["Z"], c["xyz"]):
        sym = {1: "H", 8: "O"}[int(Z)]
        for k in range(len(raw[sym + "_l"])):
            n = raw[sym + "_nprim"][k]
            l = int(raw[sym + "_l"][k])
            shells.append(g.Shell(l, raw[sym + "_alpha"][k, :n], raw[sym + "_coeff"][k, :n], x,
                                  pure=l > 1))
    basis = g.BasisSet(shells, normalize=True)
    for i in range(int(c["nentries"][0])):
        outs = g.collocation(basis, c[f"pts_{i}"], c[f"mask_{i}"], grad=True)
        for got, key in zip(outs, ("eval", "deval_x", "deval_y", "deval_z")):
            ref = c[f"{key}_{i}"].reshape(got.shape)
            assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("pure", [True, False])
def test_collocation_device_matches_oracle_up_to_g(g, pure):
    rng = np.random.default_rng(3)
    shells = [g.Shell(l, rng.uniform(0.1, 5.0, 2), rng.uniform(-1, 1, 2),
                      rng.uniform(-1, 1, 3), pure=pure) for l in range(5) for _ in range(2)]
    basis = g.BasisSet(shells)
    pts = rng.uniform(-3, 3, (200, 3))
    sl = np.arange(len(shells), dtype=np.int32)
    dev = g.collocation(basis, pts, sl, grad=True)
    ref = oracle.collocation(oracle_basis(basis), pts, sl, grad=True)
    for a, b in zip(dev, ref):
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def _device_integrator(g, lb, func, lwd="Default"):
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    mw.modify_weights(lb)
    return g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                 "Default").get_instance(g.functional_type(func), lb)


@pytest.mark.parametrize("fname,func,prune", [
    ("benzene_svwn5.npz", "SVWN5", "Unpruned"),
    ("benzene_svwn5_treutler.npz", "SVWN5", "Treutler"),
    ("benzene_pbe0.npz", "PBE0", "Unpruned"),
])
def test_exc_vxc_fp64_matches_oracle_and_golden(g, fname, func, prune):
    d, mol, basis, mg, lb = benzene_system(g, fname, prune=prune)
    tasks0 = lb.get_tasks()
    integ = _device_integrator(g, lb, func)
    exc, vxc = integ.eval_exc_vxc(d["P"])
    # oracle on the same task list with its own (host-algorithm) SSF weights
    eo, Vo, no = oracle.eval_exc_vxc(oracle_basis(basis), oracle_ssf_tasks(tasks0, mol.coords()),
                                     d["P"], func)
    print(f"\n[parity] benzene {func} {prune} FP64: vs oracle |dEXC| {abs(exc - eo):.2e} "
          f"max|dVXC| {np.abs(vxc - Vo).max():.2e}; vs golden |dEXC| {abs(exc - d['EXC'][0]):.2e} "
          f"|dVXC|/nbf {np.linalg.norm(vxc - d['VXC']) / len(vxc):.2e}")
    assert abs(exc - eo) <= TOL_EXC
    assert np.abs(vxc - Vo).max() <= TOL_VXC
    assert abs(integ.last_nel() - no) <= 1e-10
    # and against the reference's own numbers
    assert abs(exc - d["EXC"][0]) <= 1e-9
    assert np.linalg.norm(vxc - d["VXC"]) / len(vxc) <= 1e-11
    # second call reproduces (state propagation, tests/xc_integrator.cxx:206-211)
    exc1, vxc1 = integ.eval_exc_vxc(d["P"])
    assert abs(exc1 - exc) <= 1e-12 and np.abs(vxc1 - vxc).max() <= 1e-12
    # EXC-only path
    assert abs(integ.eval_exc(d["P"]) - exc) <= 1e-12


def test_integrate_den_and_weights_device(g):
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", grid="FineGrid")
    tasks0 = lb.get_tasks()
    integ = _device_integrator(g, lb, "SVWN5")
    assert lb.weights_modified()
    # device SSF weights stored in the tasks equal the oracle's
    wd = np.concatenate([t["weights"] for t in lb.get_tasks()])
    wo = np.concatenate([t[1] for t in oracle_ssf_tasks(tasks0, mol.coords())])
    w0 = np.concatenate([t["weights"] for t in tasks0])
    assert np.all(np.abs(wd - wo) <= 5e-12 * np.abs(w0))
    n = integ.integrate_den(d["P"])
    assert abs(n - 21.0) < 1e-4  # alpha electrons (tests/xc_integrator.cxx:190-196)


def test_water_config0_fp64(g):
    from gauxc_gb300 import workloads as W
    s = W.config(0)["systems"][0]
    mol, basis, mg, lb = W.build_system(s)
    tasks0 = lb.get_tasks()
    integ = _device_integrator(g, lb, s["functional"])
    exc, vxc = integ.eval_exc_vxc(s["P"])
    eo, Vo, _ = oracle.eval_exc_vxc(oracle_basis(basis), oracle_ssf_tasks(tasks0, mol.coords()),
                                    s["P"], s["functional"])
    assert abs(exc - eo) <= TOL_EXC
    assert np.abs(vxc - Vo).max() <= TOL_VXC


def test_caller_owned_device_memory(g):
    """DeviceRuntimeEnvironment over a caller buffer (gauxc_device_runtime_environment_new_mem)."""
    torch = pytest.importorskip("torch")
    buf = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    d = golden("benzene_svwn5.npz")
    mol = g.Molecule([(int(Z), *x) for Z, x in zip(d["Z"], d["xyz"])])
    shells = [g.Shell(int(d["sh_l"][i]), d["sh_alpha"][i, :d["sh_nprim"][i]],
                      d["sh_coeff"][i, :d["sh_nprim"][i]], d["sh_origin"][i],
                      bool(d["sh_pure"][i])) for i in range(len(d["sh_l"]))]
    basis = g.BasisSet(shells, normalize=False)
    mg = g.MolGridFactory.create_default_molgrid(mol, g.PruningScheme.Treutler, 512,
                                                 g.RadialQuad.MuraKnowles,
                                                 g.AtomicGridSizeDefault.FineGrid)
    rt = g.DeviceRuntimeEnvironment(mem=(buf.data_ptr(), buf.numel()))
    lb = g.LoadBalancerFactory(g.ExecutionSpace.Device).get_instance(rt, mol, mg, basis)
    tasks0 = lb.get_tasks()
    integ = _device_integrator(g, lb, "SVWN5")
    exc, vxc = integ.eval_exc_vxc(d["P"])
    eo, Vo, _ = oracle.eval_exc_vxc(oracle_basis(basis), oracle_ssf_tasks(tasks0, mol.coords()),
                                    d["P"], "SVWN5")
    assert abs(exc - eo) <= TOL_EXC and np.abs(vxc - Vo).max() <= TOL_VXC
    torch.cuda.synchronize()
