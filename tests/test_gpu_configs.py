"""Device paths against the oracle on the benchmark workloads (needs a GB300).

Workloads 1, 2 and 4 (32, 96 and 256 waters) are evaluated on a deterministic
sample of their tasks: every k-th task of the list ordered by npts * nbe
(the reference's cost order), kept in load-balancer order, so heavy and light
tasks both appear and the mixed path still merges neighbouring tasks of an
atom.  The sample is a load balancer of its own (gauxc_gb300_load_balancer_subset),
its SSF weights come from the device, and the oracle integrates the same
tasks with those weights.  Workload 3 (64 clusters) is checked on whole
members, one SVWN5 and one PBE, directly and through the batched one-graph
path.

Gates (the reference's own check is tests/xc_integrator.cxx:199-216):
  FP64 path  |dEXC| <= 1e-10 Eh, max |dVXC_ij| <= 1e-10, |dN_el| <= 1e-10
  mixed path |dEXC| <= 1e-8 Eh,  max |dVXC_ij| <= 1e-8,  |dN_el| <= 1e-8
"""
import numpy as np
import pytest

import oracle
from helpers import flat_points, oracle_basis

pytestmark = pytest.mark.gpu

GATES = {"GB300-FP64": 1e-10, "GB300-Mixed": 1e-8}
_CACHE = {}


def _sample(lb, n):
    infos = [lb.task_info(i) for i in range(lb.ntasks())]
    order = sorted(range(len(infos)), key=lambda i: -infos[i]["npts"] * infos[i]["nbe"])
    stride = max(1, len(order) // n)
    return sorted(order[::stride][:n])


def _system(g, idx, ntasks):
    """(system dict, molecule, basis, weighted sample load balancer, oracle result)."""
    key = (idx, ntasks)
    if key not in _CACHE:
        from gauxc_gb300 import workloads as W
        s = W.config(idx)["systems"][0]
        mol, basis, mg, lb = W.build_system(s)
        sub = lb.subset(_sample(lb, ntasks))
        tasks0 = sub.get_tasks()
        g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(sub)
        tasks = sub.get_tasks()
        # device SSF weights of the sample against the oracle's host algorithm
        # (weights.cxx).  Cell products are truncated at 1e-13, and where the
        # sum of a point's cell products is small the truncation order shows:
        # on 23,060 points of 256 waters (CPU emulation of both kernels) the
        # reference's device kernel (atom-index order, cuda_ssf_1d.cu) lands
        # up to 3.5e-9 of the weight away from the host algorithm and this
        # build's screened kernel (nearest atoms first) up to 6.2e-9; the
        # reference's own check is Catch's default Approx, 1.2e-5 relative
        # (tests/weights_cuda.hpp:115).
        pts, w0, ip, dn = flat_points(tasks0)
        wo = oracle.ssf_weights(pts, ip, dn, mol.coords(), w0)
        wd = np.concatenate([t["weights"] for t in tasks])
        assert np.all(np.abs(wd - wo) <= 1e-8 * np.abs(w0))
        ref = oracle.eval_exc_vxc(oracle_basis(basis),
                                  [(t["points"], t["weights"], t["shell_list"]) for t in tasks],
                                  s["P"], s["functional"])
        _CACHE.clear()  # one large system held at a time
        _CACHE[key] = (s, mol, basis, sub, ref)
    return _CACHE[key]


@pytest.mark.parametrize("idx,ntasks,lwd", [
    (1, 240, "GB300-FP64"),
    (1, 240, "GB300-Mixed"),
    (2, 200, "GB300-Mixed"),
    (4, 120, "GB300-FP64"),
    (4, 120, "GB300-Mixed"),
])
def test_workload_sample_matches_oracle(g, idx, ntasks, lwd):
    s, mol, basis, lb, (eo, Vo, no) = _system(g, idx, ntasks)
    integ = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                  "Default").get_instance(g.functional_type(s["functional"]), lb)
    exc, vxc = integ.eval_exc_vxc(s["P"])
    tol = GATES[lwd]
    print(f"\n[parity] workload {idx} ({lb.ntasks()} sampled tasks) {lwd}: |dEXC| "
          f"{abs(exc - eo):.2e} max|dVXC| {np.abs(vxc - Vo).max():.2e} "
          f"|dN_el| {abs(integ.last_nel() - no):.2e}")
    assert abs(exc - eo) <= tol, (exc, eo)
    assert np.abs(vxc - Vo).max() <= tol
    assert abs(integ.last_nel() - no) <= tol
    # the EXC-only pass and integrate_den agree with the same pass
    assert abs(integ.eval_exc(s["P"]) - exc) <= 1e-12
    assert abs(integ.integrate_den(s["P"]) - 0.5 * no) <= tol


def _members(cfg):
    """Indices of the smallest SVWN5 and the smallest PBE member with >= 3 waters."""
    out = {}
    for i, s in enumerate(cfg["systems"]):
        if s["n_water"] < 3:
            continue
        f = s["functional"]
        if f not in out or s["n_water"] < cfg["systems"][out[f]]["n_water"]:
            out[f] = i
    return [out["SVWN5"], out["PBE"]]


def test_workload3_members_match_oracle(g):
    from gauxc_gb300 import workloads as W
    cfg = W.config(3)
    mw = g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance()
    systems, refs = [], []
    for k in _members(cfg):
        s = cfg["systems"][k]
        mol, basis, mg, lb = W.build_system(s)
        mw.modify_weights(lb)
        tasks = lb.get_tasks()
        refs.append(oracle.eval_exc_vxc(oracle_basis(basis),
                                        [(t["points"], t["weights"], t["shell_list"]) for t in tasks],
                                        s["P"], s["functional"]))
        systems.append((s, lb))
    for lwd, tol in GATES.items():
        f = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd, "Default")
        integs = [f.get_instance(g.functional_type(s["functional"]), lb) for s, lb in systems]
        for integ, (s, lb), (eo, Vo, no) in zip(integs, systems, refs):
            exc, vxc = integ.eval_exc_vxc(s["P"])
            print(f"\n[parity] workload 3 member ({s['n_water']} waters, {s['functional']}) "
                  f"{lwd}: |dEXC| {abs(exc - eo):.2e} max|dVXC| {np.abs(vxc - Vo).max():.2e}")
            assert abs(exc - eo) <= tol and np.abs(vxc - Vo).max() <= tol
            assert abs(integ.last_nel() - no) <= tol
        # the batched path: first call captures the graph, the second replays it
        batch = g.IntegratorBatch(integs)
        Ps = [np.asfortranarray(s["P"]) for s, _ in systems]
        Vs = [np.zeros_like(P, order="F") for P in Ps]
        for _ in range(2):
            excs = batch.eval_exc_vxc(Ps, Vs)
            for e, V, (eo, Vo, no) in zip(excs, Vs, refs):
                assert abs(e - eo) <= tol and np.abs(V - Vo).max() <= tol
        assert batch.timings()["graph_launch"] == 1.0
        del batch
