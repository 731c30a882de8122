"""Batched evaluation (one CUDA-graph launch over many integrators) and the
plan autotuner (needs a GB300).

A batch must reproduce its members' one-by-one results: the graph replays the
same kernels, so FP64 members agree to rounding of the FP64 atomics
(1e-11 here) and mixed members stay within the mixed-path gate (1e-8) of the
FP64 results.
"""
import numpy as np
import pytest

from gauxc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL_SAME = 1e-11
TOL_MIXED = 1e-8


def _systems(g, count=6):
    """The first `count` clusters of the batched workload (mixed sizes, half
    SVWN5 and half PBE, point-batch sizes 128-1024), with SSF weights."""
    out = []
    for s in W.config(3)["systems"][:count]:
        mol, basis, mg, lb = W.build_system(s)
        g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
        out.append((s, lb, (mol, basis, mg)))
    return out


def _integrator(g, s, lb, lwd):
    return g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default", lwd,
                                 "Default").get_instance(g.functional_type(s["functional"]), lb)


@pytest.fixture(scope="module")
def members(g):
    sys = _systems(g)
    rows = []
    for s, lb, keep in sys:
        P = np.asfortranarray(s["P"])
        i64 = _integrator(g, s, lb, "GB300-FP64")
        imx = _integrator(g, s, lb, "GB300-Mixed")
        e64, v64 = i64.eval_exc_vxc(P)
        rows.append(dict(s=s, lb=lb, keep=keep, P=P, i64=i64, imx=imx, e64=e64, v64=v64))
    return rows


def test_batch_matches_members(g, members):
    integs = [r["i64"] for r in members] + [r["imx"] for r in members]
    Ps = [r["P"] for r in members] * 2
    Vs = [np.zeros_like(r["P"], order="F") for r in members + members]
    batch = g.IntegratorBatch(integs)
    n = len(members)
    for call in range(3):
        for V in Vs:
            V[:] = 0.
        exc = batch.eval_exc_vxc(Ps, Vs)
        t = batch.timings()
        assert t["graph_launch"] == (0.0 if call == 0 else 1.0)
        for k, r in enumerate(members):
            assert abs(exc[k] - r["e64"]) <= TOL_SAME
            assert np.abs(Vs[k] - r["v64"]).max() <= TOL_SAME
            assert abs(exc[n + k] - r["e64"]) <= TOL_MIXED
            assert np.abs(Vs[n + k] - r["v64"]).max() <= TOL_MIXED
    assert t["members"] == 2 * n and t["compute_ms"] > 0.


def test_batch_exc_only_and_new_buffers(g, members):
    rows = members[:3]
    batch = g.IntegratorBatch([r["i64"] for r in rows])
    exc = batch.eval_exc_vxc([r["P"] for r in rows], [None] * len(rows))
    for k, r in enumerate(rows):
        assert abs(exc[k] - r["e64"]) <= TOL_SAME
    # other arrays: the batch recaptures (first call plain), then replays
    Ps = [np.asfortranarray(r["P"].copy()) for r in rows]
    Vs = [np.zeros_like(r["P"], order="F") for r in rows]
    for call in range(2):
        exc = batch.eval_exc_vxc(Ps, Vs)
        assert batch.timings()["graph_launch"] == (0.0 if call == 0 else 1.0)
        for k, r in enumerate(rows):
            assert abs(exc[k] - r["e64"]) <= TOL_SAME
            assert np.abs(Vs[k] - r["v64"]).max() <= TOL_SAME


def test_autotune_keeps_results(g, members):
    r = members[-1]
    ms, params = r["imx"].autotune(r["P"])
    assert ms > 0.
    assert params["pb_max_pts"] in (128, 256, 384)
    assert params["nu2_weight"] in (75.0, 150.0)
    e, v = r["imx"].eval_exc_vxc(r["P"])
    assert abs(e - r["e64"]) <= TOL_MIXED
    assert np.abs(v - r["v64"]).max() <= TOL_MIXED


def test_plan_params_validated(g, members):
    from gauxc_gb300._capi import GauXCError
    r = members[0]
    with pytest.raises(GauXCError):
        r["imx"].set_plan_params(pb_max_pts=1024)
    r["imx"].set_plan_params(pb_max_pts=128, nu2_weight=100.0)
    e, v = r["imx"].eval_exc_vxc(r["P"])
    assert abs(e - r["e64"]) <= TOL_MIXED


def test_host_register_keeps_results(g, members):
    """P page-locked in place through the library gives the same results."""
    r = members[1]
    P = np.asfortranarray(r["P"].copy())
    g.host_register(P)
    try:
        assert g.host_register(P) is False  # already page-locked
        e, v = r["i64"].eval_exc_vxc(P)
    finally:
        g.host_unregister(P)
    assert abs(e - r["e64"]) <= TOL_SAME
    assert np.abs(v - r["v64"]).max() <= TOL_SAME
