"""Setup on the device (needs a GB300): the Device load balancer's screening
kernel and the screened SSF kernel.

* Task lists: the Device load balancer (collision bitset on the GPU) must
  give the Host load balancer's task list exactly -- same tasks in the same
  order, same iParent, points, weights, shell lists, nbe, dist_nearest
  (the reference's tests/load_balancer_test.cxx compares host and device
  task lists the same way).
* SSF weights: the screened kernel (used by modify_weights) against the
  oracle's host algorithm (weights.cxx) and against the reference-order
  device kernel (cuda_ssf_1d.cu, the allocation-free entry point runs it).
"""
import ctypes
import time

import numpy as np
import pytest

import oracle
from conftest import golden
from helpers import benzene_system, flat_points

pytestmark = pytest.mark.gpu


def _same_tasks(a, b, idx=None):
    assert a.ntasks() == b.ntasks()
    for i in (range(a.ntasks()) if idx is None else idx):
        ta, tb = a.task(i), b.task(i)
        for k in ("iParent", "npts", "nbe", "nshells", "dist_nearest"):
            assert ta[k] == tb[k], (i, k)
        assert np.array_equal(ta["shell_list"], tb["shell_list"]), i
        assert np.array_equal(ta["points"], tb["points"]), i
        assert np.array_equal(ta["weights"], tb["weights"]), i


@pytest.mark.parametrize("tol", [np.finfo(float).eps, 1e-10])
def test_device_load_balancer_equals_host_benzene(g, tol):
    d, mol, basis, mg, lbd = benzene_system(g, "benzene_svwn5.npz", tol=tol, device=True)
    *_, lbh = benzene_system(g, "benzene_svwn5.npz", tol=tol, device=False)
    _same_tasks(lbd, lbh)


@pytest.mark.parametrize("idx", [1, 4])
def test_device_load_balancer_equals_host_workloads(g, idx):
    from gauxc_gb300 import workloads as W
    s = W.config(idx)["systems"][0]
    t0 = time.perf_counter()
    *_, lbd = W.build_system(s, device=True)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    *_, lbh = W.build_system(s, device=False)
    t_host = time.perf_counter() - t0
    n = lbh.ntasks()
    # every task of workload 1; a strided quarter of workload 4's 183k tasks
    _same_tasks(lbd, lbh, None if n < 50000 else range(0, n, 4))
    print(f"\nworkload {idx}: {n} tasks; build_system with the Device load balancer "
          f"{t_dev:.2f} s, with the Host one {t_host:.2f} s")


def test_screened_ssf_matches_golden_and_oracle(g):
    d = golden("benzene_weights_ssf.npz")
    w = g.ssf_weights(d["points"], d["iparent"], d["dist_nearest"], d["xyz"], d["w_unm"])
    assert np.all(np.abs(w - d["w_mod"]) <= 1e-12 * np.abs(d["w_mod"]) + 1e-300)


def _noalloc_weights(g, pts, ip, dn, coords, w0):
    """Reference-order kernel through the allocation-free entry point, in
    pieces that fit its fixed work space."""
    torch = pytest.importorskip("torch")
    from gauxc_gb300._capi import GauXCStatus, check
    L = g.lib()
    natoms = len(coords)
    per = max(1, (1 << 22) // natoms - natoms)
    dev = torch.device("cuda")
    co = torch.tensor(np.ascontiguousarray(coords).reshape(-1), dtype=torch.float64, device=dev)
    out = np.empty_like(w0)
    st = GauXCStatus()
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    for a in range(0, len(w0), per):
        b = min(len(w0), a + per)
        x, y, z = (torch.tensor(pts[a:b, k].copy(), dtype=torch.float64, device=dev)
                   for k in range(3))
        ipt = torch.tensor(ip[a:b], dtype=torch.int32, device=dev)
        dnt = torch.tensor(dn[a:b], dtype=torch.float64, device=dev)
        wt = torch.tensor(w0[a:b], dtype=torch.float64, device=dev)
        L.gauxc_gb300_ssf_weights_noalloc(ctypes.byref(st), b - a, natoms, vp(x), vp(y), vp(z),
                                          vp(ipt), vp(dnt), vp(co), vp(wt), None)
        check(st, L)
        torch.cuda.synchronize()
        out[a:b] = wt.cpu().numpy()
    return out


def test_screened_ssf_on_256_waters(g):
    """Screened kernel vs the host algorithm and the reference-order kernel on
    a strided sample of workload 4's points (768 atoms, every 400th task:
    23,060 points).  Cell products truncated at 1e-13 in different orders
    differ where a point's cell products sum to little; measured on the CPU
    (emulation of both kernels on these points): reference order vs host
    algorithm up to 3.5e-9 of the weight, screened vs host 6.2e-9, screened vs
    reference order 2.7e-9."""
    from gauxc_gb300 import workloads as W
    s = W.config(4)["systems"][0]
    mol, basis, mg, lb = W.build_system(s, device=False)
    tasks = [lb.task(i) for i in range(0, lb.ntasks(), 400)]
    pts, w0, ip, dn = flat_points(tasks)
    co = mol.coords()
    t0 = time.perf_counter()
    ws = g.ssf_weights(pts, ip, dn, co, w0)
    t_s = time.perf_counter() - t0
    wo = oracle.ssf_weights(pts, ip, dn, co, w0)
    wr = _noalloc_weights(g, pts, ip, dn, co, w0)
    assert np.all(np.abs(ws - wo) <= 1e-8 * np.abs(w0))
    assert np.all(np.abs(wr - wo) <= 1e-8 * np.abs(w0))
    assert np.all(np.abs(ws - wr) <= 1e-8 * np.abs(w0))
    # the bulk agrees far more closely than the worst points
    assert np.median(np.abs(ws - wo) / np.abs(w0)) <= 1e-14
    print(f"\n{len(w0)} points: screened SSF {t_s:.3f} s (with transfers); max rel. diff "
          f"screened/host {np.max(np.abs(ws - wo) / np.abs(w0)):.2e}, reference-order/host "
          f"{np.max(np.abs(wr - wo) / np.abs(w0)):.2e}")


def test_modify_weights_on_device_load_balancer(g):
    """Device load balancer + device SSF (the whole setup on the GPU path)
    against the host load balancer's tasks weighted by the oracle."""
    d, mol, basis, mg, lb = benzene_system(g, "benzene_svwn5.npz", grid="FineGrid", device=True)
    tasks0 = lb.get_tasks()
    g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
    pts, w0, ip, dn = flat_points(tasks0)
    wo = oracle.ssf_weights(pts, ip, dn, mol.coords(), w0)
    wd = np.concatenate([t["weights"] for t in lb.get_tasks()])
    assert np.all(np.abs(wd - wo) <= 5e-12 * np.abs(w0))
