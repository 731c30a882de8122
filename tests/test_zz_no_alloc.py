"""The allocation-free SSF entry point (gauxc_gb300_ssf_weights_noalloc).

It serves callers that cannot allocate device memory when they need weights,
e.g. a host program whose own memory pool already holds the GPU.  The caller
owns every input and output on the device; the entry point's work space is a
fixed array inside the library.  Two calls in a row must reproduce the
allocating entry point (gauxc_gb300_ssf_weights) on the same inputs, and a
request larger than the fixed work space must be rejected before any work.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _dptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_ssf_noalloc_matches_allocating_entry_point(g):
    torch = pytest.importorskip("torch")
    from gauxc_gb300._capi import GauXCStatus, GauXCError, check
    L = g.lib()
    d = golden("benzene_weights_ssf.npz")
    pts = np.ascontiguousarray(d["points"])
    n, natoms = len(pts), len(d["xyz"])
    ref = g.ssf_weights(pts, d["iparent"], d["dist_nearest"], d["xyz"], d["w_unm"])

    dev = torch.device("cuda")
    x = torch.tensor(pts[:, 0], dtype=torch.float64, device=dev)
    y = torch.tensor(pts[:, 1], dtype=torch.float64, device=dev)
    z = torch.tensor(pts[:, 2], dtype=torch.float64, device=dev)
    ip = torch.tensor(d["iparent"], dtype=torch.int32, device=dev)
    dn = torch.tensor(d["dist_nearest"], dtype=torch.float64, device=dev)
    co = torch.tensor(np.ascontiguousarray(d["xyz"]).reshape(-1), dtype=torch.float64, device=dev)
    st = GauXCStatus()
    for _ in range(2):  # the shared work space keeps the previous call's contents
        w = torch.tensor(d["w_unm"], dtype=torch.float64, device=dev)
        L.gauxc_gb300_ssf_weights_noalloc(ctypes.byref(st), n, natoms, _dptr(x), _dptr(y),
                                          _dptr(z), _dptr(ip), _dptr(dn), _dptr(co), _dptr(w),
                                          None)
        check(st, L)
        torch.cuda.synchronize()
        got = w.cpu().numpy()
        assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(d["w_unm"]))

    # beyond the fixed work space: rejected before any device work
    w = torch.tensor(d["w_unm"], dtype=torch.float64, device=dev)
    L.gauxc_gb300_ssf_weights_noalloc(ctypes.byref(st), 1 << 22, natoms, _dptr(x), _dptr(y),
                                      _dptr(z), _dptr(ip), _dptr(dn), _dptr(co), _dptr(w), None)
    with pytest.raises(GauXCError, match="split the points"):
        check(st, L)
