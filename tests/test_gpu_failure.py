"""Error path of the tensor-core pipeline's bounded waits (needs a GB300).

Every mbarrier wait of the GEMM kernels gives up after a bound, records an
error code and lets the CTAs leave; the host turns the code into an error.
Here the producers are told to issue no copy at all, so that the first wait
of every consumer runs out with nothing in flight (no copy, no MMA), with a
5 ms bound.  The call must fail with the pipeline error, and the same
integrator must then run normally and reproduce its earlier result: the
error flag is cleared at the start of every call and the CUDA context stays
usable.  Nothing faults, traps or hangs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pipeline_wait_expiry_is_reported_and_recovers(g):
    from gauxc_gb300 import workloads as W
    from gauxc_gb300._capi import GauXCError
    s = W.config(5)["systems"][0]
    mol, basis, mg, lb = W.build_system(s)
    g.MolecularWeightsFactory(g.ExecutionSpace.Device).get_instance().modify_weights(lb)
    integ = g.XCIntegratorFactory(g.ExecutionSpace.Device, "Replicated", "Default",
                                  "GB300-Mixed", "Default").get_instance(
                                      g.functional_type(s["functional"]), lb)
    exc0, vxc0 = integ.eval_exc_vxc(s["P"])

    integ.set_pipeline_check(wait_ms=5.0, withhold=True)
    with pytest.raises(GauXCError, match="pipeline wait expired"):
        integ.eval_exc_vxc(s["P"])

    integ.set_pipeline_check(wait_ms=1000.0, withhold=False)
    exc1, vxc1 = integ.eval_exc_vxc(s["P"])
    assert abs(exc1 - exc0) <= 1e-12
    assert np.abs(vxc1 - vxc0).max() <= 1e-12

