"""The host-buffer stepping that bench.py times as its end-to-end figure does
the work of the step: k one-step calls through pinned host buffers and two
alternating device copies of the state end in the state that k one-step
calls in place reach, bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_e2e_stepping_matches_in_place(precision):
    import bench
    from sph import core
    wl = bench.workload("dambreak3200")
    dp, wc, cfg, ws = bench.prepare(wl, precision)
    dq, wcq, cfgq, wsq = bench.prepare(wl, precision)
    k = 7
    host = {}
    bench.e2e_steps(core, dp, wc, cfg, ws, k, wl["pa"], result=host)
    for _ in range(k):
        core.run(dq, wcq, cfgq, wsq, 1)
    ws.check()
    wsq.check()
    for f in ("x", "y", "vx", "vy", "rho", "drho", "ax", "ay", "p"):
        np.testing.assert_array_equal(host[f], dq.fields[f].cpu().numpy(), err_msg=f)
    # the steps moved the fluid
    assert not np.array_equal(host["vy"], np.asarray(wl["pa"]["vy"], dtype=np.float64))
