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


def _lattice_case(precision):
    from sph import core, scenarios, state
    pa = scenarios.jittered_lattice(60, 60, 0.01, seed=4)
    dp = state.DeviceParticles.from_array(pa)
    wc = core.wcsph_struct(0.6, 0.01, 1000.0)
    cfg = core.config_struct(precision=precision, h_fixed=0.013, cfl_c=0.25, cfl_f=0.25)
    dp.h[dp.label == 0] = 0.013
    core.eos(dp, wc)
    return dp, wc, cfg, state.DeviceWorkspace(dp.n)


def _ws_without_copy(n):
    """A workspace with room for everything but the sorted state copy
    (sph_workspace_size includes it: 19 doubles, a label and an index per
    particle, each array at a 256-byte boundary), so sph_run steps on the
    caller's arrays."""
    import ctypes as C
    import torch
    from sph import _lib as L
    from sph.state import DeviceWorkspace, current_stream
    lib = L.load()
    mc = int(lib.sph_default_max_cells(n))
    full = C.c_size_t()
    L.check(lib.sph_workspace_size(n, mc, C.byref(full)), "sph_workspace_size")

    def a256(v):
        return (v + 255) // 256 * 256
    nbytes = int(full.value) - a256(8 * 19 * n) - a256(n) - a256(4 * n)
    ws = DeviceWorkspace.__new__(DeviceWorkspace)
    ws.n_cap = n
    ws.buf = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    ws.ws = L.Workspace(ptr=ws.buf.data_ptr(), bytes=nbytes, n_cap=n, max_cells=mc)
    L.check(lib.sph_workspace_init(C.byref(ws.ws), current_stream()), "sph_workspace_init")
    return ws


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("name", ["dambreak3200", "lattice60"])
def test_run_on_sorted_copy_is_bit_exact(precision, name):
    """A run of several steps steps on a sorted copy of the state in the
    workspace (gathered once, scattered back at the end); it must end in the
    state and dt history of the same run on the caller's arrays (a workspace
    without room for the copy), bit for bit, with walls (a fixed grid) and
    without (the grid moves)."""
    import torch
    import bench
    from sph import core
    k = 9
    if name == "dambreak3200":
        wl = bench.workload(name)
        dp, wc, cfg, ws = bench.prepare(wl, precision)
        dq, wcq, cfgq, _ = bench.prepare(wl, precision)
    else:
        dp, wc, cfg, ws = _lattice_case(precision)
        dq, wcq, cfgq, _ = _lattice_case(precision)
    wsq = _ws_without_copy(dq.n)
    h1 = torch.zeros((k, 3), dtype=torch.float64, device="cuda")
    core.run(dp, wc, cfg, ws, k, h1)
    h2 = torch.zeros((k, 3), dtype=torch.float64, device="cuda")
    core.run(dq, wcq, cfgq, wsq, k, h2)
    ws.check()
    wsq.check()
    assert torch.equal(h1, h2)
    for f in ("x", "y", "vx", "vy", "rho", "drho", "ax", "ay", "p", "c", "h", "x0", "y0", "vx0", "vy0", "rho0"):
        assert torch.equal(dp.fields[f], dq.fields[f]), f
    assert torch.equal(dp.label, dq.label)
    assert not torch.equal(dp.vx, torch.zeros_like(dp.vx))
