"""Batched form (sph.batch.Ensemble over sph_batch_run): every instance of a
batched run equals a single-instance run of it, bit for bit; a captured CUDA
graph replays the eager steps exactly; the autotuner restores the state it
tunes on."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "rho", "ax", "ay", "drho", "p", "h", "x0", "y0", "vx0", "vy0", "rho0")


@pytest.fixture(scope="module")
def ens():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build
    build.build()
    from sph import batch, scenarios
    cases = scenarios.ensemble(count=6, seed=1, width=(0.2, 0.5), height=(0.3, 0.8), dx=(0.02, 0.05))
    return cases, batch.Ensemble(cases)


def _single(pa, c, max_cells, nsteps):
    from sph import core, state
    dp = state.DeviceParticles.from_array(pa)
    wc = core.wcsph_struct(c["height"], c["dx"], 1000.0)
    cfg = core.config_struct(precision="mixed", h_fixed=1.3 * c["dx"], cfl_c=0.3, cfl_f=0.25)
    core.initialize(dp, wc, cfg)
    ws = state.DeviceWorkspace(len(pa), max_cells)
    hist = torch.zeros((nsteps, 3), dtype=torch.float64, device="cuda")
    core.run(dp, wc, cfg, ws, nsteps, hist)
    ws.check()
    return dp, hist


def test_batched_instances_equal_single_runs(ens):
    cases, E = ens
    snap = E.snapshot()
    nsteps = 8
    hist = torch.zeros((nsteps, E.n_inst, 3), dtype=torch.float64, device="cuda")
    E.run(nsteps, hist)
    E.check()
    for b, (pa, c) in enumerate(cases):
        dp, h1 = _single(pa, c, E.instance_cells(b), nsteps)
        s, e = int(E.offsets_np[b]), int(E.offsets_np[b + 1])
        for k in FIELDS:
            got = E.dp.fields[k][s:e]
            assert torch.equal(got, dp.fields[k]), (b, k, (got - dp.fields[k]).abs().max().item())
        assert torch.equal(hist[:, b, :], h1), b
    E.restore(snap)


def test_graph_replay_equals_eager_steps(ens):
    _, E = ens
    snap = E.snapshot()
    E.run(4)
    want = E.dp._buf.clone()
    g = E.capture(4)
    E.restore(snap)
    E.setup()
    g.replay()
    torch.cuda.synchronize()
    E.check()
    assert torch.equal(E.dp._buf, want)
    E.restore(snap)
    E.setup()


def test_autotune_restores_the_state(ens):
    _, E = ens
    snap = E.snapshot()
    res = E.autotune(steps=2, warmup=1)
    assert len(res) == 6 and all(v > 0 for v in res.values())
    assert torch.equal(E.dp._buf, snap[0])
    E.run(1)
    E.check()
    E.restore(snap)
