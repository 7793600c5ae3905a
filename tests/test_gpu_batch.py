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
    assert len(res) == 4 and all(v > 0 for v in res.values())
    assert torch.equal(E.dp._buf, snap[0])
    E.run(1)
    E.check()
    E.restore(snap)


# ---------------------------------------------------------------------------
# The benchmark's own ensemble: 256 seeded dam breaks (seed 1), its smallest,
# median and largest instance (by fluid count) checked against the GPU's FP64
# form (a single-instance run, the oracle of the mixed form: derivatives and
# short trajectories within 1e-5) and that FP64 run against the CPU oracle
# (1e-10 after one step, 1e-9 after ten).
# ---------------------------------------------------------------------------
TOL_MIXED = 1e-5


@pytest.fixture(scope="module")
def bench_ensemble():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build
    build.build()
    from sph import batch, scenarios
    cases = scenarios.ensemble(count=256, seed=1)
    return cases, batch.Ensemble(cases)


def _picks(cases):
    sizes = [int(np.sum(pa["label"] == 0)) for pa, _ in cases]
    order = np.argsort(sizes, kind="stable")
    return [int(order[0]), int(order[len(order) // 2]), int(order[-1])]


def _rel(a, b):
    import sphcases as SC
    return SC.rel_err(a, b)


def test_bench_ensemble_instances_against_fp64_and_oracle(bench_ensemble):
    import oracle
    from sph import core, state
    cases, E = bench_ensemble
    picks = _picks(cases)
    snap = E.snapshot()
    hist = torch.zeros((10, E.n_inst, 3), dtype=torch.float64, device="cuda")
    E.run(1, hist[:1])
    E.check()
    after1 = {b: E.instance(b) for b in picks}
    E.run(9, hist[1:])
    E.check()
    after10 = {b: E.instance(b) for b in picks}
    E.restore(snap)
    E.setup()
    report = {}
    for b in picks:
        pa, c = cases[b]
        h = 1.3 * c["dx"]
        dp = state.DeviceParticles.from_array(pa)
        wc = core.wcsph_struct(c["height"], c["dx"], 1000.0)
        cfg = core.config_struct(precision="fp64", h_fixed=h, cfl_c=0.3, cfl_f=0.25)
        core.initialize(dp, wc, cfg)
        ws = state.DeviceWorkspace(dp.n)
        init = dp.soa()
        h64 = torch.zeros((10, 3), dtype=torch.float64, device="cuda")
        core.run(dp, wc, cfg, ws, 1, h64[:1])
        ws.check()
        g1 = dp.soa()
        core.run(dp, wc, cfg, ws, 9, h64[1:])
        ws.check()
        g10 = dp.soa()
        fl = init["label"] == 0
        # mixed (batched) against FP64 (single instance)
        e1 = {k: _rel(after1[b][k][fl], g1[k][fl]) for k in ("ax", "ay", "drho", "vx", "vy")}
        e10 = {k: _rel(after10[b][k][fl], g10[k][fl]) for k in ("x", "y", "vx", "vy", "rho", "ax", "ay")}
        edt = float(np.max(np.abs(hist[:, b, 0].cpu().numpy() / h64[:, 0].cpu().numpy() - 1.0)))
        # FP64 against the oracle from the same initial state
        P = oracle.Particles(arrays=init)
        par = oracle.wcsph_params(c["height"], c["dx"], 1000.0)
        nn = oracle.NN(2.0)
        d1 = oracle.run(par, nn, P, 1, h_fixed=h, gamma_c=0.3, gamma_f=0.25, nthreads=oracle.max_threads())
        o1 = {k: _rel(g1[k][fl], getattr(P, k)[fl]) for k in ("ax", "ay", "drho", "x", "y", "vx", "vy", "rho")}
        d10 = oracle.run(par, nn, P, 9, h_fixed=h, gamma_c=0.3, gamma_f=0.25, nthreads=oracle.max_threads())
        o10 = {k: _rel(g10[k][fl], getattr(P, k)[fl]) for k in ("x", "y", "vx", "vy", "rho", "ax", "ay")}
        dts = np.concatenate([d1, d10])
        report[b] = dict(n_fluid=int(fl.sum()), mixed_step1=e1, mixed_step10=e10, mixed_dt=edt,
                         oracle_step1=o1, oracle_step10=o10)
        assert all(v <= TOL_MIXED for v in e1.values()), (b, e1)
        assert all(v <= TOL_MIXED for v in e10.values()), (b, e10)
        assert edt <= TOL_MIXED, (b, edt)
        assert all(v <= 1e-10 for v in o1.values()), (b, o1)
        assert all(v <= 1e-9 for v in o10.values()), (b, o10)
        np.testing.assert_allclose(h64.cpu().numpy(), dts, rtol=1e-10)
    import json
    import os
    out = os.environ.get("SPH_BATCH_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)
