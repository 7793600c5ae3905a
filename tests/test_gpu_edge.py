"""Degenerate inputs through the C ABI, against the oracle: a lone fluid
particle (the zero-neighbour rule of src/Tools/SolverTools.py:150-153), a
tank with no fluid (TimeStep has nothing to take dt from), and a clump far
denser than the lattice, whose tile halos overflow shared memory so that every
query takes the global fallback path."""
import numpy as np
import pytest

import sphcases as SC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sph():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build, core, state
    build.build()
    return core, state


def _arrays(pa):
    return {k: pa[k] for k in pa.dtype.names if k != "deleted"}


def _device(pa, precision, h, height=1.0, r0=0.02, dt_fixed=0.0):
    from sph import core, state
    pa = pa.copy()
    pa["h"][pa["label"] == 0] = h  # Solver.setup's fixed h
    dp = state.DeviceParticles.from_array(pa)
    wc = core.wcsph_struct(height, r0, 1000.0)
    cfg = core.config_struct(precision=precision, h_fixed=h, cfl_c=0.3, cfl_f=0.25, dt_fixed=dt_fixed)
    ws = state.DeviceWorkspace(dp.n)
    return dp, wc, cfg, ws


def _oracle(pa, h, height=1.0, r0=0.02, nsteps=3, dt_fixed=0.0):
    import oracle
    pa = pa.copy()
    pa["h"][pa["label"] == 0] = h
    P = oracle.Particles(arrays=_arrays(pa))
    par = oracle.wcsph_params(height, r0, 1000.0)
    P.p[:] = oracle.eos(P.label, P.rho, par)
    P.c[:] = par.co
    dts = oracle.run(par, oracle.NN(2.0), P, nsteps, h_fixed=h, dt_fixed=dt_fixed, gamma_c=0.3, gamma_f=0.25)
    return P, dts


def _state(n, seed=0):
    from sph.Common import particle_dtype
    rng = np.random.default_rng(seed)
    pa = np.zeros(n, dtype=particle_dtype)
    pa["m"] = 0.4
    pa["rho"] = 1000.0 * (1 + rng.uniform(-0.01, 0.01, n))
    return pa, rng


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lone_fluid_particle(sph, precision):
    import torch
    core, _ = sph
    pa, _ = _state(1)
    pa["x"], pa["y"], pa["vx"], pa["vy"] = 0.3, 0.7, 0.2, -0.1
    dp, wc, cfg, ws = _device(pa, precision, h=0.026)
    core.eos(dp, wc)
    hist = torch.zeros((3, 3), dtype=torch.float64, device="cuda")
    core.run(dp, wc, cfg, ws, 3, hist)
    ws.check()
    P, dts = _oracle(pa, 0.026)
    # the mixed form takes the force dt from an FP32 a^2 (the Courant dt decides here)
    np.testing.assert_allclose(hist.cpu().numpy(), dts, rtol=1e-12 if precision == "fp64" else 1e-6)
    got = dp.soa()
    for k in ("x", "y", "vx", "vy", "rho", "ax", "ay", "drho"):
        np.testing.assert_allclose(got[k], getattr(P, k), rtol=1e-12, atol=1e-12, err_msg=k)


def test_no_fluid_reports_status(sph):
    from sph import _lib
    core, _ = sph
    pa, rng = _state(64)
    pa["label"] = 1
    pa["x"] = rng.uniform(0, 1, 64)
    pa["y"] = rng.uniform(0, 1, 64)
    dp, wc, cfg, ws = _device(pa, "mixed", h=0.026)
    before = dp.soa()
    core.compute(dp, wc, cfg, ws)
    after = dp.soa()
    for k in ("x", "y", "vx", "vy", "ax", "ay", "drho"):
        np.testing.assert_array_equal(after[k], before[k], err_msg=k)
    dt3 = core.timestep(dp, wc, cfg, ws).cpu().numpy()
    assert np.all(np.isnan(dt3))
    assert "no fluid particle" in _lib.status_names(ws.status())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dense_clump_takes_the_fallback_path(sph, precision):
    """600 fluid particles in a 0.1 m square with h = 0.026: about 60 per
    search cell, far over a tile halo's 384 slots."""
    import torch
    core, _ = sph
    n = 600
    pa, rng = _state(n, seed=4)
    pa["x"] = 0.5 + rng.uniform(0, 0.1, n)
    pa["y"] = 0.5 + rng.uniform(0, 0.1, n)
    pa["vx"] = rng.normal(0, 0.05, n)
    pa["vy"] = rng.normal(0, 0.05, n)
    dp, wc, cfg, ws = _device(pa, precision, h=0.026, dt_fixed=2e-5)
    core.eos(dp, wc)
    core.run(dp, wc, cfg, ws, 2)
    ws.check()
    P, _ = _oracle(pa, 0.026, nsteps=2, dt_fixed=2e-5)
    got = dp.soa()
    tol = 1e-9 if precision == "fp64" else 1e-4
    bad = SC.compare_state(got, P.as_dict(), ("x", "y", "vx", "vy", "rho", "ax", "ay", "drho"), tol)
    assert not bad, bad
