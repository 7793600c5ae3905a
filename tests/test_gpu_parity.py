"""GPU parity: the CUDA path (through the C ABI) against the reference's
golden vectors and the CPU oracle.

Tolerances (norm-wise relative, ||gpu - ref|| / ||ref|| per field):
  FP64 derivative evaluation   1e-10
  FP64 trajectories            1e-9 after the golden steps, 1e-8 after 20+ steps
  mixed (FP32 pair) evaluation 1e-5 on the single-evaluation lattices
Neighbour sets: bit-exact (set equality per particle).
"""
import numpy as np
import pytest

import sphcases as SC

pytestmark = pytest.mark.gpu

EVAL_FIELDS = ("rho", "p", "c", "h", "drho", "ax", "ay", "xsphx", "xsphy", "vx", "vy")
TOL64 = 1e-10


@pytest.fixture(scope="module")
def sph():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build, core, state
    build.build()
    return core, state


def _setup(meta, init, precision, max_cells=0):
    from sph import core, state
    dp = state.DeviceParticles.from_array(_to_array(init))
    wc = core.wcsph_struct(meta["height"], meta["r0"], 1000.0, use_xsph=bool(meta["useXSPH"]),
                           use_summation_density=bool(meta["sumdens"]))
    cfg = core.config_struct(kernel=int(meta["kernel"]), precision=precision, integrator=int(meta["integrator"]),
                             pec_use_xsph=bool(meta["useXSPH"]), pec_strict=bool(meta["strict"]),
                             h_fixed=meta["h"] if meta["h"] > 0 else 0.0, cfl_c=meta["gamma_c"], cfl_f=0.25,
                             dt_fixed=meta["fixed_dt"] if meta["fixed_dt"] > 0 else 0.0)
    ws = state.DeviceWorkspace(dp.n, max_cells)
    return dp, wc, cfg, ws


def _to_array(d):
    from sph.Common import particle_dtype
    pa = np.zeros(len(d["x"]), dtype=particle_dtype)
    for k, v in d.items():
        pa[k] = v
    return pa


def test_library_exports_and_version(sph):
    from sph import _lib
    L = _lib.load()
    assert L.sph_abi_version() == 1


def test_kernel_maps(sph):
    core, _ = sph
    z = SC.load("kernels")
    assert SC.rel_err(core.kernel_eval(0, z["r"], z["h"]).cpu().numpy(), z["cubic_w"]) <= 1e-14
    assert SC.rel_err(core.kernel_grad(0, z["x"], z["r"], z["h"]).cpu().numpy(), z["cubic_grad"]) <= 1e-14
    assert SC.rel_err(core.kernel_eval(1, z["r"], z["h"]).cpu().numpy(), z["gauss_w"]) <= 1e-14
    assert SC.rel_err(core.gauss_deriv(z["r"], z["h"]).cpu().numpy(), z["gauss_deriv"]) <= 1e-14
    assert SC.rel_err(core.kernel_grad(1, z["x"], z["r"], z["h"]).cpu().numpy(), z["gauss_grad"]) <= 1e-14


def _sets(off, idx):
    return [np.sort(idx[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def _assert_same_sets(off_a, idx_a, off_b, idx_b):
    a, b = _sets(off_a, idx_a), _sets(off_b, idx_b)
    assert len(a) == len(b)
    bad = [i for i in range(len(a)) if not np.array_equal(a[i], b[i])]
    assert not bad, "neighbour sets differ for %d particles, first %s" % (len(bad), bad[:5])


def _assert_same_lists(off_a, idx_a, off_b, idx_b):
    """The same lists in the same order (the reference's traversal order)."""
    _assert_same_sets(off_a, idx_a, off_b, idx_b)
    assert np.array_equal(np.asarray(off_a), np.asarray(off_b))
    same = np.asarray(idx_a) == np.asarray(idx_b)
    if not same.all():
        first = int(np.searchsorted(np.asarray(off_b), np.argmin(same), side="right") - 1)
        raise AssertionError("neighbour lists in a different order, first at particle %d" % first)


@pytest.mark.parametrize("name", ["nn_lattice", "nn_tank", "nn_alias", "nn_alias_boundary", "nn_grid26"])
@pytest.mark.parametrize("max_cells", [0, 64])
def test_nn_sets_bit_exact(sph, name, max_cells):
    """NNLinkedList.near for every particle equals the reference's lists, in
    the reference's order; max_cells = 64 forces the coarsened own-grid
    search with the reference-stencil filter."""
    core, state = sph
    from sph import _lib
    z = SC.load(name)
    d = dict(x=z["x"], y=z["y"], h=z["h"], label=z["label"])
    dp = state.DeviceParticles.from_array(_to_array(d))
    cfg = core.config_struct(nn_scale=float(z["scale"]))
    ws = state.DeviceWorkspace(dp.n, max_cells)
    core.nn_update(dp, cfg, ws)
    off, idx = core.nn_export(dp, cfg, ws)
    st = ws.check(allow=_lib.STATUS_INFO)
    _assert_same_lists(off, idx, z["offsets"], z["idx"])


@pytest.mark.parametrize("name", SC.SOLVER_CASES)
def test_eval_fp64_matches_reference(sph, name):
    core, _ = sph
    meta, init, ev, steps, dts = SC.load_case(name)
    dp, wc, cfg, ws = _setup(meta, init, "fp64")
    core.compute(dp, wc, cfg, ws)
    ws.check()
    got = dp.soa()
    bad = SC.compare_state(got, ev, EVAL_FIELDS, TOL64)
    assert not bad, bad


@pytest.mark.parametrize("name", SC.SOLVER_CASES)
def test_eval_fp64_forced_own_grid(sph, name):
    """The same evaluations with a cell capacity small enough to force the
    coarsened traversal grid: results must not change."""
    core, _ = sph
    meta, init, ev, steps, dts = SC.load_case(name)
    dp, wc, cfg, ws = _setup(meta, init, "fp64", max_cells=16)
    core.compute(dp, wc, cfg, ws)
    ws.check()
    bad = SC.compare_state(dp.soa(), ev, EVAL_FIELDS, TOL64)
    assert not bad, bad


@pytest.mark.parametrize("name", SC.SOLVER_CASES)
def test_steps_fp64_match_reference(sph, name):
    core, _ = sph
    import torch
    meta, init, ev, steps, dts = SC.load_case(name)
    if not steps:
        pytest.skip("no steps in this case")
    dp, wc, cfg, ws = _setup(meta, init, "fp64")
    hist = torch.zeros((len(steps), 3), dtype=torch.float64, device="cuda")
    core.run(dp, wc, cfg, ws, len(steps), hist)
    ws.check()
    np.testing.assert_allclose(hist.cpu().numpy(), dts, rtol=1e-12)
    bad = SC.compare_state(dp.soa(), steps[-1], SC.STATE_FIELDS, 1e-9)
    assert not bad, bad


@pytest.mark.parametrize("name", ["solver_lattice_cubic", "solver_lattice_gauss", "solver_tank_cubic",
                                  "solver_tank_gauss"])
def test_eval_mixed_close_to_fp64(sph, name):
    core, _ = sph
    meta, init, ev, steps, dts = SC.load_case(name)
    dp, wc, cfg, ws = _setup(meta, init, "mixed")
    core.compute(dp, wc, cfg, ws)
    ws.check()
    got = dp.soa()
    errs = {k: SC.rel_err(got[k], ev[k]) for k in ("drho", "ax", "ay")}
    tol = 1e-5 if "lattice" in name else 1e-4
    assert all(e <= tol for e in errs.values()), errs


def test_step_sequence_matches_oracle_dam_break(sph):
    """20 PEC steps of the 3200-fluid dam break (4808 particles), FP64,
    against the oracle (Courant 0.3, as in the reference configuration)."""
    import oracle
    import torch
    from sph import scenarios as S
    core, state = sph
    pa = S.cfg_dam_break_small()
    dx = 0.025
    P = oracle.Particles(arrays={k: pa[k] for k in pa.dtype.names if k != "deleted"})
    par = oracle.wcsph_params(2.0, dx, 1000.0)
    oracle.setup(P, par, 2.0, 1.3 * dx)
    init = P.as_dict()
    meta = dict(height=2.0, r0=dx, useXSPH=0, sumdens=0, kernel=0, integrator=0, strict=1, h=1.3 * dx,
                gamma_c=0.3, fixed_dt=-1.0)
    dp, wc, cfg, ws = _setup(meta, init, "fp64")
    nsteps = 20
    hist = torch.zeros((nsteps, 3), dtype=torch.float64, device="cuda")
    core.run(dp, wc, cfg, ws, nsteps, hist)
    ws.check()
    dts = oracle.run(par, oracle.NN(2.0), P, nsteps, h_fixed=1.3 * dx, gamma_c=0.3, gamma_f=0.25, nthreads=8)
    np.testing.assert_allclose(hist.cpu().numpy(), dts, rtol=1e-9)
    bad = SC.compare_state(dp.soa(), P.as_dict(), SC.STATE_FIELDS, 1e-8)
    assert not bad, bad


@pytest.mark.parametrize("xsph", [False, True])
def test_damped_steps_match_oracle(sph, xsph):
    """20 damped PEC steps (damping 0.05, the Solver's default while it
    settles; with and without XSPH) of the 3200-fluid dam break, FP64,
    against the oracle. This runs the damped forms of the fused
    corrector + predictor."""
    import oracle
    import torch
    from sph import scenarios as S
    core, state = sph
    pa = S.cfg_dam_break_small()
    dx, damping = 0.025, 0.05
    P = oracle.Particles(arrays={k: pa[k] for k in pa.dtype.names if k != "deleted"})
    par = oracle.wcsph_params(2.0, dx, 1000.0, use_xsph=xsph)
    oracle.setup(P, par, 2.0, 1.3 * dx)
    init = P.as_dict()
    dp = state.DeviceParticles.from_array(_to_array(init))
    wc = core.wcsph_struct(2.0, dx, 1000.0, use_xsph=xsph)
    cfg = core.config_struct(precision="fp64", pec_use_xsph=xsph, pec_strict=True, h_fixed=1.3 * dx, cfl_c=0.3,
                             cfl_f=0.25, damping=damping)
    ws = state.DeviceWorkspace(dp.n)
    nsteps = 20
    hist = torch.zeros((nsteps, 3), dtype=torch.float64, device="cuda")
    core.run(dp, wc, cfg, ws, nsteps, hist)
    ws.check()
    dts = oracle.run(par, oracle.NN(2.0), P, nsteps, h_fixed=1.3 * dx, gamma_c=0.3, gamma_f=0.25, damping=damping,
                     pec_use_xsph=xsph, nthreads=8)
    np.testing.assert_allclose(hist.cpu().numpy(), dts, rtol=1e-9)
    bad = SC.compare_state(dp.soa(), P.as_dict(), SC.STATE_FIELDS, 1e-8)
    assert not bad, bad
    # damping slowed the fluid against the undamped run
    und = oracle.Particles(arrays={k: v.copy() for k, v in init.items()})
    oracle.run(par, oracle.NN(2.0), und, nsteps, h_fixed=1.3 * dx, gamma_c=0.3, gamma_f=0.25, pec_use_xsph=xsph,
               nthreads=8)
    f = init["label"] == 0
    assert np.linalg.norm(P.vy[f]) < np.linalg.norm(und.vy[f])


def _lattice_state(n, kernel, seed=0):
    from sph import scenarios as S
    import oracle
    pa = S.jittered_lattice(n, n, 0.01, seed=seed)
    d = {k: pa[k] for k in pa.dtype.names if k != "deleted"}
    d["h"] = np.full(len(pa), 0.013)
    par = oracle.wcsph_params(n * 0.01, 0.01, 1000.0, kernel=kernel)
    d["p"] = oracle.eos(d["label"], d["rho"], par)
    d["c"] = np.full(len(pa), par.co)
    meta = dict(height=n * 0.01, r0=0.01, useXSPH=0, sumdens=0, kernel=kernel, integrator=0, strict=1, h=0.013,
                gamma_c=0.25, fixed_dt=-1.0)
    return d, meta, par


@pytest.mark.parametrize("kernel", [0, 1])
def test_lattice_eval_matches_oracle(sph, kernel):
    """A 300 x 300 jittered lattice (no boundaries: the reference's truncated
    3x3 stencil with cell size 2h) against the oracle, FP64 and mixed."""
    import oracle
    core, _ = sph
    d, meta, par = _lattice_state(300, kernel)
    P = oracle.Particles(arrays=d)
    oracle.compute(par, oracle.NN(2.0), P, 0.013, nthreads=8)
    ref = P.as_dict()
    for prec, tol in (("fp64", TOL64), ("mixed", 1e-5)):
        dp, wc, cfg, ws = _setup(meta, d, prec)
        core.compute(dp, wc, cfg, ws)
        ws.check()
        bad = SC.compare_state(dp.soa(), ref, ("drho", "ax", "ay", "p"), tol)
        assert not bad, (prec, bad)


def test_nn_sets_dam_break_vs_oracle(sph):
    import oracle
    from sph import scenarios as S
    core, state = sph
    pa = S.cfg_dam_break_small()
    pa["h"][pa["label"] == 0] = 0.0325
    nn = oracle.NN(2.0)
    nn.update(pa["x"], pa["y"], pa["h"])
    off_r, idx_r = nn.all()
    dp = state.DeviceParticles.from_array(pa)
    cfg = core.config_struct()
    ws = state.DeviceWorkspace(dp.n)
    core.nn_update(dp, cfg, ws)
    off, idx = core.nn_export(dp, cfg, ws)
    ws.check()
    _assert_same_lists(off, idx, off_r, idx_r)


def test_grid_kept_only_while_its_inputs_hold(sph):
    """One workspace through evaluations whose grid inputs change (the kernel,
    then the positions) and come back: each is bit-equal to the same
    evaluation on a fresh workspace, so a grid kept from the previous build
    is only ever one its inputs would make again."""
    from sph import _lib
    core, state = sph
    meta, init, ev, steps, dts = SC.load_case("solver_tank_cubic")
    dp, wc, cfg, ws = _setup(meta, init, "fp64")
    moved = dict(init)
    moved["x"] = np.asarray(init["x"]) + 0.37
    moved["y"] = np.asarray(init["y"]) * 1.5
    seq = [(init, _lib.KERNEL_CUBIC), (init, _lib.KERNEL_CUBIC), (init, _lib.KERNEL_GAUSSIAN),
           (init, _lib.KERNEL_CUBIC), (moved, _lib.KERNEL_CUBIC), (init, _lib.KERNEL_CUBIC)]
    for k, (st, kern) in enumerate(seq):
        cfg.kernel = kern
        dp.upload_soa(st)
        core.compute(dp, wc, cfg, ws)
        ws.check()
        got = dp.soa(("rho", "drho", "ax", "ay"))
        dp_f, _, _, ws_f = _setup(meta, st, "fp64")
        core.compute(dp_f, wc, cfg, ws_f)
        ws_f.check()
        ref = dp_f.soa(("rho", "drho", "ax", "ay"))
        for f in ("rho", "drho", "ax", "ay"):
            assert np.array_equal(got[f], ref[f]), (k, kern, f)
