"""The GPU FP64 path against the CPU oracle at the full sizes of the
benchmark configurations.

- The 1000 x 1000 jittered lattice (cubic spline, and the Gaussian cut at
  q <= 3 on the reference's truncated 3 x 3 stencil of 2h cells) and the
  1M-fluid dam break (walls with h = 0, so the reference's cells are 1 m
  wide): every particle's neighbour list bit-exact and in the reference's
  order (NNLinkedList.near, src/Tools/NNLinkedList.py:41-141), and one
  derivative evaluation
  (Solver._compute = nn.update + h + _loop, src/Solver.py:232-256,
  src/Tools/SolverTools.py:120-175) within 1e-10, norm-wise relative per
  field over the fluid, from the identical state.
- The 3200-fluid dam break of the CPU-runnable configuration for its full
  1000 PEC steps (src/Solver.py:366-410), compared at steps 1, 10, 100 and
  1000.  Round-off differences grow along a trajectory, so the tolerance at
  each step comes from a control: the oracle once more, summing every
  particle's neighbours in reverse order.  That run differs from the
  reference only by round-off; the GPU path (which sums in its own cell
  order) must stay within a fixed factor of the control's distance.
"""
import json
import os

import numpy as np
import pytest

import sphcases as SC

pytestmark = pytest.mark.gpu

TOL64 = 1e-10


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build
    build.build()
    import oracle
    oracle.build()


def _threads():
    import oracle
    return oracle.max_threads()


def _prepared(name):
    """The benchmark workload after its set-up, on the device (FP64 form)."""
    import bench
    wl = bench.workload(name)
    dp, wc, cfg, ws = bench.prepare(wl, "fp64")
    return wl, dp, wc, cfg, ws


@pytest.mark.parametrize("name", ["lattice1m", "lattice1m_gauss", "dambreak1m"])
def test_fullsize_neighbour_lists_bit_exact(lib, name):
    import oracle
    import torch
    from sph import _lib, core
    wl, dp, wc, cfg, ws = _prepared(name)
    core.nn_update(dp, cfg, ws)
    off, idx = core.nn_export(dp, cfg, ws)
    ws.check(allow=_lib.STATUS_INFO)
    st = dp.soa(("x", "y", "h"))
    del dp, ws
    torch.cuda.empty_cache()
    nn = oracle.NN(2.0)
    assert nn.update(st["x"], st["y"], st["h"]) == 0
    off_r, idx_r = nn.all(nthreads=_threads())  # the reference's traversal order
    assert np.array_equal(np.asarray(off), off_r), "neighbour counts differ"
    same = np.asarray(idx) == idx_r
    if not same.all():
        first = int(np.searchsorted(off_r, np.argmin(same), side="right") - 1)
        pytest.fail("neighbour lists differ (members or order), first at particle %d" % first)


@pytest.mark.parametrize("name", ["lattice1m", "lattice1m_gauss", "dambreak1m"])
def test_fullsize_fp64_evaluation_matches_oracle(lib, name):
    import oracle
    import torch
    from sph import core
    wl, dp, wc, cfg, ws = _prepared(name)
    init = dp.soa()
    core.compute(dp, wc, cfg, ws)
    ws.check()
    got = dp.soa(("drho", "ax", "ay", "p", "h"))
    del dp, ws
    torch.cuda.empty_cache()
    P = oracle.Particles(arrays=init)
    par = oracle.wcsph_params(wl["height"], wl["r0"], 1000.0, kernel=wl["kernel"])
    assert oracle.compute(par, oracle.NN(2.0), P, wl["h"], nthreads=_threads()) == 0
    fluid = init["label"] == 0
    errs = {k: SC.rel_err(got[k][fluid], getattr(P, k)[fluid]) for k in ("drho", "ax", "ay", "h")}
    errs["p"] = SC.rel_err(got["p"], P.p)
    assert all(e <= TOL64 for e in errs.values()), errs
    assert np.linalg.norm(P.ay[fluid]) > 0


DAM_STEPS = (1, 10, 100, 1000)
DAM_FIELDS = ("x", "y", "vx", "vy", "rho")
CONTROL_FACTOR = 30.0   # the GPU path may drift this many times the control's distance ...
FLOOR = 1e-13           # ... or this much, whichever is larger


def _dam_break_3200():
    import oracle
    from sph import scenarios as S
    pa = S.cfg_dam_break_small()
    dx = 0.025
    P = oracle.Particles(arrays={k: pa[k] for k in pa.dtype.names if k != "deleted"})
    par = oracle.wcsph_params(2.0, dx, 1000.0)
    oracle.setup(P, par, 2.0, 1.3 * dx)
    return P.as_dict(), dx


def test_dam_break_3200_for_1000_steps_against_oracle_and_control(lib):
    """The CPU-runnable configuration (3200 fluid, PEC, Courant 0.3) for its
    full 1000 steps: GPU FP64 against the oracle at steps 1, 10, 100, 1000,
    with each tolerance taken from the reversed-summation control."""
    import oracle
    import torch
    from sph import core, state
    init, dx = _dam_break_3200()
    h = 1.3 * dx
    ref = oracle.Particles(arrays={k: v.copy() for k, v in init.items()})
    ctl = oracle.Particles(arrays={k: v.copy() for k, v in init.items()})
    par = oracle.wcsph_params(2.0, dx, 1000.0)
    par_ctl = oracle.wcsph_params(2.0, dx, 1000.0, sum_order=1)
    nn_r, nn_c = oracle.NN(2.0), oracle.NN(2.0)
    from sph.Common import particle_dtype
    pa = np.zeros(len(init["x"]), dtype=particle_dtype)
    for k, v in init.items():
        pa[k] = v
    dp = state.DeviceParticles.from_array(pa)
    wc = core.wcsph_struct(2.0, dx, 1000.0)
    cfg = core.config_struct(precision="fp64", h_fixed=h, cfl_c=0.3, cfl_f=0.25)
    ws = state.DeviceWorkspace(dp.n)
    fluid = init["label"] == 0
    report = {}
    done = 0
    dt_gpu, dt_ref, dt_ctl = [], [], []
    for s in DAM_STEPS:
        k = s - done
        hist = torch.zeros((k, 3), dtype=torch.float64, device="cuda")
        core.run(dp, wc, cfg, ws, k, hist)
        ws.check()
        dt_gpu.append(hist.cpu().numpy())
        nt = _threads()
        dt_ref.append(oracle.run(par, nn_r, ref, k, h_fixed=h, gamma_c=0.3, gamma_f=0.25, nthreads=nt))
        dt_ctl.append(oracle.run(par_ctl, nn_c, ctl, k, h_fixed=h, gamma_c=0.3, gamma_f=0.25, nthreads=nt))
        done = s
        got = dp.soa(DAM_FIELDS)
        row = {}
        for f in DAM_FIELDS:
            want = getattr(ref, f)[fluid]
            e_gpu = SC.rel_err(got[f][fluid], want)
            e_ctl = SC.rel_err(getattr(ctl, f)[fluid], want)
            row[f] = (e_gpu, e_ctl)
        report[s] = row
    dts = {"gpu": np.concatenate(dt_gpu), "ref": np.concatenate(dt_ref), "ctl": np.concatenate(dt_ctl)}
    e_dt_gpu = float(np.max(np.abs(dts["gpu"][:, 0] / dts["ref"][:, 0] - 1.0)))
    e_dt_ctl = float(np.max(np.abs(dts["ctl"][:, 0] / dts["ref"][:, 0] - 1.0)))
    out = os.environ.get("SPH_PARITY_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump({"steps": {str(s): {k: list(v) for k, v in r.items()} for s, r in report.items()},
                       "dt_max_rel": {"gpu": e_dt_gpu, "control": e_dt_ctl}}, f, indent=1)
    bad = {}
    for s, row in report.items():
        for f, (e_gpu, e_ctl) in row.items():
            if not e_gpu <= max(CONTROL_FACTOR * e_ctl, FLOOR):
                bad["step %d %s" % (s, f)] = (e_gpu, e_ctl)
    assert not bad, bad
    assert e_dt_gpu <= max(CONTROL_FACTOR * e_dt_ctl, FLOOR), (e_dt_gpu, e_dt_ctl)
    # the run is a real dam break: the column has started to collapse
    assert np.max(np.abs(getattr(ref, "vx")[fluid])) > 0.1
