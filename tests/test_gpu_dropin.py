"""The drop-in classes (sph.Solver, WCSPH, CubicSpline, Gaussian, PEC, Euler,
NNLinkedList, TimeStep) used the way the reference's own tests use its
classes (test/test_kernels_cubic.py, test/test_kernels_Gaussian.py,
test/test_integrators_pec.py, test/test_integrators_euler.py,
test/test_linked_list.py), plus Solver runs against the oracle."""
import numpy as np
import pytest

import sphcases as SC

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sph():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import sph as pkg
    from sph import build
    build.build()
    return pkg


def test_cubic_known_answers(sph):
    """test/test_kernels_cubic.py:11-72"""
    k = sph.CubicSpline()
    fac = lambda h: 10 / (7 * np.pi * h * h)
    r = np.array([1.0])
    for q, h, want in [(0.5, 2.0, fac(2.0) * (1 - 1.5 * 0.25 * 0.75)), (1.0, 1.0, fac(1.0) * (1 - 1.5 * 0.5)),
                       (1.5, 2 / 3, fac(2 / 3) * 0.25 * 0.5 ** 3), (2.0, 0.5, 0.0), (3.0, 1 / 3, 0.0)]:
        assert k.evaluate(r, np.array([h]))[0] == pytest.approx(want, abs=1e-7)
    r, x = np.array([2.0]), np.array([3.0])
    for q, h, dwdq in [(0.5, 4.0, fac(4.0) * -3.0 * 0.5 * (1 - 0.375)), (1.0, 2.0, fac(2.0) * -0.75),
                       (2.0, 1.0, 0.0)]:
        assert k.gradient(x, r, np.array([h]))[0] == pytest.approx(dwdq / (h * 2.0) * 3.0, abs=1e-7)
    assert k.gradient(x, r, np.array([2 / 3]))[0] == 0.0


def test_gaussian_matches_reference(sph):
    z = SC.load("kernels")
    g = sph.Gaussian()
    assert SC.rel_err(g.evaluate(z["r"], z["h"]), z["gauss_w"]) <= 1e-14
    assert SC.rel_err(g.derivative(z["r"], z["h"]), z["gauss_deriv"]) <= 1e-14
    assert SC.rel_err(g.gradient(z["x"], z["r"], z["h"]), z["gauss_grad"]) <= 1e-14


def test_wendland_and_verlet_match_reference(sph):
    """src/Kernels/Wendland.py, src/Integrators/Verlet.py on the reference's outputs."""
    z = SC.load("wendland_verlet")
    k = sph.Wendland()
    assert SC.rel_err(k.evaluate(z["r"], z["h"]), z["wend_w"]) <= 1e-14
    assert SC.rel_err(k.gradient(z["x"], z["r"], z["h"]), z["wend_grad"]) <= 1e-14
    base = np.zeros(len(z["in_x"]), dtype=sph.particle_dtype)
    for name in base.dtype.names:
        if "in_" + name in z.files:
            base[name] = z["in_" + name]
    for xs in (0, 1):
        it = sph.Verlet(bool(xs))
        a = it.predict(0.003, base.copy(), 0.0)
        tag = "verlet_x%d" % xs
        for f in ("x", "y", "vx", "vy", "rho"):
            assert SC.rel_err(a[f], z[tag + "_pred_" + f]) <= 1e-15, (tag, f)
        a = it.correct(0.003, a, 0.0)
        for f in ("x", "y", "vx", "vy", "rho"):
            assert SC.rel_err(a[f], z[tag + "_corr_" + f]) <= 1e-15, (tag, f)


def test_probes_match_reference(sph):
    """NNLinkedList.nearPos and the ice-coupling pressure interpolation
    (examples/IceBreak.py:253-285) at 24 points, on the reference's tank state."""
    from sph import core, state
    from sph.Tools import Probes
    z = SC.load("probes")
    pa = np.zeros(len(z["st_x"]), dtype=sph.particle_dtype)
    for name in pa.dtype.names:
        if "st_" + name in z.files:
            pa[name] = z["st_" + name]
    nn = sph.NNLinkedList(2.0)
    nn.update(pa)
    h = float(z["h"])
    res = nn.nearPos_many(z["px"], z["py"], np.full(len(z["px"]), h))
    off = z["offsets"]
    for k, (hij, q, r, nb) in enumerate(res):
        assert np.array_equal(nb.astype(np.int64), z["idx"][off[k]:off[k + 1]]), k
        assert SC.rel_err(r, z["r"][off[k]:off[k + 1]]) <= 1e-15 and SC.rel_err(q, z["q"][off[k]:off[k + 1]]) <= 1e-15
    hij, q, r, nb = nn.nearPos(float(z["px"][0]), float(z["py"][0]), h, pa)
    assert np.array_equal(nb.astype(np.int64), z["idx"][off[0]:off[1]])
    # the pressure probe on a solver holding this state
    solver = sph.Solver(sph.WCSPH(0.4, 0.025, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline(), 1.0,
                        h=h, incrementalWriteout=False)
    solver.addParticles(pa.copy())
    solver._masks()
    solver._upload()
    core.nn_update(solver._dp, solver._cfg(), solver._ws)
    rho, p = Probes.pressure_SPH(z["px"], z["py"], solver, h)
    ok = np.isfinite(z["rho"])
    assert np.array_equal(np.isfinite(rho), ok)
    assert SC.rel_err(rho[ok], z["rho"][ok]) <= 1e-13 and SC.rel_err(p[ok], z["p"][ok]) <= 1e-11


def _particle(sph, label):
    p = np.zeros(1, dtype=sph.particle_dtype)
    p["label"] = label
    p["vx"], p["vy"], p["ax"], p["ay"], p["drho"] = 1.0, 3.0, 5.0, 0.0, 10.0
    return 2.0, p


def test_pec_known_answers(sph):
    """test/test_integrators_pec.py:13-76 (dt = 2)."""
    i = sph.PEC(useXSPH=False)
    dt, p = _particle(sph, sph.ParticleType.Fluid)
    p = i.predict(dt, p, 0)
    assert p["x"][0] == pytest.approx(dt * 0.5) and p["y"][0] == pytest.approx(dt * 0.5 * 3.0)
    assert p["rho"][0] == pytest.approx(dt * 0.5 * 10.0)
    p = i.correct(dt, p, 0)
    assert p["x"][0] == pytest.approx(dt * 1.0 + 0.5 * 5 * 2 * 2) and p["y"][0] == pytest.approx(dt * 3.0)
    assert p["rho"][0] == pytest.approx(10 * dt)
    # PEC equals Euler when the forces are not re-evaluated
    _, pi = _particle(sph, sph.ParticleType.Fluid)
    _, pe = _particle(sph, sph.ParticleType.Fluid)
    pi = i.correct(dt, i.predict(dt, pi, 0), 0)
    pe = sph.Euler().correct(dt, sph.Euler().predict(dt, pe, 0), 0)
    for k in ("x", "y", "vx", "vy", "rho"):
        assert pi[k][0] == pytest.approx(pe[k][0])


def test_integrators_match_reference(sph):
    z = SC.load("eos_integrators")
    base = np.zeros(len(z["in_x"]), dtype=sph.particle_dtype)
    for k in base.dtype.names:
        if "in_" + k in z.files:
            base[k] = z["in_" + k]
    for xs in (0, 1):
        for strict in (0, 1):
            for d in (0, 5):
                it = sph.PEC(useXSPH=bool(xs), strict=bool(strict))
                a = it.predict(0.003, base.copy(), d / 100.0)
                tag = "pec_x%d_s%d_d%d" % (xs, strict, d)
                for k in ("x", "y", "vx", "vy", "rho", "x0", "y0", "vx0", "vy0", "rho0"):
                    assert SC.rel_err(a[k], z[tag + "_pred_" + k]) <= 1e-13, (tag, k)
                a = it.correct(0.003, a, d / 100.0)
                for k in ("x", "y", "vx", "vy", "rho"):
                    assert SC.rel_err(a[k], z[tag + "_corr_" + k]) <= 1e-13, (tag, k)
    e = sph.Euler().correct(0.003, base.copy(), 0.0)
    for k in ("x", "y", "vx", "vy", "rho"):
        assert SC.rel_err(e[k], z["euler_" + k]) <= 1e-13
    np.testing.assert_allclose(sph.TimeStep().compute(len(base), base, 0.25, 0.25), z["ts"], rtol=1e-14)
    np.testing.assert_allclose(sph.TimeStep().compute(len(base), base, 0.3, 0.25), z["ts_c03"], rtol=1e-14)


def test_wcsph_pressure_and_initialize(sph):
    z = SC.load("eos_integrators")
    m = sph.WCSPH(height=2.0, r0=0.025, rho0=1000.0, useXSPH=False, Pb=0.0, useSummationDensity=False)
    assert m.co == pytest.approx(float(z["co"]), rel=1e-15) and m.B == pytest.approx(float(z["B"]), rel=1e-15)
    pa = np.zeros(len(z["rho"]), dtype=sph.particle_dtype)
    pa["label"], pa["rho"], pa["y"] = z["label"], z["rho"], z["y"]
    assert SC.rel_err(m.compute_pressure(pa), z["p"]) <= 1e-13
    m2 = sph.WCSPH(height=3.0, r0=0.025, rho0=1000.0, useXSPH=False, Pb=101325.0)
    assert SC.rel_err(m2.compute_pressure(pa), z["p_pb"]) <= 1e-13
    out = m.initialize(pa.copy())
    assert SC.rel_err(out["rho"], z["rho_height"]) <= 1e-13


def test_linked_list_matches_brute_force(sph):
    """test/test_linked_list.py:12-94: 26 x 26 points 1 apart, h = 1, scale 3."""
    xv = np.linspace(0, 25, 26)
    gx, gy = np.meshgrid(xv, xv, indexing="ij")
    pa = np.zeros(gx.size, dtype=sph.particle_dtype)
    pa["x"], pa["y"], pa["h"] = gx.ravel(), gy.ravel(), 1.0
    nn = sph.NNLinkedList(scale=3.0)
    nn.update(pa)
    hij, q, r, near0 = nn.near(0, pa)
    assert {0, 1, 26, 27} <= set(near0.tolist())
    d = np.hypot(pa["x"] - pa["x"][0], pa["y"] - pa["y"][0])
    assert set(near0.tolist()) == set(np.nonzero(d <= 3.0)[0].tolist())
    assert np.all(q <= 3.0)
    z = SC.load("nn_grid26")
    off, idx = nn.neighbour_sets()
    assert np.array_equal(off, z["offsets"]) and np.array_equal(idx, z["idx"])  # the reference's order too


def test_near_returns_the_reference_lists_in_order(sph):
    """NNLinkedList.near(i) (src/Tools/NNLinkedList.py:41-84) on the tank:
    nbrs in the reference's order (stencil cells with the x shift outer,
    descending index inside a cell) and the same h_ij, q, r, against the
    oracle's restatement of the reference."""
    import oracle
    from sph import scenarios as S
    pa = S.dam_break(width=0.2, height=0.4, dx=0.025, tank_width=0.8, tank_height=0.6)
    pa["h"][pa["label"] == 0] = 1.3 * 0.025
    nn = sph.NNLinkedList(2.0)
    nn.update(pa)
    ref = oracle.NN(2.0)
    ref.update(pa["x"], pa["y"], pa["h"])
    for i in (0, 1, 17, 40, len(pa) // 2, len(pa) - 1):
        hij, q, r, nb = nn.near(i, pa)
        rh, rq, rr, rn = ref.near(float(pa["x"][i]), float(pa["y"][i]), float(pa["h"][i]))
        assert nb.dtype == np.uint64
        assert np.array_equal(nb.astype(np.int64), rn), i
        assert np.array_equal(hij, rh) and np.array_equal(r, rr) and np.array_equal(q, rq), i


def _tank(sph, dx=0.025):
    from sph import scenarios as S
    return S.dam_break(width=0.2, height=0.4, dx=dx, tank_width=0.8, tank_height=0.6)


def test_solver_steps_match_oracle(sph):
    import oracle
    dx = 0.025
    pa = _tank(sph, dx)
    solver = sph.Solver(sph.WCSPH(0.4, dx, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline(), 1.0,
                        h=1.3 * dx, incrementalWriteout=False)
    solver.addParticles(pa.copy())
    solver.setup()
    P = oracle.Particles(arrays={k: pa[k] for k in pa.dtype.names if k != "deleted"})
    par = oracle.wcsph_params(0.4, dx, 1000.0)
    oracle.setup(P, par, 0.4, 1.3 * dx)
    hist = solver.step(5)
    dts = oracle.run(par, oracle.NN(2.0), P, 5, h_fixed=1.3 * dx)
    np.testing.assert_allclose(hist, dts, rtol=1e-12)
    solver._download()
    bad = SC.compare_state(solver.particleArray, P.as_dict(), SC.STATE_FIELDS, 1e-9)
    assert not bad, bad


def test_solver_run_settles_and_advances(sph, tmp_path):
    from sph.Common import ParticleType
    dx = 0.025
    pa = _tank(sph, dx)
    # a temporary wall that the end of settling removes (DamBreak.py:31)
    tmp = np.zeros(12, dtype=sph.particle_dtype)
    tmp["label"] = ParticleType.TempBoundary
    tmp["x"] = 0.21 + 0.0125
    tmp["y"] = (np.arange(12) + 0.5) * 0.0125 * 2
    pa = np.concatenate((pa, tmp))
    solver = sph.Solver(sph.WCSPH(0.4, dx, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline(),
                        duration=2e-3, h=1.3 * dx, maxSettle=5, incrementalWriteout=False,
                        exportProperties=["x", "y", "p"])
    solver.addParticles(pa)
    solver.setup()
    solver.run()
    assert solver.settled and solver.t >= 2e-3
    assert solver.t_step == len(solver.dt_a) == len(solver.export["x"])
    assert np.all(solver.particleArray["deleted"][solver.particleArray["label"] == ParticleType.TempBoundary])
    assert np.all(solver.particleArray["p"][solver.particleArray["label"] == ParticleType.TempBoundary] == -1e15)
    assert solver.settleTime == pytest.approx(sum(solver.dt_a[:6]))
    assert np.all(np.isfinite(solver.particleArray["x"]))
    path = str(tmp_path / "out.hdf5")
    solver.save(path, printLocation=False)
    s2 = sph.Solver(sph.WCSPH(0.4, dx, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline())
    import os
    s2.load(path if os.path.exists(path) else path + ".npz")
    np.testing.assert_array_equal(s2.particleArray["x"], solver.particleArray["x"])
    assert len(s2.dt_a) == len(solver.dt_a)


def test_newmark_matches_reference(sph):
    """src/Integrators/NewmarkBeta.py: predict / correct bit for bit,
    acceleration of the beam (banded) and of a dense system to rounding."""
    z = SC.load("newmark")
    n = 12
    for tag, (beta, gamma) in (("a", (0.25, 0.5)), ("b", (0.3025, 0.6))):
        pa = np.zeros(len(z["in_x"]), dtype=sph.particle_dtype)
        pa["label"] = 3
        for k in ("x", "y", "vx", "vy", "ax", "ay"):
            pa[k] = z["in_" + k]
        it = sph.NewmarkBeta(beta, gamma, np.eye(n), np.eye(n), np.eye(n))
        pa = it.predict(0.0021, pa, 0.0)
        for k in ("x", "y", "vx", "vy"):
            assert np.array_equal(pa[k], z[tag + "_pred_" + k]), (tag, k)
        pa = it.correct(0.0021, pa, 0.0)
        for k in ("x", "y", "vx", "vy"):
            assert np.array_equal(pa[k], z[tag + "_corr_" + k]), (tag, k)
    for tag, (beta, gamma, dt) in (("beam", (0.25, 0.5, 2.9e-4)), ("dense", (0.3025, 0.6, 0.01))):
        it = sph.NewmarkBeta(beta, gamma, z[tag + "_M"], z[tag + "_K"], z[tag + "_C"])
        a = it.acceleration(dt, z[tag + "_F"], z[tag + "_r"], z[tag + "_v"])
        assert SC.rel_err(a, z[tag + "_a"]) <= 1e-12, (tag, SC.rel_err(a, z[tag + "_a"]))
    kl, ku = 2, 2
    assert sph.Integrators.NewmarkBeta._bandwidths(z["beam_M"], z["beam_K"], z["beam_C"]) == (kl, ku)
    with pytest.raises(AssertionError):
        sph.NewmarkBeta(0.1, 0.5, np.eye(2), np.eye(2), np.eye(2))


def test_newmark_singular_and_large_systems(sph):
    """An exactly singular system raises LinAlgError like np.linalg.inv; a
    300-node beam and a 200-node dense system agree with numpy."""
    import oracle
    z = np.zeros((3, 3))
    it = sph.NewmarkBeta(0.25, 0.5, z, z, z)
    with pytest.raises(np.linalg.LinAlgError):
        it.acceleration(1e-3, np.ones(3), np.zeros(3), np.zeros(3))
    from sph import scenarios as S
    rng = np.random.default_rng(5)
    K, M = S.beam_matrices(300, 5e9, 0.25 ** 3 / 12, 0.25, 917.0, 0.05)
    Cm = np.eye(300) * 40.0
    F, r, v = rng.normal(0, 1e3, 300), rng.normal(0, 1e-3, 300), rng.normal(0, 1e-2, 300)
    a = sph.NewmarkBeta(0.25, 0.5, M, K, Cm).acceleration(1e-4, F, r, v)
    want = oracle.newmark_acceleration(M, K, Cm, 0.25, 0.5, 1e-4, F, r, v)
    assert SC.rel_err(a, want) <= 1e-10
    Md = np.eye(200) * 3 + rng.normal(0, 0.1, (200, 200))
    Kd, Cd = rng.normal(0, 10, (200, 200)), rng.normal(0, 1, (200, 200))
    F, r, v = rng.normal(0, 1, 200), rng.normal(0, 1, 200), rng.normal(0, 1, 200)
    a = sph.NewmarkBeta(0.25, 0.5, Md, Kd, Cd).acceleration(0.02, F, r, v)
    want = oracle.newmark_acceleration(Md, Kd, Cd, 0.25, 0.5, 0.02, F, r, v)
    assert SC.rel_err(a, want) <= 1e-10


def test_solver_coupled_run_matches_reference(sph):
    """Solver.run with a coupling function and NewmarkBeta as the coupling
    integrator (src/Solver.py:366-410), against the reference's own run of
    the same case: settling, Courant/force dt, fluid PEC, the beam's
    Newmark-beta predict / correct and its accelerations."""
    from sph import scenarios as S
    z = SC.load("solver_coupled")
    pa, P, (M, K, Cm) = SC.beam_case(S)
    dx = SC.BEAM["dx"]
    solver = sph.Solver(sph.WCSPH(0.4, dx, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline(),
                        SC.BEAM_RUN["duration"], incrementalWriteout=False, h=1.3 * dx,
                        maxSettle=SC.BEAM_RUN["maxSettle"], coupling=SC.beam_coupling,
                        couplingIntegrator=sph.NewmarkBeta(0.25, 0.5, M, K, Cm), couplingProperties=P,
                        customSettle=SC.settle_now, exportProperties=["x", "y", "p"])
    solver.addParticles(pa.copy())
    solver.setup()
    solver._download()
    for k in SC.STATE_FIELDS:
        assert SC.rel_err(solver.particleArray[k], z["init_" + k]) <= 1e-12, k  # pow / exp of the device
    solver.run()
    assert len(solver.dt_a) == len(z["dt_a"])
    np.testing.assert_allclose(solver.dt_a, z["dt_a"], rtol=1e-9)
    assert solver.settleTime == pytest.approx(float(z["settleTime"]), rel=1e-12)
    assert solver.t == pytest.approx(float(z["t"]), rel=1e-9)
    fin = solver.particleArray
    bad = {k: SC.rel_err(fin[k], z["final_" + k]) for k in ("x", "y", "vx", "vy", "rho", "p", "ax", "ay", "drho")
           if not SC.rel_err(fin[k], z["final_" + k]) <= 1e-8}
    assert not bad, bad
    c = fin["label"] == 3
    for k in ("x", "y", "vx", "vy", "ay"):
        assert SC.rel_err(fin[k][c], z["final_" + k][c]) <= 1e-8, k
    assert SC.rel_err(np.array(solver.export["y"]), z["export_y"]) <= 1e-8


def test_per_block_method_calls_match_reference(sph):
    """WCSPH.compute_density_change / compute_acceleration / compute_velocity
    on one particle and a computed_dtype block (src/Methods/WCSPH.py:151-203),
    and the boundary force of the same block, against the reference's
    equation functions on the golden blocks (src/Equations/Continuity.py,
    Momentum.py, BoundaryForce.py, XSPH.py)."""
    from sph import core
    z = SC.load("equations")
    for b in range(int(z["nblocks"])):
        J = len(z["b%d_r" % b])
        comp = np.zeros(J, dtype=sph.computed_dtype)
        for k in comp.dtype.names:
            if "b%d_%s" % (b, k) in z.files:
                comp[k] = z["b%d_%s" % (b, k)]
        p5, par6 = z["self5"][b], z["par6"][b]
        p = np.zeros(1, dtype=sph.particle_dtype)[0]
        p["p"], p["rho"], p["h"], p["c"], p["m"] = p5
        p["vx"], p["vy"] = 0.3, -0.2
        want = z["out"][b]
        for xsph in (False, True):
            m = sph.WCSPH(2.0, par6[2], 1000.0, xsph, 0.0)
            m.alpha, m.beta, m.D, m.p1, m.p2 = par6[0], par6[1], par6[3], par6[4], par6[5]

            def close(a, w):
                return abs(a - w) <= 1e-12 * max(1.0, abs(w))
            assert close(m.compute_density_change(p, comp), want[0]), b
            ax, ay = m.compute_acceleration(p, comp)
            assert close(ax, want[1]) and close(ay, want[2] - 9.81), b
            v = m.compute_velocity(p, comp)
            if xsph:
                assert v[:2] == [0.3, -0.2] and close(v[2], 0.3 + want[5]) and close(v[3], -0.2 + want[6]), b
            else:
                assert v == [0.3, -0.2, 0.0, 0.0]
            out = core.block_equations(comp, p, m.wcsph_struct())
            assert close(out[3], want[3]) and close(out[4], want[4]), b
        msd = sph.WCSPH(2.0, par6[2], 1000.0, False, 0.0, useSummationDensity=True)
        assert msd.compute_density_change(p, comp) == 0.0



def _plain_run(sph, chunk, export=("x", "y", "p")):
    from sph import scenarios as S
    pa, dx = SC.plain_run_case(S)
    solver = sph.Solver(sph.WCSPH(0.4, dx, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline(),
                        SC.PLAIN_RUN["duration"], incrementalWriteout=False, h=1.3 * dx,
                        customSettle=SC.settle_after_three, exportProperties=list(export))
    solver._chunk_max = chunk
    solver.addParticles(pa.copy())
    solver.setup()
    solver.run()
    return solver


def test_solver_plain_run_matches_reference(sph):
    """Solver.run without a coupling function (src/Solver.py:346-475): the
    settling steps one at a time, then chunks of steps with one host
    synchronisation each (rolled back and re-run when a chunk would pass the
    duration), against the reference's own run of the same case: the same
    number of steps, dt history, settling time, final state and per-step
    exports.  The same run with one step per chunk gives identical results."""
    z = SC.load("solver_plain")
    solver = _plain_run(sph, 64)
    assert solver.t_step == int(z["t_step"]) == len(solver.dt_a)
    np.testing.assert_allclose(solver.dt_a, z["dt_a"], rtol=1e-9)
    np.testing.assert_allclose(solver.dt_c, z["dt_c"], rtol=1e-9)
    np.testing.assert_allclose(solver.dt_f, z["dt_f"], rtol=1e-9)
    assert solver.settleTime == pytest.approx(float(z["settleTime"]), rel=1e-9)
    assert solver.t == pytest.approx(float(z["t"]), rel=1e-9)
    fin = solver.particleArray
    for k in ("x", "y", "vx", "vy", "rho", "p", "ax", "ay", "drho"):
        assert SC.rel_err(fin[k], z["final_" + k]) <= 1e-8, k
    assert np.array_equal(fin["deleted"], z["final_deleted"])
    every = SC.PLAIN_RUN["export_every"]
    assert len(solver.export["x"]) == solver.t_step
    assert SC.rel_err(np.array(solver.export["x"])[::every], z["export_x"]) <= 1e-8
    assert SC.rel_err(np.array(solver.export["p"])[::every], z["export_p"]) <= 1e-8
    one = _plain_run(sph, 1)
    assert one.dt_a == solver.dt_a and one.t_step == solver.t_step
    for k in ("x", "y", "vx", "vy", "rho", "p"):
        assert np.array_equal(one.particleArray[k], fin[k]), k


def test_solver_run_without_exports_runs_chunks_as_one_device_run(sph):
    """Without per-step export fields a settled chunk is one device run (its
    steps fused, on the sorted copy): the same steps, dt history and final
    state as the step-by-step chunks, within the reference tolerance of the
    plain-run case, and a neighbour table in the solver's own order after
    the run (the probes read it)."""
    from sph import core
    ref = _plain_run(sph, 64)
    bare = _plain_run(sph, 64, export=())
    assert bare.t_step == ref.t_step and len(bare.dt_a) == len(ref.dt_a)
    np.testing.assert_allclose(bare.dt_a, ref.dt_a, rtol=1e-9)
    assert bare.t == pytest.approx(ref.t, rel=1e-9)
    for k in ("x", "y", "vx", "vy", "rho", "p"):
        assert SC.rel_err(bare.particleArray[k], ref.particleArray[k]) <= 1e-8, k
    # c and the fixed h as the step-by-step chunks left them (the fused run
    # writes them back on its first and last steps only)
    for k in ("c", "h"):
        assert np.array_equal(bare.particleArray[k], ref.particleArray[k]), k
    # the table of the last build refers to the solver's own particle order
    off, idx = core.nn_export(bare._dp, bare._cfg(), bare._ws)
    core.nn_update(bare._dp, bare._cfg(), bare._ws)
    off2, idx2 = core.nn_export(bare._dp, bare._cfg(), bare._ws)
    assert np.array_equal(np.asarray(off), np.asarray(off2)) and np.array_equal(np.asarray(idx), np.asarray(idx2))
