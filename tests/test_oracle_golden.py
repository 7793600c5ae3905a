"""Pin the CPU oracle to the reference: every golden vector in tests/golden/
was produced by the unmodified Offshore-SPH source (see make_golden.py).

Formula-level cases mirror the reference's own unit tests
(test/test_kernels_cubic.py, test/test_kernels_Gaussian.py,
test/test_numba_momentum.py, test/test_numba_continuity.py,
test/test_eq_boundary.py, test/test_integrators_pec.py,
test/test_integrators_euler.py, test/test_linked_list.py); the solver cases
pin whole derivative evaluations and bare time steps, which the reference's
tests do not cover.
"""
import numpy as np
import pytest

import sphcases as SC

TOL = 1e-12


def test_kernels(oracle_lib):
    O = oracle_lib
    z = SC.load("kernels")
    assert SC.rel_err(O.kernel_eval(0, z["r"], z["h"]), z["cubic_w"]) <= TOL
    assert SC.rel_err(O.kernel_grad(0, z["x"], z["r"], z["h"]), z["cubic_grad"]) <= TOL
    assert SC.rel_err(O.kernel_eval(1, z["r"], z["h"]), z["gauss_w"]) <= TOL
    assert SC.rel_err(O.gauss_deriv(z["r"], z["h"]), z["gauss_deriv"]) <= TOL
    assert SC.rel_err(O.kernel_grad(1, z["x"], z["r"], z["h"]), z["gauss_grad"]) <= TOL
    # known answers of test/test_kernels_cubic.py:11-72
    fac = lambda h: 10 / (7 * np.pi * h * h)
    for q, h, want in [(0.5, 2.0, fac(2.0) * (1 - 1.5 * 0.25 * 0.75)), (1.0, 1.0, fac(1.0) * 0.25),
                       (1.5, 2 / 3, fac(2 / 3) * 0.25 * 0.125), (3.0, 1 / 3, 0.0)]:
        assert O.kernel_eval(0, [1.0], [h])[0] == pytest.approx(want, abs=1e-7)


def test_wendland_and_verlet(oracle_lib):
    """src/Kernels/Wendland.py and src/Integrators/Verlet.py against the
    reference's own outputs."""
    import oracle
    z = SC.load("wendland_verlet")
    assert SC.rel_err(oracle.kernel_eval(2, z["r"], z["h"]), z["wend_w"]) <= 1e-15
    assert SC.rel_err(oracle.kernel_grad(2, z["x"], z["r"], z["h"]), z["wend_grad"]) <= 1e-15
    for xs in (0, 1):
        P = oracle.Particles(arrays={k[3:]: z[k] for k in z.files if k.startswith("in_")})
        oracle.verlet_predict(P, 0.003)
        tag = "verlet_x%d" % xs
        for k in ("x", "y", "vx", "vy", "rho"):
            assert np.array_equal(getattr(P, k), z[tag + "_pred_" + k]), (tag, k)
        oracle.verlet_correct(P, 0.003, use_xsph=bool(xs))
        for k in ("x", "y", "vx", "vy", "rho"):
            assert np.array_equal(getattr(P, k), z[tag + "_corr_" + k]), (tag, k)


def test_newmark(oracle_lib):
    """src/Integrators/NewmarkBeta.py (predict, correct, acceleration) against
    the reference's own outputs."""
    import types
    import oracle
    z = SC.load("newmark")
    for tag, (beta, gamma) in (("a", (0.25, 0.5)), ("b", (0.3025, 0.6))):
        P = types.SimpleNamespace(**{k[3:]: z[k].copy() for k in z.files if k.startswith("in_")})
        oracle.newmark_predict(P, 0.0021, beta, gamma)
        for k in ("x", "y", "vx", "vy"):
            assert np.array_equal(getattr(P, k), z[tag + "_pred_" + k]), (tag, k)
        oracle.newmark_correct(P, 0.0021, beta, gamma)
        for k in ("x", "y", "vx", "vy"):
            assert np.array_equal(getattr(P, k), z[tag + "_corr_" + k]), (tag, k)
    for tag, (beta, gamma, dt) in (("beam", (0.25, 0.5, 2.9e-4)), ("dense", (0.3025, 0.6, 0.01))):
        a = oracle.newmark_acceleration(z[tag + "_M"], z[tag + "_K"], z[tag + "_C"], beta, gamma, dt,
                                        z[tag + "_F"], z[tag + "_r"], z[tag + "_v"])
        assert SC.rel_err(a, z[tag + "_a"]) <= 1e-13, tag


def test_probes(oracle_lib):
    """nearPos at points and the ice-coupling example's pressure interpolation
    (examples/IceBreak.py:253-285) against the reference's outputs."""
    import oracle
    z = SC.load("probes")
    P = oracle.Particles(arrays={k[3:]: z[k] for k in z.files if k.startswith("st_")})
    nn = oracle.NN(2.0)
    nn.update(P.x, P.y, P.h)
    h = float(z["h"])
    off = z["offsets"]
    for k, (x, y) in enumerate(zip(z["px"], z["py"])):
        hij, q, r, idx = nn.near(float(x), float(y), h)
        want = z["idx"][off[k]:off[k + 1]]  # the reference's own order
        assert np.array_equal(idx, want), k
        assert np.array_equal(r, z["r"][off[k]:off[k + 1]]) and np.array_equal(q, z["q"][off[k]:off[k + 1]])
        assert np.array_equal(hij, z["hij"][off[k]:off[k + 1]])
    par = oracle.wcsph_params(0.4, 0.025, 1000.0)
    rho, p = oracle.probe_density(nn, P, z["px"], z["py"], np.full(len(z["px"]), h), np.full(len(z["px"]), h), 0,
                                  1000.0, par.B, 7.0)
    ok = np.isfinite(z["rho"])
    assert np.array_equal(np.isfinite(rho), ok)
    assert SC.rel_err(rho[ok], z["rho"][ok]) <= 1e-14 and SC.rel_err(p[ok], z["p"][ok]) <= 1e-12


def test_equations(oracle_lib):
    O = oracle_lib
    z = SC.load("equations")
    for b in range(int(z["nblocks"])):
        comp = {k: z["b%d_%s" % (b, k)] for k in ("label", "m", "p", "rho", "h", "r", "w", "dw_x", "dw_y",
                                                  "x", "y", "vx", "vy")}
        out = O.equations(comp, z["self5"][b], z["par6"][b])
        want = z["out"][b]
        for k in range(7):
            assert abs(out[k] - want[k]) <= 1e-12 * max(1.0, abs(want[k])), (b, k, out[k], want[k])


def test_boundary_force_sign(oracle_lib):
    """test/test_eq_boundary.py:9-26: a boundary at (-1, 0), r0 = 2 pushes +x."""
    comp = dict(label=np.array([1, 0], np.int8), m=np.zeros(2), p=np.zeros(2), rho=np.zeros(2), h=np.zeros(2),
                r=np.array([1.0, 1.0]), w=np.zeros(2), dw_x=np.zeros(2), dw_y=np.zeros(2),
                x=np.array([1.0, -1.0]), y=np.zeros(2), vx=np.zeros(2), vy=np.zeros(2))
    out = oracle_lib.equations(comp, [0, 1, 1, 0, 1], [0.01, 0.0, 2.0, 5 * 9.81, 4.0, 2.0])
    assert out[3] > 0 and out[4] == 0


def test_eos_and_integrators(oracle_lib):
    O = oracle_lib
    z = SC.load("eos_integrators")
    par = O.wcsph_params(2.0, 0.025, 1000.0)
    assert par.co == pytest.approx(float(z["co"]), rel=1e-15)
    assert par.B == pytest.approx(float(z["B"]), rel=1e-15)
    assert SC.rel_err(O.eos(z["label"], z["rho"], par), z["p"]) <= TOL
    par2 = O.wcsph_params(3.0, 0.025, 1000.0, Pb=101325.0)
    assert SC.rel_err(O.eos(z["label"], z["rho"], par2), z["p_pb"]) <= TOL
    assert SC.rel_err(O.tait_height(z["y"], par, 2.0), z["rho_height"]) <= TOL

    base = {k: z["in_" + k] for k in ("label",) + SC.STATE_FIELDS}
    for xs in (0, 1):
        for strict in (0, 1):
            for d in (0, 5):
                P = O.Particles(arrays=base)
                O.pec_predict(P, 0.003, d / 100.0, xs, strict)
                tag = "pec_x%d_s%d_d%d" % (xs, strict, d)
                for k in ("x", "y", "vx", "vy", "rho", "x0", "y0", "vx0", "vy0", "rho0"):
                    assert SC.rel_err(getattr(P, k), z[tag + "_pred_" + k]) <= TOL, (tag, k)
                O.pec_correct(P, 0.003, d / 100.0, xs, strict)
                for k in ("x", "y", "vx", "vy", "rho"):
                    assert SC.rel_err(getattr(P, k), z[tag + "_corr_" + k]) <= TOL, (tag, k)
    P = O.Particles(arrays=base)
    O.euler_correct(P, 0.003)
    for k in ("x", "y", "vx", "vy", "rho"):
        assert SC.rel_err(getattr(P, k), z["euler_" + k]) <= TOL
    P = O.Particles(arrays=base)
    np.testing.assert_allclose(O.timestep(P, 0.25, 0.25), z["ts"], rtol=1e-14)
    np.testing.assert_allclose(O.timestep(P, 0.3, 0.25), z["ts_c03"], rtol=1e-14)
    P.ax[:] = 0
    P.ay[:] = 0
    np.testing.assert_allclose(O.timestep(P, 0.3, 0.25), z["ts_zero_a"], rtol=1e-14)


def test_pec_single_particle_known_answers(oracle_lib):
    """test/test_integrators_pec.py:13-76 with dt = 2, useXSPH False."""
    O = oracle_lib
    P = O.Particles(1)
    P.vx[0], P.vy[0], P.ax[0], P.ay[0], P.drho[0] = 1.0, 3.0, 5.0, 0.0, 10.0
    O.pec_predict(P, 2.0, 0.0, False, True)
    assert P.x[0] == pytest.approx(1.0) and P.y[0] == pytest.approx(3.0) and P.rho[0] == pytest.approx(10.0)
    O.pec_correct(P, 2.0, 0.0, False, True)
    assert P.x[0] == pytest.approx(2.0 + 0.5 * 5 * 2 * 2) and P.y[0] == pytest.approx(6.0)
    assert P.rho[0] == pytest.approx(20.0)
    E = O.Particles(1)
    E.vx[0], E.vy[0], E.ax[0], E.ay[0], E.drho[0] = 1.0, 3.0, 5.0, 0.0, 10.0
    O.euler_correct(E, 2.0)
    for k in ("x", "y", "vx", "vy", "rho"):
        assert getattr(E, k)[0] == pytest.approx(getattr(P, k)[0])


@pytest.mark.parametrize("name", ["nn_lattice", "nn_tank", "nn_alias", "nn_alias_boundary", "nn_grid26"])
def test_nn_lists_bit_exact(oracle_lib, name):
    O = oracle_lib
    z = SC.load(name)
    nn = O.NN(float(z["scale"]))
    st = nn.update(z["x"], z["y"], z["h"])
    assert st == 0
    g = nn.grid()
    np.testing.assert_array_equal([g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["cell_size"]], z["grid"])
    np.testing.assert_array_equal([g["ncx"], g["ncy"], g["n_cells"]], z["ncells"])
    heads, nexts = nn.lists()
    np.testing.assert_array_equal(heads, z["heads"])
    np.testing.assert_array_equal(nexts, z["nexts"])
    off, idx = nn.all()
    np.testing.assert_array_equal(off, z["offsets"])
    np.testing.assert_array_equal(idx, z["idx"])


def test_nn_grid26_matches_brute_force(oracle_lib):
    """test/test_linked_list.py:12-94: with scale 3 (cell >= 3h) particle 0's
    neighbour set equals the brute-force set {q <= 3}."""
    z = SC.load("nn_grid26")
    nn = oracle_lib.NN(3.0)
    nn.update(z["x"], z["y"], z["h"])
    _, _, _, near0 = nn.near(z["x"][0], z["y"][0], z["h"][0])
    r = np.hypot(z["x"] - z["x"][0], z["y"] - z["y"][0])
    assert set(near0.tolist()) == set(np.nonzero(r / 1.0 <= 3.0)[0].tolist())
    assert {0, 1, 26, 27} <= set(near0.tolist())


def test_nn_alias_semantics(oracle_lib):
    """The x-overflow alias: particles at x = xmax with an integral extent sit
    in cell (0, cy+1) and are invisible to their physical neighbours."""
    z = SC.load("nn_alias_boundary")
    nn = oracle_lib.NN(2.0)
    nn.update(z["x"], z["y"], z["h"])
    g = nn.grid()
    assert g["cell_size"] == 1.0 and g["ncx"] == 3
    off, idx = nn.all()
    right = set(np.nonzero(z["x"] == 3.0)[0].tolist())
    fluid = np.nonzero(z["label"] == 0)[0]
    # no fluid particle sees the aliased right wall, although many are within 3 h_ij
    seen = set()
    for i in fluid:
        seen |= set(idx[off[i]:off[i + 1]].tolist())
    assert not (seen & right)


def test_nn_reports_cell_overflow(oracle_lib):
    """A particle at y = ymax with an integral y extent gets a flat id past
    heads[] (an out-of-bounds write in the reference): the oracle reports it."""
    x = np.array([0.0, 1.0, 2.0, 0.5])
    y = np.array([0.0, 0.0, 2.0, 1.0])
    h = np.full(4, 0.5)
    nn = oracle_lib.NN(2.0)
    assert nn.update(x, y, h) == oracle_lib.OR_ERR_CELL_OVERFLOW


@pytest.mark.parametrize("name", SC.SOLVER_CASES)
def test_solver_cases(oracle_lib, name):
    meta, init, ev, steps, dts = SC.load_case(name)
    P, st = SC.oracle_eval(meta, init)
    assert st == 0
    bad = SC.compare_state(P, ev, ("rho", "p", "c", "drho", "h", "ax", "ay", "xsphx", "xsphy", "vx", "vy"), TOL)
    assert not bad, bad
    if steps:
        P, got_dts = SC.oracle_steps(meta, init, len(steps))
        np.testing.assert_allclose(got_dts, dts, rtol=1e-12)
        bad = SC.compare_state(P, steps[-1], SC.STATE_FIELDS, 1e-11)
        assert not bad, bad


def test_solver_cases_threaded_equal(oracle_lib):
    """OpenMP over particles gives the same bits (each particle writes only itself)."""
    meta, init, ev, steps, dts = SC.load_case("solver_tank_cubic")
    P1, _ = SC.oracle_eval(meta, init, nthreads=1)
    P4, _ = SC.oracle_eval(meta, init, nthreads=4)
    for k in ("drho", "ax", "ay"):
        np.testing.assert_array_equal(getattr(P1, k), getattr(P4, k))


def test_large_dam_break_eval(oracle_lib):
    import os
    if not os.path.exists(SC.os.path.join(SC.GOLDEN, "solver_cfg_dam_break_small.npz")):
        pytest.skip("full-size golden not generated")
    meta, init, ev, steps, dts = SC.load_case("solver_cfg_dam_break_small")
    P, st = SC.oracle_eval(meta, init, nthreads=4)
    assert st == 0
    bad = SC.compare_state(P, ev, ("rho", "p", "drho", "ax", "ay"), TOL)
    assert not bad, bad
    P, got = SC.oracle_steps(meta, init, len(steps), nthreads=4)
    np.testing.assert_allclose(got, dts, rtol=1e-12)
    bad = SC.compare_state(P, steps[-1], SC.STATE_FIELDS, 1e-11)
    assert not bad, bad
