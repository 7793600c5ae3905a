"""Generate the golden vectors in tests/golden/ from the reference itself.

Offshore-SPH is pure Python + numba 0.42 (``requirements.txt:8``); numba is not
installable offline, so this script installs a small pure-Python stand-in
before importing the reference: ``njit``/``jit``/``jitclass`` become
pass-through decorators, ``vectorize`` becomes ``numpy.vectorize`` with a
float64 output, ``prange`` becomes ``range`` and the numba type objects are
inert.  h5py, colorama and prettytable (imported by ``src/Solver.py`` but not
used by the step) are stubbed the same way.  The reference source itself runs
unmodified, read from the path given by ``--ref``.

Everything runs in pure Python, so the cases are small (the full 4808-particle
dam break costs about a minute per derivative evaluation).

Usage:  python tests/golden/make_golden.py --ref <Offshore-SPH checkout> [--skip-large]
"""
import argparse
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "offshore-sph_gb300"))


# ---------------------------------------------------------------------------
# numba / h5py / colorama / prettytable stand-ins
# ---------------------------------------------------------------------------
def _install_shims():
    nb = types.ModuleType("numba")

    def _passthrough(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    def _jitclass(spec=None):
        return lambda cls: cls

    def _vectorize(*args, **kwargs):
        def deco(f):
            return np.vectorize(f, otypes=[np.float64])
        return deco

    class _Type:
        def __getitem__(self, item):
            return self

        def __call__(self, *a, **k):
            return self

    nb.njit = _passthrough
    nb.jit = _passthrough
    nb.jitclass = _jitclass
    nb.vectorize = _vectorize
    nb.prange = range
    for t in ("float64", "int64", "boolean", "int8", "float32", "int32", "uint64", "void"):
        setattr(nb, t, _Type())
    sys.modules["numba"] = nb

    h5 = types.ModuleType("h5py")
    h5.File = None
    sys.modules["h5py"] = h5

    col = types.ModuleType("colorama")

    class _Attr:
        def __getattr__(self, k):
            return ""

    col.Fore = _Attr()
    col.Style = _Attr()
    sys.modules["colorama"] = col

    pt = types.ModuleType("prettytable")

    class PrettyTable:
        def __init__(self, *a, **k):
            pass

        def add_row(self, *a, **k):
            pass

    pt.PrettyTable = PrettyTable
    sys.modules["prettytable"] = pt


# ---------------------------------------------------------------------------
def _save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, "(%.1f KB)" % (os.path.getsize(path) / 1024.0))


def gen_kernels(ref):
    from src.Kernels.CubicSpline import CubicSpline
    from src.Kernels.Gaussian import Gaussian
    rng = np.random.default_rng(11)
    n = 600
    h = rng.uniform(0.05, 2.0, n)
    q = rng.uniform(0.0, 3.6, n)
    q[:8] = [0.0, 0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 3.0000001]
    r = q * h
    x = r * np.cos(rng.uniform(0, 2 * np.pi, n))
    r[8] = 5e-11  # below the cubic gradient's r guard
    _save("kernels.npz", r=r, h=h, x=x,
          cubic_w=CubicSpline.evaluate(r, h), cubic_grad=CubicSpline.gradient(x, r, h),
          gauss_w=np.asarray(Gaussian.evaluate(r, h), dtype=np.float64),
          gauss_deriv=np.asarray(Gaussian.derivative(r, h), dtype=np.float64),
          gauss_grad=np.asarray(Gaussian.gradient(x, r, h), dtype=np.float64))


def gen_equations(ref):
    from src.Common import computed_dtype, particle_dtype, ParticleType
    from src.Equations.Continuity import Continuity
    from src.Equations.Momentum import Momentum
    from src.Equations.BoundaryForce import BoundaryForce
    from src.Equations.XSPH import XSPH
    rng = np.random.default_rng(12)
    blocks = []
    outs = []
    selfs = []
    pars = []
    for b in range(6):
        J = int(rng.integers(1, 60))
        comp = np.zeros(J, dtype=computed_dtype)
        comp["label"] = rng.integers(0, 2, J)
        comp["m"] = rng.uniform(0.1, 1.0, J)
        comp["p"] = rng.uniform(-100, 5000, J)
        comp["rho"] = rng.uniform(950, 1050, J)
        comp["h"] = rng.uniform(0.01, 0.05, J)
        comp["x"] = rng.uniform(-0.06, 0.06, J)
        comp["y"] = rng.uniform(-0.06, 0.06, J)
        comp["r"] = np.sqrt(comp["x"] ** 2 + comp["y"] ** 2)
        comp["r"][0] = 0.0
        comp["vx"] = rng.normal(0, 1, J)
        comp["vy"] = rng.normal(0, 1, J)
        comp["w"] = rng.uniform(0, 500, J)
        comp["dw_x"] = rng.normal(0, 1e4, J)
        comp["dw_y"] = rng.normal(0, 1e4, J)
        p = np.zeros(1, dtype=particle_dtype)[0]
        p["p"] = rng.uniform(0, 5000)
        p["rho"] = rng.uniform(950, 1050)
        p["h"] = rng.uniform(0.01, 0.05)
        p["c"] = rng.uniform(10, 100)
        p["m"] = rng.uniform(0.1, 1)
        alpha, beta = 0.01 * (b + 1), 0.1 * b
        r0, D = 0.04, 5 * 9.81 * 2.0
        drho = Continuity(p, comp)
        ax, ay = Momentum(alpha, beta, p, comp)
        bx, by = BoundaryForce(r0, D, 4.0, 2.0, p, comp)
        sx, sy = XSPH(0.5, p, comp)
        blocks.append(comp)
        outs.append([drho, ax, ay, bx, by, sx, sy])
        selfs.append([p["p"], p["rho"], p["h"], p["c"], p["m"]])
        pars.append([alpha, beta, r0, D, 4.0, 2.0])
    d = {}
    for b, comp in enumerate(blocks):
        for k in comp.dtype.names:
            d["b%d_%s" % (b, k)] = comp[k]
    _save("equations.npz", nblocks=len(blocks), out=np.array(outs), self5=np.array(selfs),
          par6=np.array(pars), **d)


def _soa(pa):
    return {k: np.array(pa[k]) for k in pa.dtype.names}


def gen_eos_integrators(ref):
    from src.Common import particle_dtype, ParticleType
    from src.Methods.WCSPH import WCSPH
    from src.Integrators.PEC import PEC
    from src.Integrators.Euler import Euler
    from src.Equations.TimeStep import TimeStep
    from src.Equations import TaitEOS
    rng = np.random.default_rng(13)
    n = 200
    pa = np.zeros(n, dtype=particle_dtype)
    pa["label"] = rng.integers(0, 2, n)
    pa["rho"] = rng.uniform(900, 1100, n)
    pa["y"] = rng.uniform(0, 2, n)
    m = WCSPH(height=2.0, r0=0.025, rho0=1000.0, useXSPH=False, Pb=0.0, useSummationDensity=False)
    p = np.asarray(m.compute_pressure(pa), dtype=np.float64)
    m2 = WCSPH(height=3.0, r0=0.025, rho0=1000.0, useXSPH=False, Pb=101325.0, useSummationDensity=False)
    p2 = np.asarray(m2.compute_pressure(pa), dtype=np.float64)
    rho_h = np.asarray(TaitEOS.TaitEOS_height(m.rho0, m.height, m.B, m.gamma, pa["y"]), dtype=np.float64)

    # integrators on fluid-only arrays, as the Solver passes them
    f = np.zeros(64, dtype=particle_dtype)
    f["label"] = 0
    for k in ("x", "y", "vx", "vy", "ax", "ay", "drho", "xsphx", "xsphy"):
        f[k] = rng.normal(0, 1, len(f))
    f["rho"] = rng.uniform(-1, 1000, len(f))
    f["h"] = rng.uniform(0.01, 0.03, len(f))
    f["c"] = 62.6
    res = {}
    for xs in (False, True):
        for strict in (False, True):
            for damping in (0.0, 0.05):
                it = PEC(useXSPH=xs, strict=strict)
                a = f.copy()
                a = it.predict(0.003, a, damping)
                pred = a.copy()
                a = it.correct(0.003, a, damping)
                tag = "pec_x%d_s%d_d%d" % (xs, strict, int(damping * 100))
                for k in ("x", "y", "vx", "vy", "rho", "x0", "y0", "vx0", "vy0", "rho0"):
                    res[tag + "_pred_" + k] = pred[k]
                    res[tag + "_corr_" + k] = a[k]
    e = f.copy()
    e = Euler().correct(0.003, e, 0.0)
    for k in ("x", "y", "vx", "vy", "rho"):
        res["euler_" + k] = e[k]
    ts = np.array(TimeStep().compute(len(f), f, 0.25, 0.25))
    ts2 = np.array(TimeStep().compute(len(f), f, 0.3, 0.25))
    g = f.copy()
    g["ax"] = 0.0
    g["ay"] = 0.0
    ts3 = np.array(TimeStep().compute(len(g), g, 0.3, 0.25))
    _save("eos_integrators.npz", label=pa["label"], rho=pa["rho"], y=pa["y"], p=p, p_pb=p2, rho_height=rho_h,
          co=m.co, B=m.B, co2=m2.co, B2=m2.B, ts=ts, ts_c03=ts2, ts_zero_a=ts3,
          **{"in_" + k: np.array(f[k]) for k in f.dtype.names if k != "deleted"}, **res)


def gen_extra(ref):
    """Wendland C4 kernel values and gradients; Verlet predict / correct on a
    fluid-only array."""
    from src.Common import particle_dtype
    from src.Kernels.Wendland import Wendland
    from src.Integrators.Verlet import Verlet
    rng = np.random.default_rng(11)
    n = 500
    h = rng.uniform(0.01, 0.05, n)
    r = rng.uniform(0, 2.2, n) * h
    r[:5] = [0.0, 1e-11, 2.0 * h[2], 1.999999 * h[3], 1.0 * h[4]]
    x = r * rng.uniform(-1, 1, n)
    res = dict(r=r, h=h, x=x, wend_w=np.asarray(Wendland.evaluate(r, h), dtype=np.float64),
               wend_grad=np.asarray(Wendland.gradient(x, r, h), dtype=np.float64))
    rng = np.random.default_rng(17)
    f = np.zeros(64, dtype=particle_dtype)
    f["label"] = 0
    for k in ("x", "y", "vx", "vy", "ax", "ay", "drho", "xsphx", "xsphy"):
        f[k] = rng.normal(0, 1, len(f))
    f["rho"] = rng.uniform(900, 1100, len(f))
    for k in f.dtype.names:
        if k != "deleted":
            res["in_" + k] = np.array(f[k])
    for xs in (False, True):
        it = Verlet(xs)
        a = it.predict(0.003, f.copy(), 0.0)
        tag = "verlet_x%d" % xs
        for k in ("x", "y", "vx", "vy", "rho"):
            res[tag + "_pred_" + k] = np.array(a[k])
        a = it.correct(0.003, a, 0.0)
        for k in ("x", "y", "vx", "vy", "rho"):
            res[tag + "_corr_" + k] = np.array(a[k])
    _save("wendland_verlet.npz", **res)


def gen_probes(ref):
    """nearPos at points and the ice-coupling example's pressure
    interpolation (examples/IceBreak.py:253-285) on the small tank after
    Solver.setup and one _compute."""
    from src.Solver import Solver
    from src.Methods.WCSPH import WCSPH
    from src.Kernels.CubicSpline import CubicSpline
    from src.Integrators.PEC import PEC
    from src.Tools.NNLinkedList import NNLinkedList
    from src.Equations.Shepard import Shepard
    from src.Equations.SummationDensity import SummationDensity
    from sph import scenarios as S
    dx = 0.025
    tank = S.dam_break(width=0.2, height=0.4, dx=dx, tank_width=0.8, tank_height=0.6)
    method = WCSPH(height=0.4, r0=dx, rho0=1000.0, useXSPH=False, Pb=0.0, useSummationDensity=False)
    solver = Solver(method, PEC(False, True), CubicSpline(), 1.0, incrementalWriteout=False, h=1.3 * dx, damping=0.0)
    Solver.particleArray = None
    solver.particleArray = None
    solver.addParticles(tank.copy())
    solver.setup()
    solver._compute()
    pA = solver.particleArray
    nn = NNLinkedList(2.0)
    nn.update(pA)
    rng = np.random.default_rng(23)
    px = np.concatenate([rng.uniform(-0.05, 0.85, 16), [0.1, 0.19, 0.01, 0.21, 0.4, -0.3, 1.2, 0.0]])
    py = np.concatenate([rng.uniform(-0.05, 0.5, 16), [0.2, 0.39, 0.01, 0.05, 0.1, 0.2, 0.1, 0.0]])
    h = 1.3 * dx
    offs, idx, hijs, qs, rs, rhos, ps = [0], [], [], [], [], [], []
    for x, y in zip(px, py):
        hij, q, r, nb = nn.nearPos(float(x), float(y), h, pA)
        # the reference's own order (stencil cells, head-insert order inside)
        idx.extend(np.asarray(nb).tolist())
        hijs.extend(np.asarray(hij).tolist())
        qs.extend(np.asarray(q).tolist())
        rs.extend(np.asarray(r).tolist())
        offs.append(len(idx))
        w = CubicSpline.evaluate(np.asarray(r, dtype=np.float64), np.ones(len(nb)) * h)
        wt = Shepard(w, pA[nb]["label"], pA[nb]["m"], pA[nb]["rho"])
        rho = SummationDensity(pA[nb]["label"], pA[nb]["m"], wt)
        p = ((rho / method.rho0) ** method.gamma - 1.0) * method.B
        rhos.append(rho)
        ps.append(p)
    _save("probes.npz", px=px, py=py, h=h, offsets=np.array(offs), idx=np.array(idx, dtype=np.int64),
          hij=np.array(hijs), q=np.array(qs), r=np.array(rs), rho=np.array(rhos), p=np.array(ps),
          **{"st_" + k: np.array(pA[k]) for k in pA.dtype.names if k != "deleted"})


def gen_newmark(ref):
    """NewmarkBeta (src/Integrators/NewmarkBeta.py): predict / correct of
    Coupled particles, acceleration of the coupling example's beam and of a
    dense system; then Solver.run with a beam coupling function
    (src/Solver.py:346-475 with coupling, couplingIntegrator)."""
    from src.Common import particle_dtype
    from src.Integrators.NewmarkBeta import NewmarkBeta
    from sph import scenarios as S
    sys.path.insert(0, os.path.dirname(HERE))
    import sphcases as SC
    res = {}
    rng = np.random.default_rng(31)
    f = np.zeros(40, dtype=particle_dtype)
    f["label"] = 3
    for k in ("x", "y", "vx", "vy", "ax", "ay"):
        f[k] = rng.normal(0, 1, len(f))
    for k in ("x", "y", "vx", "vy", "ax", "ay"):
        res["in_" + k] = np.array(f[k])
    n = 12
    K0, M0 = S.beam_matrices(n, 2e6, 0.02 ** 3 / 12, 0.02, 917.0, 0.025)
    for tag, (beta, gamma) in (("a", (0.25, 0.5)), ("b", (0.3025, 0.6))):
        it = NewmarkBeta(beta, gamma, M0, K0, np.eye(n))
        a = it.predict(0.0021, f.copy(), 0.0)
        for k in ("x", "y", "vx", "vy"):
            res[tag + "_pred_" + k] = np.array(a[k])
        a = it.correct(0.0021, a, 0.0)
        for k in ("x", "y", "vx", "vy"):
            res[tag + "_corr_" + k] = np.array(a[k])
    # accelerations: the beam (banded) and a dense, nonsymmetric system
    M, K, C = SC.beam_case(S)[2]
    nb = M.shape[0]
    F, r, v = rng.normal(0, 10, nb), rng.normal(0, 1e-3, nb), rng.normal(0, 1e-2, nb)
    res.update(beam_M=M, beam_K=K, beam_C=C, beam_F=F, beam_r=r, beam_v=v,
               beam_a=NewmarkBeta(0.25, 0.5, M, K, C).acceleration(2.9e-4, F, r, v))
    nd = 24
    Md = np.diag(rng.uniform(1, 2, nd)) + 0.1 * rng.normal(0, 1, (nd, nd))
    Kd = rng.normal(0, 50, (nd, nd))
    Cd = rng.normal(0, 5, (nd, nd))
    F, r, v = rng.normal(0, 1, nd), rng.normal(0, 1, nd), rng.normal(0, 1, nd)
    res.update(dense_M=Md, dense_K=Kd, dense_C=Cd, dense_F=F, dense_r=r, dense_v=v,
               dense_a=NewmarkBeta(0.3025, 0.6, Md, Kd, Cd).acceleration(0.01, F, r, v))
    _save("newmark.npz", **res)
    gen_coupled_run(ref)


def gen_coupled_run(ref):
    """Solver.run of the small tank with the beam of Coupled particles above
    the water, coupling = sphcases.beam_coupling, NewmarkBeta(1/4, 1/2)."""
    from src.Solver import Solver
    from src.Methods.WCSPH import WCSPH
    from src.Kernels.CubicSpline import CubicSpline
    from src.Integrators.PEC import PEC
    from src.Integrators.NewmarkBeta import NewmarkBeta
    from sph import scenarios as S
    sys.path.insert(0, os.path.dirname(HERE))
    import sphcases as SC
    pa, P, (M, K, C) = SC.beam_case(S)
    dx = SC.BEAM["dx"]
    method = WCSPH(height=0.4, r0=dx, rho0=1000.0, useXSPH=False, Pb=0.0, useSummationDensity=False)
    solver = Solver(method, PEC(False, True), CubicSpline(), SC.BEAM_RUN["duration"], incrementalWriteout=False,
                    h=1.3 * dx, maxSettle=SC.BEAM_RUN["maxSettle"], coupling=SC.beam_coupling,
                    couplingIntegrator=NewmarkBeta(0.25, 0.5, M, K, C), couplingProperties=P,
                    customSettle=SC.settle_now, exportProperties=["x", "y", "p"])
    Solver.particleArray = None
    solver.particleArray = None
    solver.addParticles(pa.copy())
    t0 = time.time()
    solver.setup()
    init = solver.particleArray.copy()
    solver.run()
    fin = solver.particleArray
    _save("solver_coupled.npz", dt_a=np.array(solver.dt_a), t=solver.t, settleTime=solver.settleTime,
          **{"init_" + k: np.array(init[k]) for k in init.dtype.names},
          **{"final_" + k: np.array(fin[k]) for k in fin.dtype.names},
          export_y=np.array(solver.export["y"]))
    print("  solver_coupled: %.1f s, %d steps" % (time.time() - t0, len(solver.dt_a)))


def gen_plain_run(ref):
    """Solver.run of the small tank with a temporary gate, no coupling:
    settling (damping 0.05) ended by customSettle after three steps, the
    gate deleted, then Courant/force dt steps to the duration."""
    from src.Solver import Solver
    from src.Methods.WCSPH import WCSPH
    from src.Kernels.CubicSpline import CubicSpline
    from src.Integrators.PEC import PEC
    from sph import scenarios as S
    sys.path.insert(0, os.path.dirname(HERE))
    import sphcases as SC
    pa, dx = SC.plain_run_case(S)
    method = WCSPH(height=0.4, r0=dx, rho0=1000.0, useXSPH=False, Pb=0.0, useSummationDensity=False)
    solver = Solver(method, PEC(False, True), CubicSpline(), SC.PLAIN_RUN["duration"], incrementalWriteout=False,
                    h=1.3 * dx, customSettle=SC.settle_after_three, exportProperties=["x", "y", "p"])
    Solver.particleArray = None
    solver.particleArray = None
    solver.addParticles(pa.copy())
    t0 = time.time()
    solver.setup()
    init = solver.particleArray.copy()
    solver.run()
    fin = solver.particleArray
    _save("solver_plain.npz", dt_a=np.array(solver.dt_a), dt_c=np.array(solver.dt_c), dt_f=np.array(solver.dt_f),
          t=solver.t, settleTime=solver.settleTime, t_step=solver.t_step,
          **{"init_" + k: np.array(init[k]) for k in init.dtype.names},
          **{"final_" + k: np.array(fin[k]) for k in fin.dtype.names},
          export_x=np.array(solver.export["x"])[::SC.PLAIN_RUN["export_every"]],
          export_p=np.array(solver.export["p"])[::SC.PLAIN_RUN["export_every"]])
    print("  solver_plain: %.1f s, %d steps" % (time.time() - t0, len(solver.dt_a)))


def _nn_case(name, pa, scale=2.0):
    from src.Tools.NNLinkedList import NNLinkedList
    nn = NNLinkedList(scale)
    nn.update(pa)
    offs = [0]
    idx = []
    qs = []
    for i in range(len(pa)):
        h_i, q_i, r_i, nb = nn.near(i, pa)
        idx.extend(list(nb))
        qs.extend(list(q_i))
        offs.append(len(idx))
    _save(name, x=pa["x"], y=pa["y"], h=pa["h"], label=pa["label"], scale=scale,
          grid=np.array([nn.xmin, nn.xmax, nn.ymin, nn.ymax, nn.cell_size]),
          ncells=np.array([nn.ncells_per_dim[0], nn.ncells_per_dim[1], nn.n_cells]),
          heads=np.array(nn.heads), nexts=np.array(nn.nexts),
          offsets=np.array(offs, dtype=np.int64), idx=np.array(idx, dtype=np.int64), q=np.array(qs))


def alias_case():
    """All-fluid lattice where (xmax - xmin)/cell_size is an exact integer, so
    the particles at x = xmax bin to cx = ncx and alias into cell (0, cy+1)
    (src/Tools/NNLinkedList.py:112-141, 200-208).  The top rows stay below
    x = xmax so that no flat index leaves heads[]."""
    from sph.Common import particle_dtype
    xs = np.arange(17) * 0.25
    ys = np.arange(10) * 0.3
    x, y = np.meshgrid(xs, ys, indexing="ij")
    keep = ~((x > 3.99) & (y >= 2.0))
    pa = np.zeros(int(keep.sum()), dtype=particle_dtype)
    pa["x"] = x[keep]
    pa["y"] = y[keep]
    pa["h"] = 0.5
    pa["m"] = 0.0625 * 1000.0
    rng = np.random.default_rng(5)
    pa["rho"] = 1000.0 * (1 + rng.uniform(-0.01, 0.01, len(pa)))
    pa["vx"] = rng.normal(0, 0.1, len(pa))
    pa["vy"] = rng.normal(0, 0.1, len(pa))
    return pa


def alias_boundary_case():
    """Tank with h = 0 boundaries (so cell_size = 1.0) spanning x in [0, 3]
    exactly: the right-wall particles at x = 3 bin to cx = ncx = 3 and alias
    into column 0 of the next row, where fluid in column 2 never looks
    (src/Tools/NNLinkedList.py:112-141, 178-208).  The right wall stops below
    y = 1 so that the aliased flat ids stay inside heads[]."""
    from sph.Common import particle_dtype, ParticleType
    s = 0.0125
    floor_x = (np.arange(240) + 0.5) * s
    parts = []
    def rows(xs, ys, lab):
        gx, gy = np.meshgrid(xs, ys, indexing="ij")
        pa = np.zeros(gx.size, dtype=particle_dtype)
        pa["x"], pa["y"], pa["label"] = gx.ravel(), gy.ravel(), lab
        return pa
    dx = 0.025
    fl = rows(3.0 - 0.2 + (np.arange(8) + 0.5) * dx, (np.arange(12) + 0.5) * dx, ParticleType.Fluid)
    fl["m"] = 1000.0 * dx * dx
    fl["rho"] = 1000.0
    parts.append(fl)
    parts.append(rows(floor_x, np.array([0.0]), ParticleType.Boundary))
    parts.append(rows(np.array([0.0]), np.arange(121) * s, ParticleType.Boundary))
    parts.append(rows(np.array([3.0]), np.arange(73) * s, ParticleType.Boundary))
    return np.concatenate(parts)


def gen_nn(ref):
    from sph import scenarios as S
    lat = S.jittered_lattice(24, 24, 0.01, seed=3)
    lat["h"] = 0.013
    _nn_case("nn_lattice.npz", lat)
    tank = S.dam_break(width=0.2, height=0.4, dx=0.025, tank_width=0.8, tank_height=0.6)
    tank["h"][tank["label"] == 0] = 1.3 * 0.025
    _nn_case("nn_tank.npz", tank)
    _nn_case("nn_alias.npz", alias_case())
    ab = alias_boundary_case()
    ab["h"][ab["label"] == 0] = 1.3 * 0.025
    _nn_case("nn_alias_boundary.npz", ab)
    # the reference's own linked-list test geometry: 26 x 26 points 1 apart, h = 1, scale 3
    from sph.Common import particle_dtype
    xv = np.linspace(0, 25, 26)
    gx, gy = np.meshgrid(xv, xv, indexing="ij")
    pa = np.zeros(gx.size, dtype=particle_dtype)
    pa["x"] = gx.ravel()
    pa["y"] = gy.ravel()
    pa["h"] = 1.0
    _nn_case("nn_grid26.npz", pa, scale=3.0)


def _solver_case(name, pa, height, r0, kernel, useXSPH=False, sumdens=False, h=None, steps=0,
                 integrator="pec", gamma_c=0.25, strict=True, fixed_dt=None, setup=True):
    """Run Solver.setup, one _compute (the evaluation golden) and `steps` bare
    steps dt -> predict -> _compute -> correct with damping 0."""
    from src.Solver import Solver
    from src.Methods.WCSPH import WCSPH
    from src.Kernels.CubicSpline import CubicSpline
    from src.Kernels.Gaussian import Gaussian
    from src.Integrators.PEC import PEC
    from src.Integrators.Euler import Euler
    from src.Equations.TimeStep import TimeStep
    method = WCSPH(height=height, r0=r0, rho0=1000.0, useXSPH=useXSPH, Pb=0.0, useSummationDensity=sumdens)
    from src.Kernels.Wendland import Wendland
    from src.Integrators.Verlet import Verlet
    kern = (CubicSpline(), Gaussian(), Wendland())[kernel]
    integ = {"pec": lambda: PEC(useXSPH=useXSPH, strict=strict), "euler": Euler,
             "verlet": lambda: Verlet(useXSPH)}[integrator]()
    solver = Solver(method, integ, kern, 1.0, incrementalWriteout=False, h=h, damping=0.0)
    Solver.particleArray = None
    solver.particleArray = None
    solver.addParticles(pa.copy())
    t0 = time.time()
    if setup:
        solver.setup()
    else:
        # keep the given densities (no hydrostatic initialize), but prepare h,
        # p and c the way Solver.setup does (src/Solver.py:184-196)
        solver.num_particles, solver.indexes = (len(pa), np.ones(len(pa), dtype=bool))
        solver.f_indexes = solver.particleArray["label"] == 0
        solver.fluid_count = int(np.sum(solver.f_indexes))
        fi = solver.f_indexes
        solver.particleArray["h"][fi] = h
        solver.particleArray["p"][fi] = method.compute_pressure(solver.particleArray[fi])
        solver.particleArray["c"][fi] = method.compute_speed_of_sound(solver.particleArray[fi])
    init = solver.particleArray.copy()
    out = {"init_" + k: np.array(init[k]) for k in init.dtype.names if k != "deleted"}
    solver._compute()
    ev = solver.particleArray.copy()
    out.update({"eval_" + k: np.array(ev[k]) for k in ev.dtype.names if k != "deleted"})
    # steps start again from the post-setup state
    solver.particleArray = init.copy()
    dts = []
    for s in range(steps):
        if fixed_dt is None:
            m, c, f = TimeStep().compute(solver.fluid_count, solver.particleArray[solver.f_indexes], gamma_c, 0.25)
        else:
            m, c, f = fixed_dt, 0.0, 0.0
        dts.append([m, c, f])
        solver.particleArray[solver.f_indexes] = integ.predict(m, solver.particleArray[solver.f_indexes], 0.0)
        solver._compute()
        solver.particleArray[solver.f_indexes] = integ.correct(m, solver.particleArray[solver.f_indexes], 0.0)
        st = solver.particleArray.copy()
        out.update({"step%d_%s" % (s + 1, k): np.array(st[k]) for k in st.dtype.names if k != "deleted"})
    meta = dict(height=height, r0=r0, kernel=kernel, useXSPH=int(useXSPH), sumdens=int(sumdens),
                h=-1.0 if h is None else h, steps=steps, integrator={"pec": 0, "euler": 1, "verlet": 2}[integrator],
                gamma_c=gamma_c, strict=int(strict), fixed_dt=-1.0 if fixed_dt is None else fixed_dt,
                setup=int(setup))
    _save(name, dts=np.array(dts).reshape(-1, 3), **{"meta_" + k: v for k, v in meta.items()}, **out)
    print("  %s: %.1f s" % (name, time.time() - t0))


def _new_solver_cases(tank, dx):
    _solver_case("solver_tank_wendland.npz", tank, 0.4, dx, 2, h=1.3 * dx, steps=2, gamma_c=0.3)
    _solver_case("solver_tank_verlet.npz", tank, 0.4, dx, 0, h=1.3 * dx, steps=2, integrator="verlet")


def gen_solver(ref, skip_large=False, only_large=False):
    from sph import scenarios as S
    if only_large:
        big = S.cfg_dam_break_small()
        _solver_case("solver_cfg_dam_break_small.npz", big, 2.0, 0.025, 0, h=1.3 * 0.025, steps=1, gamma_c=0.3)
        return
    dx = 0.025
    tank = S.dam_break(width=0.2, height=0.4, dx=dx, tank_width=0.8, tank_height=0.6)
    _solver_case("solver_tank_cubic.npz", tank, 0.4, dx, 0, h=1.3 * dx, steps=3, gamma_c=0.3)
    _solver_case("solver_tank_gauss.npz", tank, 0.4, dx, 1, h=1.3 * dx, steps=2, gamma_c=0.25)
    _solver_case("solver_tank_xsph.npz", tank, 0.4, dx, 0, useXSPH=True, h=1.3 * dx, steps=2, strict=False)
    _solver_case("solver_tank_sumdens.npz", tank, 0.4, dx, 0, sumdens=True, h=1.3 * dx, steps=2)
    _solver_case("solver_tank_dynh.npz", tank, 0.4, dx, 0, h=None, steps=2)
    _solver_case("solver_tank_euler.npz", tank, 0.4, dx, 0, h=1.3 * dx, steps=2, integrator="euler",
                 fixed_dt=1e-4)
    _new_solver_cases(tank, dx)
    lat = S.jittered_lattice(24, 24, 0.01, seed=3)
    _solver_case("solver_lattice_cubic.npz", lat, 0.24, 0.01, 0, h=0.013, steps=2, setup=False)
    _solver_case("solver_lattice_gauss.npz", lat, 0.24, 0.01, 1, h=0.013, steps=2, setup=False)
    al = alias_case()
    _solver_case("solver_alias.npz", al, 3.0, 0.25, 1, h=0.5, steps=1, setup=False)
    if not skip_large:
        big = S.cfg_dam_break_small()
        _solver_case("solver_cfg_dam_break_small.npz", big, 2.0, 0.025, 0, h=1.3 * 0.025, steps=1, gamma_c=0.3)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("SPH_REFERENCE", ""), help="Offshore-SPH checkout")
    ap.add_argument("--skip-large", action="store_true")
    ap.add_argument("--only", default="")
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(os.path.join(a.ref, "src")):
        sys.exit("--ref must point at an Offshore-SPH checkout")
    _install_shims()
    sys.path.insert(0, a.ref)
    gens = dict(kernels=gen_kernels, equations=gen_equations, eos=gen_eos_integrators, nn=gen_nn, extra=gen_extra, probes=gen_probes,
                newmark=gen_newmark, plain_run=gen_plain_run)
    for k, g in gens.items():
        if a.only and k not in a.only.split(","):
            continue
        g(a.ref)
    if "new_solver" in a.only.split(","):
        from sph import scenarios as S
        _new_solver_cases(S.dam_break(width=0.2, height=0.4, dx=0.025, tank_width=0.8, tank_height=0.6), 0.025)
    elif not a.only or "solver" in a.only.split(","):
        gen_solver(a.ref, a.skip_large)
    elif "large" in a.only.split(","):
        gen_solver(a.ref, only_large=True)


if __name__ == "__main__":
    main()
