"""Shared helpers for the parity tests: golden-case loading, oracle drivers,
error norms."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

STATE_FIELDS = ("m", "rho", "p", "c", "drho", "h", "x", "y", "vx", "vy", "ax", "ay",
                "xsphx", "xsphy", "x0", "y0", "vx0", "vy0", "rho0")

SOLVER_CASES = ["solver_tank_cubic", "solver_tank_gauss", "solver_tank_xsph", "solver_tank_sumdens",
                "solver_tank_dynh", "solver_tank_euler", "solver_lattice_cubic", "solver_lattice_gauss",
                "solver_alias", "solver_tank_wendland", "solver_tank_verlet"]


def load(name):
    return np.load(os.path.join(GOLDEN, name if name.endswith(".npz") else name + ".npz"))


def load_case(name):
    z = load(name)
    meta = {k[5:]: z[k].item() for k in z.files if k.startswith("meta_")}
    init = {k: z["init_" + k] for k in STATE_FIELDS + ("label",)}
    ev = {k: z["eval_" + k] for k in STATE_FIELDS + ("label",)}
    steps = []
    for s in range(int(meta["steps"])):
        steps.append({k: z["step%d_%s" % (s + 1, k)] for k in STATE_FIELDS + ("label",)})
    return meta, init, ev, steps, z["dts"]


def rel_err(a, b):
    """Norm-wise relative error ||a - b|| / ||b|| (absolute when ||b|| == 0)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(a - b)
    n = np.linalg.norm(b)
    return d / n if n > 0 else d


def oracle_params(meta):
    import oracle
    return oracle.wcsph_params(meta["height"], meta["r0"], 1000.0, use_xsph=bool(meta["useXSPH"]),
                               use_summation_density=bool(meta["sumdens"]), kernel=int(meta["kernel"]))


def oracle_eval(meta, init, nthreads=1):
    import oracle
    P = oracle.Particles(arrays=init)
    nn = oracle.NN(2.0)
    h_fixed = meta["h"] if meta["h"] > 0 else 0.0
    st = oracle.compute(oracle_params(meta), nn, P, h_fixed, nthreads)
    return P, st


def oracle_steps(meta, init, nsteps, nthreads=1):
    import oracle
    P = oracle.Particles(arrays=init)
    nn = oracle.NN(2.0)
    h_fixed = meta["h"] if meta["h"] > 0 else 0.0
    dts = oracle.run(oracle_params(meta), nn, P, nsteps, h_fixed=h_fixed,
                     dt_fixed=meta["fixed_dt"] if meta["fixed_dt"] > 0 else 0.0,
                     gamma_c=meta["gamma_c"], gamma_f=0.25, damping=0.0, integrator=int(meta["integrator"]),
                     pec_use_xsph=bool(meta["useXSPH"]), pec_strict=bool(meta["strict"]), nthreads=nthreads)
    return P, dts


def compare_state(got, want, fields, tol):
    """Return {field: rel_err} for fields whose error exceeds tol."""
    bad = {}
    for k in fields:
        if isinstance(got, dict) or (isinstance(got, np.ndarray) and got.dtype.names):
            g = got[k]
        else:
            g = getattr(got, k)
        e = rel_err(g, want[k])
        if not (e <= tol):
            bad[k] = e
    return bad


# ---------------------------------------------------------------------------
# Beam coupling case (NewmarkBeta, Solver.run with a coupling function)
# ---------------------------------------------------------------------------
BEAM = dict(dx=0.025, E=2.0e6, thick=0.02, rho_ice=917.0, g=9.81, tip=5.0, xi=0.5)


def beam_case(S):
    """The small tank with a row of Coupled particles just above the water
    (S: sph.scenarios); returns (particles, couplingProperties, (M, K, C))."""
    b = BEAM
    dx = b["dx"]
    tank = S.dam_break(width=0.2, height=0.4, dx=dx, tank_width=0.8, tank_height=0.6)
    y0 = 0.4 - dx / 2 + 0.9 * dx
    beam = S.beam_layer(0.0125, 0.3125, y0, dx)
    n = len(beam)
    L_n = dx
    A = b["thick"] * 1.0
    I = b["thick"] ** 3 / 12.0
    K, M = S.beam_matrices(n, b["E"], I, A, b["rho_ice"], L_n)
    C = np.eye(n) * 2 * b["xi"] * np.sqrt(b["rho_ice"] * A * 1000.0 * b["g"])
    P = dict(y0=y0, m=b["rho_ice"] * A, g=b["g"], tip=b["tip"], L_n=L_n)
    return np.concatenate((tank, beam)), P, (M, K, C)


def beam_coupling(pA, solver):
    """A coupling function in the style of the ice-sheet example's model 0
    (examples/IceBreak.py:110-178): beam weight on every node, a static tip
    load on the last, Newmark-beta accelerations into ay."""
    P = solver.couplingProperties
    c = pA["label"] == 3
    w = pA["y"][c] - P["y0"]
    wdot = pA["vy"][c]
    F = np.full(len(w), -P["m"] * P["g"])
    F[-1] = F[-1] + P["tip"] / P["L_n"]
    a = solver.couplingIntegrator.acceleration(solver.dt, F, w, wdot)
    pA["ay"][c] = a
    return pA


BEAM_RUN = dict(duration=1.5e-3, maxSettle=2)


def settle_now(pA, solver):
    """customSettle: end the settling at the first check (the reference's
    kinetic-energy check, src/Solver.py:416, passes the total particle count
    as the loop length over the fluid-only array, which plain Python rejects
    when boundaries exist)."""
    return True


# ---------------------------------------------------------------------------
# Plain Solver.run case: the small tank with a temporary wall that the end of
# settling removes (the dam-break example's gate, examples/DamBreak.py:31)
# ---------------------------------------------------------------------------
PLAIN_RUN = dict(dx=0.025, duration=0.02, settle_steps=3, export_every=50)  # exports kept: every 50th step


def plain_run_case(S):
    """(particles, dx) of the plain run: the small tank plus 12 TempBoundary
    particles just right of the column."""
    dx = PLAIN_RUN["dx"]
    tank = S.dam_break(width=0.2, height=0.4, dx=dx, tank_width=0.8, tank_height=0.6)
    gate = np.zeros(12, dtype=tank.dtype)
    gate["label"] = 2
    gate["x"] = 0.21 + 0.0125
    gate["y"] = (np.arange(12) + 0.5) * 0.0125 * 2
    return np.concatenate((tank, gate)), dx


def settle_after_three(pA, solver):
    """customSettle: end the settling once three steps have run."""
    return len(solver.dt_a) >= PLAIN_RUN["settle_steps"]

