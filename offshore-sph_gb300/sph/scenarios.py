"""Synthetic scenario builders for the WCSPH step.

They produce ``particle_dtype`` arrays with the conventions of the reference's
examples: boundary particles carry m = rho = h = 0
(``examples/Containment.py:37-39``, ``examples/DamBreak.py:17-34``) and the
fluid column is a square lattice of spacing ``dx``.  The reference's own
lattice helper (``src/Helpers.py:7-87``) spaces points by
``range / (ceil(range/r0) - 1)``, not by ``r0``; these builders place points
exactly ``dx`` apart instead, so that the lattice sizes are the ones stated.

Workloads (all 2D):

* ``dam_break``        -- a fluid column in a tank whose floor and side walls
  are ``layers`` rows of boundary particles at ``dx/2`` spacing.
* ``jittered_lattice`` -- an all-fluid square lattice with seeded position
  jitter, random velocities and densities (no boundaries).
* ``ensemble``         -- seeded random dam breaks for the batched form.
* ``beam_layer`` / ``beam_matrices`` -- a row of Coupled particles and the
  clamped-free beam matrices of the ice-sheet coupling example, for
  ``NewmarkBeta``.
"""
import math

import numpy as np

from .Common import ParticleType, particle_dtype


def _wall_rows(xs, ys, label):
    x, y = np.meshgrid(xs, ys, indexing="ij")
    pa = np.zeros(x.size, dtype=particle_dtype)
    pa["x"] = x.ravel()
    pa["y"] = y.ravel()
    pa["label"] = label
    return pa


def dam_break(width=1.0, height=2.0, dx=0.025, tank_width=4.0, tank_height=3.0, rho0=1000.0,
              layers=2, boundary_spacing=None, side="left"):
    """Fluid column ``width x height`` at lattice spacing ``dx`` (points at
    ((i+1/2) dx, (j+1/2) dx)), in a tank ``tank_width x tank_height`` with a
    floor and two side walls of ``layers`` boundary rows at ``dx/2`` spacing,
    offset (k+1/2) dx/2 outside the fluid domain.  ``side="right"`` stands the
    column against the right wall instead of the left one.

    Returns the particle array (fluid first, then floor, left, right wall).
    Fluid mass is rho0 dx^2; boundary m = rho = h = 0.
    """
    s = dx / 2.0 if boundary_spacing is None else boundary_spacing
    nfx = int(round(width / dx))
    nfy = int(round(height / dx))
    fx = (np.arange(nfx) + 0.5) * dx
    fy = (np.arange(nfy) + 0.5) * dx
    if side == "right":
        fx = tank_width - width + fx
    fluid = _wall_rows(fx, fy, ParticleType.Fluid)
    fluid["m"] = rho0 * dx * dx
    fluid["rho"] = rho0

    nbx = int(round(tank_width / s))
    nby = int(round(tank_height / s)) + layers
    offs = -(np.arange(layers) + 0.5) * s
    bx = (np.arange(nbx) + 0.5) * s
    wy = (np.arange(nby) + 0.5) * s - layers * s
    floor = _wall_rows(bx, offs, ParticleType.Boundary)
    left = _wall_rows(offs, wy, ParticleType.Boundary)
    right = _wall_rows(tank_width - offs, wy, ParticleType.Boundary)
    return np.concatenate((fluid, floor, left, right))


def jittered_lattice(nx=1000, ny=1000, dx=0.01, jitter=0.05, v_sigma=0.1, rho_rel=0.01, rho0=1000.0,
                     seed=0):
    """All-fluid lattice (i+1/2, j+1/2) dx, jittered by U(-jitter, jitter) dx per
    coordinate, velocities N(0, v_sigma) per component, densities
    rho0 (1 + U(-rho_rel, rho_rel)), mass rho0 dx^2.  Seeded with
    numpy.random.default_rng(seed), drawing jitter_x, jitter_y, vx, vy, rho
    in that order."""
    n = nx * ny
    rng = np.random.default_rng(seed)
    jx = rng.uniform(-jitter, jitter, n) * dx
    jy = rng.uniform(-jitter, jitter, n) * dx
    vx = rng.normal(0.0, v_sigma, n)
    vy = rng.normal(0.0, v_sigma, n)
    rho = rho0 * (1.0 + rng.uniform(-rho_rel, rho_rel, n))
    gx, gy = np.meshgrid((np.arange(nx) + 0.5) * dx, (np.arange(ny) + 0.5) * dx, indexing="ij")
    pa = np.zeros(n, dtype=particle_dtype)
    pa["label"] = ParticleType.Fluid
    pa["x"] = gx.ravel() + jx
    pa["y"] = gy.ravel() + jy
    pa["vx"] = vx
    pa["vy"] = vy
    pa["rho"] = rho
    pa["m"] = rho0 * dx * dx
    return pa


def ensemble(count=256, seed=1, width=(0.5, 2.0), height=(1.0, 3.0), dx=(0.02, 0.05), rho0=1000.0):
    """Seeded batch of dam breaks: per instance column width, height and dx
    drawn uniformly from the given ranges, tank 4x the width and 1.5x the
    height.  Returns a list of (particle array, dict(width, height, dx))."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(*width, count)
    h = rng.uniform(*height, count)
    d = rng.uniform(*dx, count)
    out = []
    for k in range(count):
        # keep whole lattice cells: round the column to a multiple of dx
        wk = max(1, int(round(w[k] / d[k]))) * d[k]
        hk = max(1, int(round(h[k] / d[k]))) * d[k]
        pa = dam_break(width=wk, height=hk, dx=d[k], tank_width=4.0 * wk, tank_height=1.5 * hk, rho0=rho0)
        out.append((pa, dict(width=wk, height=hk, dx=float(d[k]))))
    return out


def beam_layer(x0, x1, y, dx, mass=0.0, rho0=0.0):
    """A row of Coupled particles from x0 to x1 at height y, dx apart (the
    ice sheet of examples/IceBreak.py:76-78, one particle per beam node)."""
    n = int(round((x1 - x0) / dx)) + 1
    pa = np.zeros(n, dtype=particle_dtype)
    pa["label"] = ParticleType.Coupled
    pa["x"] = x0 + dx * np.arange(n)
    pa["y"] = y
    pa["m"] = mass
    pa["rho"] = rho0
    return pa


def beam_matrices(n, E, I, A, rho, L_n):
    """(K, M) of the coupling example's clamped-free Euler-Bernoulli beam
    (examples/IceBreak.py:80-108): K = E I / L_n^4 times the central
    fourth-difference operator, with the example's boundary rows at the
    clamped (first) and free (last two) nodes; M = rho A times the identity."""
    D = np.zeros((n, n))
    for i in range(n):
        for k, c in zip(range(-2, 3), (1.0, -4.0, 6.0, -4.0, 1.0)):
            if 0 <= i + k < n:
                D[i, i + k] = c
    D[0, 0] = 7.0
    D[n - 1, n - 1] = 2.0
    D[n - 1, n - 3] = 2.0
    D[n - 2, n - 1] = -2.0
    D[n - 2, n - 2] = 5.0
    return (E * I / L_n ** 4) * D, np.eye(n, n) * rho * A


def count_fluid(pa):
    return int(np.sum(pa["label"] == ParticleType.Fluid))


def cfg_dam_break_small():
    """3200-fluid dam break: 1.0 x 2.0 m column at dx = 0.025 in a 4 x 3 m tank."""
    return dam_break(1.0, 2.0, 0.025, 4.0, 3.0)


def cfg_dam_break_large(scale_dx=0.01):
    """2M-fluid dam break: 10 x 20 m column at dx = 0.01 in a 40 x 30 m tank."""
    return dam_break(10.0, 20.0, scale_dx, 40.0, 30.0)


def cfg_dam_break_1m(dx=0.01):
    """1M-fluid dam break: the 1:2 column of the 3200-particle case at 707 x 1414
    particles (7.07 x 14.14 m at dx = 0.01) in a tank 4x its width and 1.5x its
    height, 2 wall layers at dx/2."""
    w, h = 707 * dx, 1414 * dx
    return dam_break(w, h, dx, 4.0 * w, 1.5 * h)


def cfg_adjoint(dx=0.01, width=1.0, height=2.0, tank_width=4.0, tank_height=3.0):
    """20k-fluid dam break for the differentiation form: a 1.0 x 2.0 m column
    at dx = 0.01 in the 4 x 3 m tank, standing against the RIGHT wall so that
    the right wall carries a load from the first step."""
    return dam_break(width, height, dx, tank_width, tank_height, side="right")


def isclose_int(v):
    return abs(v - round(v)) < 1e-9 and math.isfinite(v)
