"""Full-size cases: the 1000 x 1000 jittered lattice (cubic and Gaussian) and
the 1M-fluid dam break, checked through properties that hold at any size.

- The mixed form (FP32 pair arithmetic) against the GPU's own FP64 form on the
  same state: per-step derivatives within 1e-5, norm-wise relative per field
  (drho, ax, ay).
- Momentum of the pair forces on the cubic lattice: with one h for all
  particles and no boundaries, every pair term of Momentum.py (pressure and
  artificial viscosity) is antisymmetric in (i, j), so sum_i m_i (a_i + g e_y)
  vanishes up to rounding. Tolerance: 1e-10 (FP64) and 1e-6 (mixed) of
  sum_i m_i |a_i + g e_y|.
"""
import numpy as np
import pytest

import sphcases as SC

pytestmark = pytest.mark.gpu

G = 9.81


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build
    build.build()


def _evaluate(wl, precision):
    import torch
    import bench
    from sph import core
    dp, wc, cfg, ws = bench.prepare(wl, precision)
    core.compute(dp, wc, cfg, ws)
    ws.check()
    out = dp.soa(("m", "drho", "ax", "ay"))
    del dp, ws
    torch.cuda.empty_cache()
    return out


@pytest.mark.parametrize("name", ["lattice1m", "lattice1m_gauss", "dambreak1m"])
def test_mixed_derivatives_within_tolerance_of_fp64(lib, name):
    import bench
    wl = bench.workload(name)
    ref = _evaluate(wl, "fp64")
    got = _evaluate(wl, "mixed")
    fluid = ref["label"] == 0
    errs = {k: SC.rel_err(got[k][fluid], ref[k][fluid]) for k in ("drho", "ax", "ay")}
    assert all(e <= 1e-5 for e in errs.values()), errs
    assert np.linalg.norm(ref["ay"][fluid]) > 0


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_lattice_pair_forces_conserve_momentum(lib, precision, tol):
    import bench
    d = _evaluate(bench.workload("lattice1m"), precision)
    fx = d["m"] * d["ax"]
    fy = d["m"] * (d["ay"] + G)
    scale = np.sum(np.hypot(fx, fy))
    assert scale > 0
    resid = np.hypot(np.sum(fx), np.sum(fy))
    assert resid <= tol * scale, (resid, scale)
