"""sph_compute_static against sph_compute, through the C ABI.

sph_compute_static is for callers that cannot allocate device memory (their
GPU memory belongs to another allocator or a fixed budget, or they bind the
library through a foreign-function layer without a CUDA allocator): it keeps
its scratch in a device array the library owns instead of a caller
workspace.  Its results must equal sph_compute's, within the tolerance the
parity tests use, on two calls in a row -- the array keeps what the previous
call left, so the second call checks that the entry point resets what has to
start from zero.
"""
import ctypes as C

import numpy as np
import pytest

import sphcases as SC

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "p", "c", "h", "drho", "ax", "ay", "xsphx", "xsphy")
TOL = 1e-10


@pytest.fixture(scope="module")
def lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import _lib, build
    build.build()
    return _lib.load()


def _arr(d):
    from sph.Common import particle_dtype
    pa = np.zeros(len(d["x"]), dtype=particle_dtype)
    for k, v in d.items():
        pa[k] = v
    return pa


def _cases():
    meta, init, _, _, _ = SC.load_case("solver_tank_cubic")
    yield "tank", meta, init
    meta, init, _, _, _ = SC.load_case("solver_lattice_gauss")
    yield "lattice_gauss", meta, init
    from sph import scenarios as S
    pa = S.jittered_lattice(150, 150, 0.01, seed=7)
    d = {k: pa[k] for k in pa.dtype.names if k != "deleted"}
    meta = dict(height=1.5, r0=0.01, useXSPH=1, sumdens=0, kernel=0, integrator=0, strict=1, h=0.013,
                gamma_c=0.25, fixed_dt=-1.0)
    yield "lattice_xsph", meta, d


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_matches_workspace_entry_point(lib, precision):
    import torch
    from sph import core, state
    from sph.state import current_stream
    for name, meta, init in _cases():
        wc = core.wcsph_struct(meta["height"], meta["r0"], 1000.0, use_xsph=bool(meta["useXSPH"]),
                               use_summation_density=bool(meta["sumdens"]))
        cfg = core.config_struct(kernel=int(meta["kernel"]), precision=precision, h_fixed=meta["h"])
        pa = _arr(init)
        ref = state.DeviceParticles.from_array(pa)
        ws = state.DeviceWorkspace(ref.n)
        core.compute(ref, wc, cfg, ws)
        ws.check()
        want = ref.soa(FIELDS)
        status = torch.zeros(1, dtype=torch.int32, device="cuda")
        for call in range(2):
            dp = state.DeviceParticles.from_array(pa)
            rc = lib.sph_compute_static(C.byref(dp.cstruct()), C.byref(wc), C.byref(cfg), status.data_ptr(),
                                        current_stream())
            assert rc == 0, (name, call, lib.sph_status_string(rc))
            torch.cuda.synchronize()
            assert int(status.item()) & ~0x22 == 0, (name, call, int(status.item()))
            bad = SC.compare_state(dp.soa(FIELDS), want, FIELDS, TOL)
            assert not bad, (name, precision, call, bad)


def _clusters(limit):
    """`limit` particles in 32 jittered 32 x 32 lattice patches (dx = 0.01)
    spread over a 20 x 20 m domain: at h = 0.013 its search grid would need
    millions of cells, so the static entry point's cell cap coarsens it."""
    from sph import scenarios as S
    rng = np.random.default_rng(11)
    per = 32 * 32
    parts = []
    for c in range(limit // per):
        pa = S.jittered_lattice(32, 32, 0.01, seed=100 + c)
        ox, oy = rng.uniform(0.0, 19.6, 2)
        pa["x"] += ox
        pa["y"] += oy
        parts.append(pa)
    pa = np.concatenate(parts)
    assert len(pa) == limit
    return {k: pa[k] for k in pa.dtype.names if k != "deleted"}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_at_the_particle_limit_with_coarsened_grid(lib, precision):
    """Exactly SPH_STATIC_MAX_PARTICLES particles on a sparse domain: the
    static entry point coarsens its search grid (status bit set) and still
    matches sph_compute with the same cell capacity; a small dense case right
    after it must not carry the coarsened bit over."""
    import torch
    from sph import _lib, core, state
    from sph.state import current_stream
    init = _clusters(_lib.STATIC_MAX_PARTICLES)
    wc = core.wcsph_struct(0.32, 0.01, 1000.0)
    cfg = core.config_struct(kernel=0, precision=precision, h_fixed=0.013)
    pa = _arr(init)
    ref = state.DeviceParticles.from_array(pa)
    ws = state.DeviceWorkspace(ref.n, _lib.STATIC_MAX_CELLS)
    core.compute(ref, wc, cfg, ws)
    st_ref = ws.check(allow=_lib.STATUS_INFO)
    assert st_ref & _lib.STATUS_GRID_COARSENED
    want = ref.soa(FIELDS)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    dp = state.DeviceParticles.from_array(pa)
    rc = lib.sph_compute_static(C.byref(dp.cstruct()), C.byref(wc), C.byref(cfg), status.data_ptr(),
                                current_stream())
    assert rc == 0, lib.sph_status_string(rc)
    torch.cuda.synchronize()
    assert int(status.item()) & _lib.STATUS_GRID_COARSENED
    bad = SC.compare_state(dp.soa(FIELDS), want, FIELDS, TOL)
    assert not bad, bad
    # a dense 40 x 40 lattice next: its grid fits, so no coarsened bit
    small = _dense_small()
    dp2 = state.DeviceParticles.from_array(_arr(small))
    rc = lib.sph_compute_static(C.byref(dp2.cstruct()), C.byref(wc), C.byref(cfg), status.data_ptr(),
                                current_stream())
    assert rc == 0, lib.sph_status_string(rc)
    torch.cuda.synchronize()
    assert (int(status.item()) & _lib.STATUS_GRID_COARSENED) == 0, int(status.item())


def _dense_small():
    from sph import scenarios as S
    pa = S.jittered_lattice(40, 40, 0.01, seed=5)
    return {k: pa[k] for k in pa.dtype.names if k != "deleted"}


def test_static_rejects_too_many_particles(lib):
    from sph import _lib
    from sph.state import current_stream
    pa = _lib.Particles()
    pa.n = _lib.STATIC_MAX_PARTICLES + 1
    from sph import core
    wc = core.wcsph_struct(1.0, 0.01, 1000.0)
    cfg = core.config_struct()
    rc = lib.sph_compute_static(C.byref(pa), C.byref(wc), C.byref(cfg), None, current_stream())
    assert rc == _lib.SPH_ERR_STATIC_LIMIT
    assert b"static" in lib.sph_status_string(rc)
