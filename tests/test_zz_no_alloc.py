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
