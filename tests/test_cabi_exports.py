"""The C ABI library loads and exports every function include/*.h declares.
Host-only calls (no GPU needed): version, workspace sizing, status strings,
argument validation."""
import ctypes as C
import glob
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?(?:int|int64_t|void|char|size_t)\s*\*?\s*(sph_\w+)\s*\(", text,
                             re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from sph import _lib, build
    build.build()
    return _lib.load()


def test_header_declares_functions():
    names = declared_functions()
    assert "sph_compute" in names and "sph_run" in names and len(names) >= 15


def test_every_declared_function_is_exported(lib):
    from sph import _lib
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(declared_functions()) == set(_lib.EXPORTS)


def test_host_only_calls(lib):
    assert lib.sph_abi_version() == 1
    nbytes = C.c_size_t()
    assert lib.sph_workspace_size(1000, 0, C.byref(nbytes)) == 0
    assert nbytes.value > 1000 * 100
    assert lib.sph_workspace_size(-1, 0, C.byref(nbytes)) != 0
    assert lib.sph_default_max_cells(10) == 65536
    assert lib.sph_status_string(0) == b"ok"
    assert b"non-finite" in lib.sph_status_bit_string(4)
    assert b"coarsened" in lib.sph_status_bit_string(2)
    assert b"staging" in lib.sph_status_bit_string(64)
    assert b"workspace" in lib.sph_status_string(2)


def test_invalid_arguments_rejected_on_host(lib):
    from sph import _lib, core
    wc = core.wcsph_struct(1.0, 0.01, 1000.0)
    cfg = core.config_struct()
    bad = core.config_struct()
    bad.kernel = 7
    pa = _lib.Particles()
    pa.n = 10  # null arrays
    ws = _lib.Workspace()
    assert lib.sph_compute(C.byref(pa), C.byref(wc), C.byref(cfg), C.byref(ws), None) == 1  # invalid argument
    assert lib.sph_run(None, C.byref(wc), C.byref(cfg), C.byref(ws), 1, None, None) != 0
    assert lib.sph_compute(C.byref(pa), C.byref(wc), C.byref(bad), C.byref(ws), None) == 1


def test_empty_inputs_return_before_any_device_work(lib):
    """n = 0 (no active particles, or an empty map) is valid and returns ok
    from the argument checks, before anything touches the device; a negative
    size, an unknown kernel or too small a workspace is refused."""
    from sph import _lib, core
    wc = core.wcsph_struct(1.0, 0.01, 1000.0)
    cfg = core.config_struct()
    empty = _lib.Particles()
    empty.n = 0
    nbytes = C.c_size_t()
    assert lib.sph_workspace_size(0, 0, C.byref(nbytes)) == 0
    ws = _lib.Workspace()
    ws.ptr = 256  # never dereferenced: every call below returns on the host
    ws.bytes = nbytes.value
    ws.n_cap = 0
    ws.max_cells = lib.sph_default_max_cells(0)
    dt = C.c_double(1e-4)
    stages = (C.c_double * 16)()
    assert lib.sph_initialize(C.byref(empty), C.byref(wc), C.byref(cfg), None) == 0
    assert lib.sph_eos(C.byref(empty), C.byref(wc), None) == 0
    assert lib.sph_predict(C.byref(empty), C.byref(cfg), C.byref(dt), None) == 0
    assert lib.sph_correct(C.byref(empty), C.byref(cfg), C.byref(dt), None) == 0
    assert lib.sph_nn_update(C.byref(empty), C.byref(cfg), C.byref(ws), None) == 0
    assert lib.sph_compute(C.byref(empty), C.byref(wc), C.byref(cfg), C.byref(ws), None) == 0
    assert lib.sph_run(C.byref(empty), C.byref(wc), C.byref(cfg), C.byref(ws), 5, None, None) == 0
    assert lib.sph_run_profiled(C.byref(empty), C.byref(wc), C.byref(cfg), C.byref(ws), 5, stages, None) == 0
    assert all(v == 0.0 for v in stages)
    for k in (0, 1, 2):
        assert lib.sph_kernel_eval(k, 0, None, None, None, None) == 0
        assert lib.sph_kernel_grad(k, 0, None, None, None, None, None) == 0
    assert lib.sph_gauss_deriv(0, None, None, None, None) == 0
    # refused
    assert lib.sph_kernel_eval(7, 0, None, None, None, None) == 1
    assert lib.sph_kernel_eval(0, -1, None, None, None, None) == 1
    assert lib.sph_kernel_eval(0, 3, None, None, None, None) == 1
    assert lib.sph_run(C.byref(empty), C.byref(wc), C.byref(cfg), C.byref(ws), -1, None, None) == 1
    small = _lib.Workspace()  # bytes below the layout of its own capacity
    small.ptr, small.bytes, small.n_cap, small.max_cells = 256, 16, 0, 65536
    assert lib.sph_compute(C.byref(empty), C.byref(wc), C.byref(cfg), C.byref(small), None) != 0


def test_newmark_arguments_checked_on_host(lib):
    from sph import _lib
    nbytes = C.c_size_t()
    assert lib.sph_newmark_work_size(40, 2, 2, C.byref(nbytes)) == 0
    assert nbytes.value >= 40 * 7 * 8 + 40 * 8 + 40 * 4
    assert lib.sph_newmark_work_size(40, 40, 0, C.byref(nbytes)) == 1  # band wider than the matrix
    assert lib.sph_newmark_work_size(-1, 0, 0, C.byref(nbytes)) == 1
    pa = _lib.Particles()
    pa.n = 10  # null arrays
    assert lib.sph_newmark_predict(C.byref(pa), 0.25, 0.5, None, None) == 1
    assert lib.sph_newmark_correct(None, 0.25, 0.5, None, None) == 1
    # 2 beta >= gamma (src/Integrators/NewmarkBeta.py:32)
    assert lib.sph_newmark_acceleration(4, 0, 0, None, None, None, 0.1, 0.5, 1e-3, None, None, None, None, None,
                                        0, None, None) == 1
