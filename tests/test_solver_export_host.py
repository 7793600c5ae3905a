"""Solver.save / Solver.load on the host (src/Solver.py:497-531, 143-158):
the reference's HDF5 layout -- particleArray (the 154-byte record), dt_a,
dt_c, dt_f, settleTime, one dataset per export property stacked over the
steps, arrays gzip-compressed with the shuffle filter -- when h5py imports,
and the .npz stand-in with the same datasets otherwise."""
import numpy as np
import pytest


def _solver():
    import sph
    from sph import scenarios as S
    s = sph.Solver(sph.WCSPH(0.4, 0.025, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline(), 1.0,
                   exportProperties=["x", "y", "p"], incrementalWriteout=False)
    pa = S.dam_break(width=0.2, height=0.4, dx=0.025, tank_width=0.8, tank_height=0.6)
    s.addParticles(pa)
    rng = np.random.default_rng(0)
    s.dt_a, s.dt_c, s.dt_f = list(rng.uniform(1e-5, 2e-5, 7)), list(rng.uniform(1e-5, 2e-5, 7)), list(
        rng.uniform(1e-5, 2e-5, 7))
    s.settleTime = 3.5e-5
    s.export = {k: [np.array(s.particleArray[k]) + i for i in range(7)] for k in ("x", "y", "p")}
    return s


def test_save_load_hdf5_layout(tmp_path):
    h5py = pytest.importorskip("h5py")
    import sph
    s = _solver()
    path = str(tmp_path / "run.hdf5")
    s.save(path, printLocation=False)
    with h5py.File(path, "r") as f:
        assert set(f.keys()) >= {"particleArray", "dt_a", "dt_c", "dt_f", "settleTime", "x", "y", "p"}
        assert f["particleArray"].dtype.itemsize == 154
        assert f["x"].shape == (7, len(s.particleArray))
        assert f["x"].compression == "gzip" and f["x"].shuffle
        np.testing.assert_array_equal(f["dt_a"][:], s.dt_a)
    t = sph.Solver(sph.WCSPH(0.4, 0.025, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline())
    t.load(path)
    np.testing.assert_array_equal(t.particleArray, s.particleArray)
    assert t.dt_a == s.dt_a and t.dt_c == s.dt_c and t.dt_f == s.dt_f


def test_save_load_without_hdf5(tmp_path, monkeypatch):
    import builtins
    import sph
    real_import = builtins.__import__

    def no_h5py(name, *a, **k):
        if name == "h5py":
            raise ImportError("h5py hidden for this test")
        return real_import(name, *a, **k)
    monkeypatch.setattr(builtins, "__import__", no_h5py)
    s = _solver()
    path = str(tmp_path / "run.hdf5")
    s.save(path, printLocation=False)
    z = np.load(path + ".npz")
    assert set(z.files) >= {"particleArray", "dt_a", "dt_c", "dt_f", "settleTime", "x", "y", "p"}
    assert z["x"].shape == (7, len(s.particleArray))
    t = sph.Solver(sph.WCSPH(0.4, 0.025, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline())
    t.load(path + ".npz")
    np.testing.assert_array_equal(t.particleArray, s.particleArray)
    assert t.dt_a == s.dt_a
