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


class _StandInDataset:
    def __init__(self, data, options):
        self.data = np.asarray(data)
        self.options = options

    def __getitem__(self, idx):
        return self.data[idx]


class _StandInFile:
    """The part of h5py.File that Solver.save / Solver.load use: datasets
    kept in memory per path, with the options they were created with."""
    files = {}

    def __init__(self, path, mode):
        if mode == "w":
            _StandInFile.files[path] = {}
        self.sets = _StandInFile.files[path]

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def create_dataset(self, name, data=None, **options):
        assert name not in self.sets, name
        self.sets[name] = _StandInDataset(data, options)

    def __getitem__(self, name):
        return self.sets[name]


def test_hdf5_branch_writes_the_reference_layout(tmp_path, monkeypatch):
    """The h5py branch, run against a stand-in h5py module (neither machine
    has h5py): the datasets and filter options of src/Solver.py:518-527 --
    particleArray, dt_a, dt_c, dt_f and the export keys with shuffle + gzip,
    settleTime and the extra properties plain -- and load reading them back."""
    import sys
    import types
    import sph
    monkeypatch.setitem(sys.modules, "h5py", types.SimpleNamespace(File=_StandInFile))
    s = _solver()
    path = str(tmp_path / "run.hdf5")
    extra = {"tank_width": np.float64(0.8), "probe_x": np.linspace(0.0, 0.8, 5)}
    s.save(path, printLocation=False, extraProperties=extra)
    sets = _StandInFile.files[path]
    packed = {"particleArray", "dt_a", "dt_c", "dt_f", "x", "y", "p"}
    assert set(sets) == packed | {"settleTime", "tank_width", "probe_x"}
    for k in packed:
        assert sets[k].options == {"shuffle": True, "compression": "gzip"}, k
    for k in ("settleTime", "tank_width", "probe_x"):
        assert sets[k].options == {}, k
    assert sets["particleArray"].data.dtype.itemsize == 154
    np.testing.assert_array_equal(sets["particleArray"].data, s.particleArray)
    np.testing.assert_array_equal(sets["x"].data, np.stack(s.export["x"]))
    np.testing.assert_array_equal(sets["dt_c"].data, s.dt_c)
    assert float(sets["settleTime"].data) == s.settleTime
    np.testing.assert_array_equal(sets["probe_x"].data, extra["probe_x"])
    t = sph.Solver(sph.WCSPH(0.4, 0.025, 1000.0, False, 0.0), sph.PEC(False, True), sph.CubicSpline())
    t.load(path)
    np.testing.assert_array_equal(t.particleArray, s.particleArray)
    assert t.dt_a == s.dt_a and t.dt_c == s.dt_c and t.dt_f == s.dt_f
