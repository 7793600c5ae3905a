"""Drop-in Solver (src/Solver.py:26-531) for the GB300 WCSPH step.

Same constructor, attributes and methods as the reference's Solver; the
particle state lives on the GPU between calls and every stage of the step
(TimeStep, predict, neighbour build, EOS, continuity, momentum, boundary
force, XSPH, correct) runs in libsph_gb300.  Extra keyword arguments:
``precision`` ("fp64", the reference's arithmetic, or "mixed", FP32 pair
arithmetic over FP64 state) and ``device``.

run() follows the reference's loop (Solver.py:346-475): a settling phase with
damping until the kinetic energy drops below kE times its initial value (or
maxSettle steps, or customSettle), then the temporary boundary is removed,
damping switches off and time advances.  Without a coupling function every
step is one device call of the step body (dt -> predict -> _compute ->
correct, sph_run).  Once settled, steps run in chunks with one host
synchronisation per chunk: the dt history and the export properties of every
step stay on the device until the chunk ends and come down together.  A
chunk that would pass the end of the run is rolled back to a device snapshot
and re-run to the exact step, so the steps taken are the reference's.  With
a coupling function (user Python on the host array) every step synchronises.
step(n) runs n bare steps without settling or storage.
"""
import math
import sys
from time import perf_counter

import numpy as np
import torch

from . import _lib, core, state
from .Common import FLOAT_FIELDS, ParticleType, particle_dtype
from .Tools.NNLinkedList import NNLinkedList


class Solver:
    def __init__(self, method, integrator, kernel, duration: float = 1.0, quick: bool = True,
                 incrementalWriteout: bool = True, incrementalFile: str = "export", incrementalFreq: int = 1000,
                 exportProperties=("x", "y", "p"), kE: float = 0.8, maxSettle: int = 500, timeStep: float = None,
                 h: float = None, coupling=None, couplingIntegrator=None, couplingProperties=None,
                 customSettle=None, damping: float = 0.05, precision: str = "fp64", device: str = "cuda"):
        self.method = method
        self.integrator = integrator
        self.kernel = kernel
        self.nn = NNLinkedList(scale=2.0)
        self.duration = duration
        self.quick = quick
        self.kEF = kE
        self.maxSettle = maxSettle
        self.timeStep = timeStep
        self.h = h
        self.ts_error = 0
        self.damping = damping
        self.coupling = coupling
        self.couplingIntegrator = couplingIntegrator
        self.couplingProperties = couplingProperties
        self.customSettle = customSettle
        self.incrementalWriteout = incrementalWriteout
        self.incrementalFreq = incrementalFreq
        self.incrementalFile = incrementalFile
        self.exportProperties = list(exportProperties)
        self.precision = precision
        self.device = device
        self.particleArray = None
        self.num_particles = 0
        self.data = []
        self.export = {}
        self.settleTime = 0.0
        self.dt_a, self.dt_c, self.dt_f = [], [], []
        self.timing_data = {k: 0.0 for k in ("total", "storage", "integrate_correction", "integrate_prediction",
                                             "compute", "time_step", "neighbour_hood", "coupling")}
        self._dp = None
        self._ws = None
        self._chunk_max = 64  # settled steps per host synchronisation, with per-step export fields
        self._chunk_max_bare = 256  # the same without them (one device run per chunk)

    # ------------------------------------------------------------------ state
    def addParticles(self, particles):
        """Solver.addParticles (Solver.py:160-171)."""
        if self.particleArray is None:
            self.particleArray = np.array(particles, dtype=particle_dtype)
        else:
            self.particleArray = np.concatenate((self.particleArray, np.array(particles, dtype=particle_dtype)))

    def _masks(self):
        pa = self.particleArray
        self.indexes = ~pa["deleted"]
        self.num_particles = int(np.sum(self.indexes))
        self.f_indexes = (pa["label"] == ParticleType.Fluid) & (~pa["deleted"])
        self.c_indexes = (pa["label"] == ParticleType.Coupled) & (~pa["deleted"])
        self.fluid_count = int(np.sum(self.f_indexes))

    def _upload(self):
        """Device copy of the active particles (the reference's pA[indexes])."""
        active = self.particleArray[self.indexes]
        if self._dp is None or self._dp.n != len(active):
            self._dp = state.DeviceParticles(len(active), self.device)
            self._ws = state.DeviceWorkspace(len(active), 0, self.device)
        self._dp.upload(active)

    def _download(self):
        """Bring the device state back into particleArray."""
        act = self._dp.to_array()
        full = self.particleArray
        idx = np.nonzero(self.indexes)[0]
        for k in FLOAT_FIELDS:
            full[k][idx] = act[k]

    def _cfg(self, damping=None):
        it = self.integrator
        return core.config_struct(kernel=self.kernel.kernel_id, precision=self.precision,
                                  integrator=it.integrator_id, pec_use_xsph=getattr(it, "useXSPH", False),
                                  pec_strict=getattr(it, "strict", False), nn_scale=self.nn.scale,
                                  h_fixed=self.h if self.h is not None else 0.0, cfl_c=0.25, cfl_f=0.25,
                                  damping=self.damping if damping is None else damping,
                                  dt_fixed=self.timeStep if self.timeStep is not None else 0.0)

    # ------------------------------------------------------------------ setup
    def setup(self):
        """Solver.setup (Solver.py:173-208) on the device: h for fluid (fixed
        or computeH), WCSPH.initialize, p and c for fluid, initial KE."""
        self._masks()
        self._upload()
        core.initialize(self._dp, self.method.wcsph_struct(), self._cfg())
        self.kE = self._kinetic_energy() * self.kEF
        for key in self.exportProperties:
            self.export[key] = []
        self.data = [self.particleArray.copy()]

    def _kinetic_energy(self):
        """KineticEnergy over fluid (src/Equations/KineticEnergy.py:5-12)."""
        dp = self._dp
        f = dp.label == ParticleType.Fluid
        return float((0.5 * dp.m[f] * (dp.vx[f] ** 2 + dp.vy[f] ** 2)).sum().item())

    # ------------------------------------------------------------------ steps
    def _minTimeStep(self) -> float:
        """TimeStep over fluid with gamma 0.25 / 0.25 (Solver.py:210-230)."""
        start = perf_counter()
        dt3 = core.timestep(self._dp, self.method.wcsph_struct(), self._cfg(), self._ws).cpu().numpy()
        m, c, f = float(dt3[0]), float(dt3[1]), float(dt3[2])
        if m < 1e-6:
            self.ts_error = len(self.dt_a)
        self.dt_c.append(c)
        self.dt_f.append(f)
        self.dt_a.append(m)
        self.timing_data["time_step"] += perf_counter() - start
        return m

    def _compute(self):
        """Solver._compute (Solver.py:232-256): neighbour build, h, _loop."""
        start = perf_counter()
        core.compute(self._dp, self.method.wcsph_struct(), self._cfg(), self._ws)
        torch.cuda.synchronize()
        self.timing_data["compute"] += perf_counter() - start

    def step(self, nsteps: int = 1, damping: float = 0.0):
        """nsteps bare steps on the device (dt -> predict -> _compute ->
        correct); appends the dt history."""
        hist = torch.zeros((max(nsteps, 1), 3), dtype=torch.float64, device=self.device)
        start = perf_counter()
        core.run(self._dp, self.method.wcsph_struct(), self._cfg(damping), self._ws, nsteps, hist)
        self._table_in_own_order(nsteps)
        h = hist.cpu().numpy()
        self.timing_data["compute"] += perf_counter() - start
        self._ws.check()
        for s in range(nsteps):
            self.dt_a.append(float(h[s, 0]))
            if self.timeStep is None:
                self.dt_c.append(float(h[s, 1]))
                self.dt_f.append(float(h[s, 2]))
        return h[:nsteps]

    def run(self):
        """Solver.run (Solver.py:346-475)."""
        start_all = perf_counter()
        if self.particleArray is None or len(self.particleArray) == 0 or \
                len(self.particleArray) != self.num_particles:
            raise Exception("No or invalid particles set!")
        t_step = 0
        self.t = 0.0
        self.settled = False
        dt_dev = torch.zeros(1, dtype=torch.float64, device=self.device)
        while self.t < self.duration:
            if self.coupling is None:
                t_step = self._device_steps(t_step)
                continue
            if self.timeStep is None:
                self.dt = self._minTimeStep()
            else:
                self.dt_a.append(self.timeStep)
                self.dt = self.timeStep
            dt_dev.fill_(self.dt)
            cfg = self._cfg()
            if self.integrator.isMultiStage():
                self._compute()
            start = perf_counter()
            core.predict(self._dp, cfg, dt_dev)
            if self.coupling is not None:
                self._coupled_update(dt_dev, predict=True)
            self.timing_data["integrate_prediction"] += perf_counter() - start
            self._compute()
            if self.coupling is not None:
                start = perf_counter()
                self._download()
                self.particleArray = self.coupling(self.particleArray, self)
                self._dp.upload(self.particleArray[self.indexes])
                self.timing_data["coupling"] += perf_counter() - start
            start = perf_counter()
            core.correct(self._dp, cfg, dt_dev)
            if self.coupling is not None:
                self._coupled_update(dt_dev, predict=False)
            self.timing_data["integrate_correction"] += perf_counter() - start
            start = perf_counter()
            self._store(t_step)
            self.timing_data["storage"] += perf_counter() - start
            if self.settled:
                self.t += self.dt
            t_step += 1
            if not self.settled and t_step > 1:
                ke, cs = 1e12, False
                if self.customSettle is None:
                    ke = self._kinetic_energy()
                else:
                    self._download()
                    cs = self.customSettle(self.particleArray, self)
                if (ke < self.kE) or (t_step > self.maxSettle) or cs:
                    if t_step > self.maxSettle:
                        print("\nWARNING! Maximum settle steps reached, check configuration, maybe increase "
                              "spacing between wall and particles.")
                    self._settle()
        self._download()
        self.timing_data["total"] = perf_counter() - start_all
        self.t_step = t_step

    # ------------------------------------------------------ device-side loop
    def _chunk_steps(self, t_step):
        """Steps of the next settled chunk: up to _chunk_max, ending at the
        next incremental write-out, and no more than the remaining time
        allows at the last dt (a chunk that still overshoots is rolled
        back)."""
        k = self._chunk_max if any(key in FLOAT_FIELDS for key in self.exportProperties) else self._chunk_max_bare
        if self.incrementalWriteout:
            k = min(k, self.incrementalFreq - t_step % self.incrementalFreq)
        if self.dt_a and self.dt_a[-1] > 0:
            k = min(k, max(1, int(0.9 * (self.duration - self.t) / self.dt_a[-1])))
        return max(1, k)

    def _table_in_own_order(self, nsteps):
        """A device run of four or more steps works on a copy of the state
        sorted by cell and leaves the neighbour table in that copy's order;
        the probes read the table of the last build in the solver's own
        order, so rebuild it."""
        if nsteps >= 4:
            core.nn_update(self._dp, self._cfg(), self._ws)

    def _device_steps(self, t_step):
        """One settling step, or one chunk of settled steps, of run()'s loop
        body on the device (no coupling function).  Returns the new t_step."""
        wc = self.method.wcsph_struct()
        cfg = self._cfg()
        need = [k for k in self.exportProperties if k in FLOAT_FIELDS]
        k = self._chunk_steps(t_step) if self.settled else 1
        snap = self._dp._buf.clone() if (self.settled and k > 1) else None
        taken = k
        for attempt in range(2):
            hist = torch.zeros((taken, 3), dtype=torch.float64, device=self.device)
            exp = torch.empty((taken, len(need), self._dp.n), dtype=torch.float64, device=self.device) \
                if need else None
            start = perf_counter()
            if exp is None:
                # no per-step output: the chunk is one device run (its steps
                # fused, on the sorted copy), with its dt history
                core.run(self._dp, wc, cfg, self._ws, taken, hist)
                self._table_in_own_order(taken)
            else:
                for s in range(taken):
                    core.run(self._dp, wc, cfg, self._ws, 1, hist[s])
                    for j, key in enumerate(need):
                        exp[s, j].copy_(self._dp.fields[key])
            h = hist.cpu().numpy()  # the chunk's one synchronisation
            self.timing_data["compute"] += perf_counter() - start
            self._ws.check()
            if not self.settled:
                break
            # the reference's loop takes step s only while t < duration
            t, run_steps = self.t, taken
            for s in range(taken):
                if t >= self.duration:
                    run_steps = s
                    break
                t += float(h[s, 0])
            if run_steps == taken:
                break
            self._dp._buf.copy_(snap)  # roll back, then take exactly the steps the reference takes
            taken = run_steps
        start = perf_counter()
        ex = exp.cpu().numpy() if exp is not None else None
        idx = np.nonzero(self.indexes)[0]
        for s in range(taken):
            self.dt_a.append(float(h[s, 0]))
            self.dt = float(h[s, 0])
            if self.timeStep is None:
                self.dt_c.append(float(h[s, 1]))
                self.dt_f.append(float(h[s, 2]))
                if h[s, 0] < 1e-6:
                    self.ts_error = len(self.dt_a) - 1
            for key in self.exportProperties:
                full = np.array(self.particleArray[key], copy=True)
                if key in need:
                    full[idx] = ex[s, need.index(key)]
                self.export[key].append(full)
            if self.settled:
                self.t += self.dt
            if self.incrementalWriteout and (t_step + s) % self.incrementalFreq == 0:
                self._download()
                self.data = [self.particleArray.copy()]
                self.save("{0}-{1}.hdf5".format(self.incrementalFile, t_step + s), printLocation=False)
        self.timing_data["storage"] += perf_counter() - start
        t_step += taken
        if not self.settled and t_step > 1:
            ke, cs = 1e12, False
            if self.customSettle is None:
                ke = self._kinetic_energy()
            else:
                self._download()
                cs = self.customSettle(self.particleArray, self)
            if (ke < self.kE) or (t_step > self.maxSettle) or cs:
                if t_step > self.maxSettle:
                    print("\nWARNING! Maximum settle steps reached, check configuration, maybe increase "
                          "spacing between wall and particles.")
                self._settle()
        return t_step

    def _coupled_update(self, dt_dev, predict):
        """couplingIntegrator.predict / correct of the Coupled particles
        (Solver.py:381-382, 397-398): on the device for an integrator that
        has a device path (NewmarkBeta), else on the host array."""
        ci = self.couplingIntegrator
        fn = getattr(ci, "device_predict" if predict else "device_correct", None)
        if fn is not None:
            fn(self._dp, dt_dev)
            return
        self._download()
        c = self.c_indexes
        self.particleArray[c] = (ci.predict if predict else ci.correct)(self.dt, self.particleArray[c], self.damping)
        self._upload()

    def _settle(self):
        """End of settling (Solver.py:420-451): delete TempBoundary
        particles (p = -1e15), damping off, settleTime."""
        self._download()
        pa = self.particleArray
        inds = np.nonzero((pa["label"] == ParticleType.TempBoundary) & (~pa["deleted"]))[0]
        pa["deleted"][inds] = True
        self._masks()
        pa["p"][inds] = -1e15
        self._upload()
        self.settleTime = float(sum(self.dt_a))
        self.damping = 0.0
        self.settled = True

    def _store(self, t_step: int):
        """Solver._store (Solver.py:477-486): the export properties of this
        step; the full array of the latest step in data; incremental save."""
        need = set(self.exportProperties)
        active = self._dp.soa([k for k in FLOAT_FIELDS if k in need]) if need else {}
        idx = np.nonzero(self.indexes)[0]
        for key in self.exportProperties:
            full = np.array(self.particleArray[key], copy=True)
            full[idx] = active[key] if key in active else full[idx]
            self.export[key].append(full)
        if self.incrementalWriteout and t_step % self.incrementalFreq == 0:
            self._download()
            self.data = [self.particleArray.copy()]
            self.save("{0}-{1}.hdf5".format(self.incrementalFile, t_step), printLocation=False)

    # ------------------------------------------------------------------ io
    def timing(self):
        """Timing table (Solver.py:489-495)."""
        total = self.timing_data["total"] or 1e-30
        print("\nDetailed timing statistics:")
        print("%-24s %12s %16s" % ("Name", "Time [s]", "Percentage [%]"))
        for k, v in self.timing_data.items():
            print("%-24s %12.3f %16.2f" % (k, v, v / total * 100))

    def save(self, location: str, printLocation: bool = True, extraProperties: dict = None):
        """Solver.save (Solver.py:497-531): the HDF5 layout of the reference
        (particleArray, dt_a, dt_c, dt_f and one dataset per export key,
        gzip-compressed with the shuffle filter; settleTime and the extra
        properties plain); written with h5py, or as an .npz of the same
        datasets when h5py is not installed."""
        if self._dp is not None:
            self._download()
        packed = {"particleArray": self.particleArray, "dt_a": np.asarray(self.dt_a), "dt_c": np.asarray(self.dt_c),
                  "dt_f": np.asarray(self.dt_f)}
        for key in self.exportProperties:
            if self.export.get(key):
                packed[key] = np.stack(self.export[key])
        plain = {"settleTime": np.asarray(self.settleTime)}
        if extraProperties:
            plain.update(extraProperties)
        try:
            import h5py
        except ImportError:
            h5py = None
        if h5py is not None:
            with h5py.File(location, "w") as h5f:
                for k, v in packed.items():
                    h5f.create_dataset(k, data=v, shuffle=True, compression="gzip")
                for k, v in plain.items():
                    h5f.create_dataset(k, data=v)
        else:
            data = dict(packed)
            data.update(plain)
            np.savez_compressed(location if location.endswith(".npz") else location + ".npz", **data)
        if printLocation:
            print('\nExported arrays to: "{0}".'.format(location))

    def load(self, file: str):
        """Solver.load (Solver.py:143-158): particleArray and the dt series."""
        try:
            import h5py
        except ImportError:
            h5py = None
        if h5py is not None and not file.endswith(".npz"):
            with h5py.File(file, "r") as h5f:
                self.particleArray = h5f["particleArray"][:]
                self.dt_a = list(h5f["dt_a"][:])
                self.dt_c = list(h5f["dt_c"][:])
                self.dt_f = list(h5f["dt_f"][:])
        else:
            z = np.load(file if file.endswith(".npz") else file + ".npz")
            self.particleArray = z["particleArray"]
            self.dt_a, self.dt_c, self.dt_f = list(z["dt_a"]), list(z["dt_c"]), list(z["dt_f"])
