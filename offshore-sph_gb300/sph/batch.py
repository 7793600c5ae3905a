"""Batched form: many independent WCSPH instances advanced together.

The reference runs one tank per ``Solver``; an ``Ensemble`` runs many -- each
with its own column, resolution, WCSPH constants (H = its column height),
fixed h = 1.3 dx and its own Courant dt -- as one particle set, with every
stage of a step one launch over all instances (``sph_batch_run``).  Steps can
be captured in a CUDA graph (``capture``), and ``autotune`` picks the cell
tile shape and the pair kernel's resident blocks by timing them on the
ensemble itself.  Instance b's results equal a single-instance run of it
(mixed form) with the cell capacity ``instance_cells(b)``.
"""
import ctypes as C
import time

import numpy as np
import torch

from . import _lib as L
from . import core
from .Common import particle_dtype
from .state import DeviceParticles, current_stream


class Ensemble:
    """cases: list of (particle_dtype array, dict with 'height' (the column
    height H) and 'dx'), e.g. ``scenarios.ensemble()``."""

    def __init__(self, cases, kernel=L.KERNEL_CUBIC, cfl_c=0.3, cfl_f=0.25, rho0=1000.0, max_cells=0,
                 device="cuda"):
        lib = L.load()
        self.n_inst = len(cases)
        if self.n_inst < 1:
            raise L.SphError("an ensemble needs at least one instance")
        sizes = [len(pa) for pa, _ in cases]
        self.offsets_np = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.n = int(self.offsets_np[-1])
        self.offsets = (C.c_int64 * (self.n_inst + 1))(*self.offsets_np.tolist())
        self.dp = DeviceParticles.from_array(np.concatenate([pa for pa, _ in cases]), device)
        self.fluid = self.dp.label == 0
        self.params = [dict(c) for _, c in cases]
        self.wc = (L.Wcsph * self.n_inst)()
        self.h = (C.c_double * self.n_inst)()
        for b, (_, c) in enumerate(cases):
            self.wc[b] = core.wcsph_struct(c["height"], c["dx"], rho0)
            self.h[b] = 1.3 * c["dx"]
        self.cfg = core.config_struct(kernel=kernel, precision="mixed", cfl_c=cfl_c, cfl_f=cfl_f)
        # hydrostatic start of every instance (WCSPH.initialize with its H and h)
        for b in range(self.n_inst):
            cb = core.config_struct(kernel=kernel, precision="mixed", h_fixed=self.h[b])
            sub = self.dp.cstruct_range(self.offsets_np[b], sizes[b])
            L.check(lib.sph_initialize(C.byref(sub), C.byref(self.wc[b]), C.byref(cb), current_stream()),
                    "sph_initialize")
        mc = int(max_cells) if max_cells and max_cells > 0 else \
            2 * int(lib.sph_default_max_cells(self.n)) + 2 * self.n_inst
        nbytes = C.c_size_t()
        L.check(lib.sph_batch_workspace_size(self.n, self.n_inst, mc, C.byref(nbytes)), "sph_batch_workspace_size")
        self.buf = torch.empty(int(nbytes.value), dtype=torch.uint8, device=device)
        self.ws = L.Workspace(ptr=self.buf.data_ptr(), bytes=int(nbytes.value), n_cap=self.n, max_cells=mc)
        self.tile_shift = -1
        self.tile_blocks = 0
        self.setup()

    # -- configuration -----------------------------------------------------
    def setup(self, tile_shift=None):
        if tile_shift is not None:
            self.tile_shift = int(tile_shift)
        L.check(L.load().sph_batch_setup(C.byref(self.ws), self.n_inst, self.offsets, self.wc, self.h,
                                         C.byref(self.cfg), self.tile_shift, current_stream()), "sph_batch_setup")

    def instance_cells(self, b):
        return int(L.load().sph_batch_instance_cells(C.byref(self.ws), self.n_inst, self.offsets, int(b)))

    def status(self):
        v = C.c_uint32()
        L.check(L.load().sph_get_status(C.byref(self.ws), C.byref(v), current_stream()), "sph_get_status")
        return int(v.value)

    def check(self, allow=L.STATUS_INFO):
        bad = self.status() & ~allow
        if bad:
            raise L.SphError("device status: " + "; ".join(L.status_names(bad)))

    # -- stepping ----------------------------------------------------------
    def run(self, nsteps, dt_hist=None):
        """nsteps steps of every instance; dt_hist: optional device float64
        tensor (nsteps, n_inst, 3)."""
        ptr = None
        if dt_hist is not None:
            assert dt_hist.dtype == torch.float64 and dt_hist.is_cuda and dt_hist.numel() >= 3 * self.n_inst * nsteps
            ptr = dt_hist.data_ptr()
        self._c = self.dp.cstruct()
        L.check(L.load().sph_batch_run(C.byref(self._c), C.byref(self.cfg), C.byref(self.ws), self.n_inst,
                                       int(nsteps), ptr, int(self.tile_blocks), current_stream()), "sph_batch_run")

    def capture(self, nsteps):
        """A CUDA graph of nsteps steps (replay with graph.replay())."""
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.run(1)  # warm-up outside the capture (first-launch work)
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(nsteps)
        return g

    # -- state -------------------------------------------------------------
    def snapshot(self):
        return self.dp._buf.clone(), self.dp.label.clone()

    def restore(self, snap):
        self.dp._buf.copy_(snap[0])
        self.dp.label.copy_(snap[1])

    def instance(self, b):
        """Particle array of instance b (a host copy)."""
        s, e = int(self.offsets_np[b]), int(self.offsets_np[b + 1])
        full = np.zeros(e - s, dtype=particle_dtype)
        host = self.dp._buf[:, s:e].cpu().numpy()
        from .Common import FLOAT_FIELDS
        for j, k in enumerate(FLOAT_FIELDS):
            full[k] = host[j]
        full["label"] = self.dp.label[s:e].cpu().numpy()
        return full

    def fluid_count(self):
        return int(self.fluid.sum().item())

    # -- autotuning --------------------------------------------------------
    def autotune(self, shifts=(3, 4), blocks=(2, 3), steps=5, warmup=2):
        """Times every (tile shift, resident tile-kernel blocks per SM) pair
        on this ensemble from the current state (restored afterwards) and
        keeps the fastest.  Returns {(shift, blocks): ms per step}."""
        snap = self.snapshot()
        res = {}
        for ts in shifts:
            self.setup(ts)
            for tb in blocks:
                self.tile_blocks = tb
                self.restore(snap)
                self.run(warmup)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                self.run(steps)
                e1.record()
                torch.cuda.synchronize()
                res[(ts, tb)] = e0.elapsed_time(e1) / steps
        best = min(res, key=res.get)
        self.restore(snap)
        self.setup(best[0])
        self.tile_blocks = best[1]
        self.check()
        return res
