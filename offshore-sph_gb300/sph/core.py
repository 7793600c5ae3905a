"""Functional layer over the C ABI: parameter packing and the calls the
drop-in classes (Solver, WCSPH, PEC, ...) are built from."""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L
from .state import DeviceParticles, DeviceWorkspace, current_stream

PRECISIONS = {"fp64": L.PREC_FP64, "mixed": L.PREC_MIXED}


def wcsph_struct(height, r0, rho0, use_xsph=False, Pb=0.0, use_summation_density=False, alpha=0.01,
                 beta=0.0, epsilon=0.5, gamma=7.0, co=None, B=None, D=None, p1=4.0, p2=2.0):
    """sph_wcsph_t with WCSPH's derived constants (src/Methods/WCSPH.py:35-79,
    src/Equations/TaitEOS.py:33-44) unless given explicitly."""
    if co is None:
        co = 10.0 * math.sqrt(2 * 9.81 * height)
    if B is None:
        B = co * co * rho0 / gamma
    if D is None:
        D = 5 * 9.81 * height
    return L.Wcsph(rho0=rho0, gamma=gamma, co=co, B=B, Pb=Pb, alpha=alpha, beta=beta, epsilon=epsilon, r0=r0,
                   D=D, p1=p1, p2=p2, height=height, use_xsph=int(bool(use_xsph)),
                   use_summation_density=int(bool(use_summation_density)))


def config_struct(kernel=L.KERNEL_CUBIC, precision="fp64", integrator=L.INTEGRATOR_PEC, pec_use_xsph=False,
                  pec_strict=True, nn_scale=2.0, h_fixed=0.0, cfl_c=0.25, cfl_f=0.25, damping=0.0,
                  dt_fixed=0.0):
    if isinstance(precision, str):
        precision = PRECISIONS[precision]
    return L.Config(kernel=int(kernel), precision=int(precision), integrator=int(integrator),
                    pec_use_xsph=int(bool(pec_use_xsph)), pec_strict=int(bool(pec_strict)), nn_scale=nn_scale,
                    h_fixed=h_fixed if h_fixed else 0.0, cfl_c=cfl_c, cfl_f=cfl_f, damping=damping,
                    dt_fixed=dt_fixed if dt_fixed else 0.0)


def _P(dp):
    return C.byref(dp.cstruct())


def initialize(dp, wc, cfg):
    L.check(L.load().sph_initialize(_P(dp), C.byref(wc), C.byref(cfg), current_stream()), "sph_initialize")


def eos(dp, wc):
    L.check(L.load().sph_eos(_P(dp), C.byref(wc), current_stream()), "sph_eos")


def compute(dp, wc, cfg, ws):
    """Solver._compute on the device."""
    L.check(L.load().sph_compute(_P(dp), C.byref(wc), C.byref(cfg), C.byref(ws.ws), current_stream()),
            "sph_compute")


def run(dp, wc, cfg, ws, nsteps, dt_hist=None):
    """nsteps bare steps; dt_hist: optional device float64 tensor (nsteps, 3)."""
    ptr = None
    if dt_hist is not None:
        assert dt_hist.dtype == torch.float64 and dt_hist.is_cuda and dt_hist.numel() >= 3 * nsteps
        ptr = dt_hist.data_ptr()
    L.check(L.load().sph_run(_P(dp), C.byref(wc), C.byref(cfg), C.byref(ws.ws), int(nsteps), ptr,
                             current_stream()), "sph_run")


class StepGraph:
    """`steps` bare steps (sph_run) captured once in a CUDA graph; replay()
    advances the state by that many steps with one launch from the host.
    Capturing needs the device state and workspace to stay where they are."""

    def __init__(self, dp, wc, cfg, ws, steps):
        self.steps = int(steps)
        self._keep = (wc, cfg)  # the ctypes blocks the launches were made from
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            run(dp, wc, cfg, ws, 1)  # first-launch work outside the capture
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            run(dp, wc, cfg, ws, self.steps)

    def replay(self):
        self.graph.replay()


def run_profiled(dp, wc, cfg, ws, nsteps):
    """sph_run with CUDA-event laps per stage; returns {stage: ms summed over steps}."""
    ms = (C.c_double * len(L.STAGES))()
    L.check(L.load().sph_run_profiled(_P(dp), C.byref(wc), C.byref(cfg), C.byref(ws.ws), int(nsteps), ms,
                                      current_stream()), "sph_run_profiled")
    return {k: ms[j] for j, k in enumerate(L.STAGES)}


def timestep(dp, wc, cfg, ws, dt3=None):
    if dt3 is None:
        dt3 = torch.zeros(3, dtype=torch.float64, device=dp.device)
    L.check(L.load().sph_timestep(_P(dp), C.byref(wc), C.byref(cfg), C.byref(ws.ws), dt3.data_ptr(),
                                  current_stream()), "sph_timestep")
    return dt3


def predict(dp, cfg, dt_dev):
    L.check(L.load().sph_predict(_P(dp), C.byref(cfg), dt_dev.data_ptr(), current_stream()), "sph_predict")


def correct(dp, cfg, dt_dev):
    L.check(L.load().sph_correct(_P(dp), C.byref(cfg), dt_dev.data_ptr(), current_stream()), "sph_correct")


def nn_update(dp, cfg, ws):
    L.check(L.load().sph_nn_update(_P(dp), C.byref(cfg), C.byref(ws.ws), current_stream()), "sph_nn_update")


def nn_export(dp, cfg, ws):
    """Neighbour lists of the last nn_update: (offsets[n+1], idx) as numpy
    int64, each list in the reference's order (stencil cells x shift outer,
    y shift inner; descending index inside a cell)."""
    lib = L.load()
    counts = torch.zeros(dp.n, dtype=torch.int64, device=dp.device)
    L.check(lib.sph_nn_count(_P(dp), C.byref(cfg), C.byref(ws.ws), counts.data_ptr(), current_stream()),
            "sph_nn_count")
    offsets = torch.zeros(dp.n + 1, dtype=torch.int64, device=dp.device)
    offsets[1:] = torch.cumsum(counts, 0)
    total = int(offsets[-1].item())
    idx = torch.zeros(max(total, 1), dtype=torch.int64, device=dp.device)
    L.check(lib.sph_nn_export(_P(dp), C.byref(cfg), C.byref(ws.ws), offsets.data_ptr(), idx.data_ptr(),
                              current_stream()), "sph_nn_export")
    return offsets.cpu().numpy(), idx[:total].cpu().numpy()


def _dev(v, n=None):
    t = torch.as_tensor(v, dtype=torch.float64, device="cuda").reshape(-1).contiguous()
    if n is not None and t.numel() == 1 and n > 1:
        t = t.expand(n).contiguous()
    return t


def nn_probe(dp, ws, px, py, ph):
    """NNLinkedList.nearPos for many points on the table of the last build:
    (offsets[np+1], idx, h_ij, q, r) as numpy, each list in the reference's
    order."""
    lib = L.load()
    px = _dev(px)
    n = px.numel()
    py, ph = _dev(py, n), _dev(ph, n)
    counts = torch.zeros(n, dtype=torch.int64, device=dp.device)
    L.check(lib.sph_nn_probe_count(_P(dp), C.byref(ws.ws), n, px.data_ptr(), py.data_ptr(), ph.data_ptr(),
                                   counts.data_ptr(), current_stream()), "sph_nn_probe_count")
    offsets = torch.zeros(n + 1, dtype=torch.int64, device=dp.device)
    offsets[1:] = torch.cumsum(counts, 0)
    total = int(offsets[-1].item())
    idx = torch.zeros(max(total, 1), dtype=torch.int64, device=dp.device)
    hij, q, r = (torch.zeros(max(total, 1), dtype=torch.float64, device=dp.device) for _ in range(3))
    L.check(lib.sph_nn_probe_export(_P(dp), C.byref(ws.ws), n, px.data_ptr(), py.data_ptr(), ph.data_ptr(),
                                    offsets.data_ptr(), idx.data_ptr(), hij.data_ptr(), q.data_ptr(), r.data_ptr(),
                                    current_stream()), "sph_nn_probe_export")
    return (offsets.cpu().numpy(), idx[:total].cpu().numpy(), hij[:total].cpu().numpy(), q[:total].cpu().numpy(),
            r[:total].cpu().numpy())


def probe_density(dp, wc, kernel, ws, px, py, h_search, h_kernel):
    """Density and pressure at points (Shepard-normalised summation density +
    Tait EOS over the nearPos sets); device tensors (rho, p)."""
    px = _dev(px)
    n = px.numel()
    py, hs, hk = _dev(py, n), _dev(h_search, n), _dev(h_kernel, n)
    rho = torch.empty(n, dtype=torch.float64, device=dp.device)
    p = torch.empty(n, dtype=torch.float64, device=dp.device)
    L.check(L.load().sph_probe_density(_P(dp), C.byref(wc), int(kernel), C.byref(ws.ws), n, px.data_ptr(),
                                       py.data_ptr(), hs.data_ptr(), hk.data_ptr(), rho.data_ptr(), p.data_ptr(),
                                       current_stream()), "sph_probe_density")
    return rho, p


def block_equations(comp, p, wc):
    """The per-block equations of one particle on the device
    (sph_block_equations): comp is a computed_dtype array (host), p the
    particle (a particle_dtype record or a mapping with p, rho, h, c).
    Returns the 7 sums (continuity, momentum x, y without gravity, boundary
    force x, y, XSPH x, y) as a numpy array."""
    n = len(comp)
    arrs = {k: torch.as_tensor(np.ascontiguousarray(comp[k], dtype=np.float64), device="cuda")
            for k in L.BLOCK_ARRAYS}
    lab = torch.as_tensor(np.ascontiguousarray(comp["label"], dtype=np.int8), device="cuda")
    blk = L.Block(n=n, label=lab.data_ptr(), **{k: v.data_ptr() for k, v in arrs.items()})
    self4 = (C.c_double * 4)(float(p["p"]), float(p["rho"]), float(p["h"]), float(p["c"]))
    out = torch.zeros(7, dtype=torch.float64, device="cuda")
    L.check(L.load().sph_block_equations(C.byref(blk), self4, C.byref(wc), out.data_ptr(), current_stream()),
            "sph_block_equations")
    return out.cpu().numpy()


def kernel_eval(kernel, r, h):
    r = torch.as_tensor(r, dtype=torch.float64, device="cuda").contiguous()
    h = torch.as_tensor(h, dtype=torch.float64, device="cuda").contiguous()
    out = torch.empty_like(r)
    L.check(L.load().sph_kernel_eval(int(kernel), r.numel(), r.data_ptr(), h.data_ptr(), out.data_ptr(),
                                     current_stream()), "sph_kernel_eval")
    return out


def kernel_grad(kernel, x, r, h):
    x = torch.as_tensor(x, dtype=torch.float64, device="cuda").contiguous()
    r = torch.as_tensor(r, dtype=torch.float64, device="cuda").contiguous()
    h = torch.as_tensor(h, dtype=torch.float64, device="cuda").contiguous()
    out = torch.empty_like(r)
    L.check(L.load().sph_kernel_grad(int(kernel), r.numel(), x.data_ptr(), r.data_ptr(), h.data_ptr(),
                                     out.data_ptr(), current_stream()), "sph_kernel_grad")
    return out


def gauss_deriv(r, h):
    r = torch.as_tensor(r, dtype=torch.float64, device="cuda").contiguous()
    h = torch.as_tensor(h, dtype=torch.float64, device="cuda").contiguous()
    out = torch.empty_like(r)
    L.check(L.load().sph_gauss_deriv(r.numel(), r.data_ptr(), h.data_ptr(), out.data_ptr(), current_stream()),
            "sph_gauss_deriv")
    return out


def on_device(pA, op, fields, as_fluid=False):
    """Run op(dp) on a device copy of the particle array pA and copy the
    listed fields back into pA (the reference's functions return the array
    they were given, modified)."""
    dp = DeviceParticles.from_array(pA)
    if as_fluid:
        dp.label.zero_()
    op(dp)
    for f in fields:
        pA[f] = dp.fields[f].cpu().numpy()
    return pA
