"""Newmark-beta integrator of coupled structures (src/Integrators/NewmarkBeta.py:13-95)
on the device.

The ice-sheet coupling example drives a beam with it: Solver.run predicts and
corrects the particles labelled Coupled with it (src/Solver.py:381-382,
397-398), and the user's coupling function calls ``acceleration`` with the
nodal forces, displacements and velocities (examples/IceBreak.py:171).

predict / correct run as sph_newmark_predict / sph_newmark_correct, bit for
bit the reference's arithmetic.  ``acceleration`` solves
(M + C gamma dt + K beta dt^2) a = F - K r - C v on the device by a banded LU
(sph_newmark_acceleration); the band widths come from the nonzeros of M, K
and C, so the example's beam (pentadiagonal K, diagonal M and C) costs
O(n), and a dense system runs the same solver in O(n^3).  Like
``np.linalg.inv`` in the reference, an exactly singular system raises
``numpy.linalg.LinAlgError``.
"""
import ctypes as C

import numpy as np
import torch

from .. import _lib, core
from ..Common import ParticleType
from ..state import DeviceParticles, current_stream
from .Integrator import Integrator

_MSG = "\nNewmark-Beta integration method is only suited for solid coupling particles."


def _bandwidths(*mats):
    """(kl, ku): the widest lower and upper band holding every nonzero."""
    kl = ku = 0
    for m in mats:
        i, j = np.nonzero(m)
        if len(i):
            kl = max(kl, int((i - j).max()))
            ku = max(ku, int((j - i).max()))
    return kl, ku


def _to_band(m, kl, ku):
    """Row band storage: row i, column j at [i, j - i + kl]."""
    n = m.shape[0]
    w = kl + ku + 1
    out = np.zeros((n, w), dtype=np.float64)
    for d in range(-kl, ku + 1):
        diag = np.diagonal(m, offset=d)
        rows = np.arange(len(diag)) + (0 if d >= 0 else -d)
        out[rows, d + kl] = diag
    return out


class NewmarkBeta(Integrator):
    integrator_id = None  # not a fluid integrator of the C ABI's config

    def __init__(self, beta: float, gamma: float, M: np.ndarray, K: np.ndarray, C: np.ndarray):
        assert (beta * 2 >= gamma)
        self.beta = beta
        self.gamma = gamma
        self.M = M
        self.K = K
        self.C = C
        self._dev = None

    def isMultiStage(self) -> bool:
        return False

    # -- particle updates ---------------------------------------------------
    def _dt(self, dt):
        return torch.tensor([float(dt)], dtype=torch.float64, device="cuda")

    def device_predict(self, dp, dt_dev):
        """predict on the Coupled particles of a device state (Solver.run)."""
        _lib.check(_lib.load().sph_newmark_predict(core._P(dp), float(self.beta), float(self.gamma),
                                                   dt_dev.data_ptr(), current_stream()), "sph_newmark_predict")

    def device_correct(self, dp, dt_dev):
        """correct on the Coupled particles of a device state (Solver.run)."""
        _lib.check(_lib.load().sph_newmark_correct(core._P(dp), float(self.beta), float(self.gamma),
                                                   dt_dev.data_ptr(), current_stream()), "sph_newmark_correct")

    def _on_array(self, pA, op):
        for lab in np.asarray(pA["label"]):
            self.checkCoupling({"label": lab})
        dp = DeviceParticles.from_array(pA)
        dp.label.fill_(int(ParticleType.Coupled))  # the reference updates every particle it is given
        op(dp)
        for f in ("x", "y", "vx", "vy"):
            pA[f] = dp.fields[f].cpu().numpy()
        return pA

    def predict(self, dt: float, pA, damping: float):
        return self._on_array(pA, lambda dp: self.device_predict(dp, self._dt(dt)))

    def correct(self, dt: float, pA, damping: float):
        return self._on_array(pA, lambda dp: self.device_correct(dp, self._dt(dt)))

    # -- acceleration -------------------------------------------------------
    def _device_system(self):
        key = (id(self.M), id(self.K), id(self.C))
        if self._dev is None or self._dev[0] != key:
            M, K, Cm = (np.asarray(x, dtype=np.float64) for x in (self.M, self.K, self.C))
            n = M.shape[0]
            if M.shape != (n, n) or K.shape != (n, n) or Cm.shape != (n, n):
                raise ValueError("M, K and C must be n x n matrices of the same n")
            kl, ku = _bandwidths(M, K, Cm)
            band = torch.from_numpy(np.stack([_to_band(x, kl, ku) for x in (M, K, Cm)])).to("cuda")
            nbytes = C.c_size_t(0)
            _lib.check(_lib.load().sph_newmark_work_size(n, kl, ku, C.byref(nbytes)), "sph_newmark_work_size")
            work = torch.empty(max(int(nbytes.value), 1), dtype=torch.uint8, device="cuda")
            self._dev = (key, n, kl, ku, band, work)
        return self._dev

    def acceleration(self, dt: float, F: np.ndarray, r: np.ndarray, v: np.ndarray):
        """a = (M + C gamma dt + K beta dt^2)^-1 (F - K r - C v), an n-vector."""
        _, n, kl, ku, band, work = self._device_system()
        vec = torch.from_numpy(np.stack([np.asarray(x, dtype=np.float64).reshape(n) for x in (F, r, v)])).to("cuda")
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        _lib.check(_lib.load().sph_newmark_acceleration(
            n, kl, ku, band[0].data_ptr(), band[1].data_ptr(), band[2].data_ptr(), float(self.beta),
            float(self.gamma), float(dt), vec[0].data_ptr(), vec[1].data_ptr(), vec[2].data_ptr(), out.data_ptr(),
            work.data_ptr(), work.numel(), info.data_ptr(), current_stream()), "sph_newmark_acceleration")
        if int(info.item()) != 0:
            raise np.linalg.LinAlgError("Singular matrix")
        return out.cpu().numpy()

    def checkCoupling(self, p):
        if p["label"] != ParticleType.Coupled:
            print(_MSG)
