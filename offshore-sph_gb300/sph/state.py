"""Device-resident particle state and workspace.

The state is the reference's ``particle_dtype`` record (``src/Common.py:26-57``)
laid out as structure-of-arrays in HBM: one FP64 tensor per field, an int8
label tensor, all of length n (the active particles, in the caller's order).
Conversion to and from the reference's numpy record array happens only at the
edges (``from_array`` / ``to_array``).
"""
import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .Common import FLOAT_FIELDS, particle_dtype


def current_stream():
    return torch.cuda.current_stream().cuda_stream


class DeviceParticles:
    """SoA device copy of a particle array's active particles."""

    def __init__(self, n, device="cuda"):
        self.n = int(n)
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise L.SphError("DeviceParticles needs a CUDA device; the WCSPH step has no CPU fallback")
        self.label = torch.zeros(self.n, dtype=torch.int8, device=self.device)
        self._buf = torch.zeros((len(FLOAT_FIELDS), max(self.n, 1)), dtype=torch.float64, device=self.device)
        self.fields = {k: self._buf[j, :self.n] for j, k in enumerate(FLOAT_FIELDS)}
        self._c = None

    def __getattr__(self, k):
        f = self.__dict__.get("fields")
        if f is not None and k in f:
            return f[k]
        raise AttributeError(k)

    @classmethod
    def from_array(cls, pa, device="cuda"):
        """Copy the particle array's fields to the device (all rows of pa)."""
        dp = cls(len(pa), device)
        dp.upload(pa)
        return dp

    def upload(self, pa, non_blocking=False):
        assert len(pa) == self.n
        host = np.empty((len(FLOAT_FIELDS), self.n), dtype=np.float64)
        for j, k in enumerate(FLOAT_FIELDS):
            host[j] = pa[k]
        self._buf[:, :self.n].copy_(torch.from_numpy(host), non_blocking=non_blocking)
        self.label.copy_(torch.from_numpy(np.ascontiguousarray(pa["label"], dtype=np.int8)))

    def upload_soa(self, soa, non_blocking=False):
        """soa: dict of numpy arrays (any subset of the fields, plus 'label')."""
        for k, v in soa.items():
            t = self.label if k == "label" else self.fields[k]
            t.copy_(torch.as_tensor(np.ascontiguousarray(v)), non_blocking=non_blocking)

    def to_array(self, out=None):
        """Copy back into a particle_dtype array (new, or `out`)."""
        if out is None:
            out = np.zeros(self.n, dtype=particle_dtype)
        host = self._buf[:, :self.n].cpu().numpy()
        for j, k in enumerate(FLOAT_FIELDS):
            out[k] = host[j]
        out["label"] = self.label.cpu().numpy()
        return out

    def soa(self, fields=None):
        fields = fields or FLOAT_FIELDS
        d = {k: self.fields[k].cpu().numpy() for k in fields}
        d["label"] = self.label.cpu().numpy()
        return d

    def cstruct(self):
        s = L.Particles()
        s.n = self.n
        s.label = self.label.data_ptr()
        for k in FLOAT_FIELDS:
            setattr(s, k, self.fields[k].data_ptr())
        self._c = s
        return s

    def cstruct_range(self, off, n):
        """sph_particles_t of the particles [off, off + n)."""
        s = L.Particles()
        s.n = int(n)
        s.label = self.label.data_ptr() + int(off)
        for k in FLOAT_FIELDS:
            setattr(s, k, self.fields[k].data_ptr() + 8 * int(off))
        return s


class DeviceWorkspace:
    """Scratch of the neighbour build and pair kernels (sph_workspace_t)."""

    def __init__(self, n_cap, max_cells=0, device="cuda"):
        lib = L.load()
        self.n_cap = int(n_cap)
        mc = int(max_cells) if max_cells and max_cells > 0 else int(lib.sph_default_max_cells(self.n_cap))
        nbytes = C.c_size_t()
        L.check(lib.sph_workspace_size(self.n_cap, mc, C.byref(nbytes)), "sph_workspace_size")
        self.buf = torch.empty(int(nbytes.value), dtype=torch.uint8, device=device)
        self.ws = L.Workspace(ptr=self.buf.data_ptr(), bytes=int(nbytes.value), n_cap=self.n_cap, max_cells=mc)
        L.check(lib.sph_workspace_init(C.byref(self.ws), current_stream()), "sph_workspace_init")

    @property
    def max_cells(self):
        return self.ws.max_cells

    def status(self):
        v = C.c_uint32()
        L.check(L.load().sph_get_status(C.byref(self.ws), C.byref(v), current_stream()), "sph_get_status")
        return int(v.value)

    def check(self, allow=L.STATUS_INFO):
        """Raise if the device status word has an error bit set (clears it)."""
        st = self.status()
        bad = st & ~allow
        if bad:
            raise L.SphError("device status: " + "; ".join(L.status_names(bad)))
        return st
