"""Neighbour finder with the interface of src/Tools/NNLinkedList.py:21-208.

update(pA) builds the device cell table (a counting sort over cell ids
instead of linked lists); near(i, pA) and nearPos(x, y, h, pA) return the
reference's (h_ij, q, r, nbrs) for one point; neighbour_sets() returns every
particle's list at once (CSR).  The lists equal the reference's bit for bit
and in its order (stencil cells with the x shift outer and the y shift
inner, descending index inside a cell: the head-insert order of its linked
lists), including its 3x3-cell stencil truncation and its x-overflow cell
aliasing."""
import numpy as np
import torch

from .. import core, state


class NNLinkedList:
    def __init__(self, scale: float = 2.0):
        self.scale = scale
        self.shifts = np.array([-1, 0, 1], dtype=np.int64)
        self._dp = None

    def update(self, pA):
        self._dp = state.DeviceParticles.from_array(pA)
        self._cfg = core.config_struct(nn_scale=self.scale)
        self._ws = state.DeviceWorkspace(self._dp.n)
        core.nn_update(self._dp, self._cfg, self._ws)
        self._csr = None

    def neighbour_sets(self):
        if self._csr is None:
            self._csr = core.nn_export(self._dp, self._cfg, self._ws)
            self._ws.check()
        return self._csr

    def near(self, i: int, pA):
        """(h_ij, q, r, nbrs) of particle i on the table of the last update
        (NNLinkedList.py:84): nbrs from the device export, h_ij, q and r
        formed on the device from the particles' positions and h."""
        off, idx = self.neighbour_sets()
        nb = torch.as_tensor(idx[off[i]:off[i + 1]], device="cuda")
        dp = self._dp
        dx = dp.x[i] - dp.x[nb]
        dy = dp.y[i] - dp.y[nb]
        r = torch.sqrt(dx * dx + dy * dy)
        hij = 0.5 * (dp.h[i] + dp.h[nb])
        return (hij.cpu().numpy(), (r / hij).cpu().numpy(), r.cpu().numpy(),
                nb.cpu().numpy().astype(np.uint64))

    def nearPos(self, x: float, y: float, h: float, pA=None):
        """(h_ij, q, r, nbrs) of the point (x, y) with smoothing length h on
        the table of the last update (NNLinkedList.py:41-82), on the device."""
        return self.nearPos_many([x], [y], [h])[0]

    def nearPos_many(self, x, y, h):
        """nearPos for many points at once: a list of (h_ij, q, r, nbrs)."""
        off, idx, hij, q, r = core.nn_probe(self._dp, self._ws, x, y, h)
        return [(hij[off[k]:off[k + 1]], q[off[k]:off[k + 1]], r[off[k]:off[k + 1]],
                 idx[off[k]:off[k + 1]].astype(np.uint64)) for k in range(len(off) - 1)]
