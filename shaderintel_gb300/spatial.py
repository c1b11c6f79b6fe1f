"""SpatialGrid — uniform-grid neighbour binning by counting sort (src/prims/grid.js) over libsi_cuda.

The host mirror of the si_spatial_* entry points: build() sorts points into cells on the GPU (the
same stable radix sort as the MPM block sort), read() returns `order` (point indices by cell) and
`start` (first sorted slot of each cell, numCells + 1 entries), gather() permutes an attribute into
cell order, neighbors() lists the 27-cell ranges the reference's WGSL snippet visits.
"""
import ctypes
import math

import numpy as np

from . import _lib as L
from ._lib import check, dptr, fptr
from .mpm import MPM, World


class SpatialGrid:
    def __init__(self, maxCount, min, max, cellSize, world=None):   # noqa: A002 - the reference's names
        self.world = world if world is not None else World()
        self._own = world is None
        h = ctypes.c_void_p()
        check(L.lib().si_spatial_create(self.world._h, int(maxCount), dptr(min), dptr(max), float(cellSize),
                                        ctypes.byref(h)))
        self._h = h
        d = (ctypes.c_int32 * 3)()
        cells = ctypes.c_int64()
        check(L.lib().si_spatial_info(self._h, d, ctypes.byref(cells), None))
        self.maxCount = int(maxCount)
        self.cellSize = float(cellSize)
        self.origin = [float(x) for x in min]
        self.dims = list(d)
        self.numCells = cells.value
        self.count = 0

    def build(self, pos, count=None):
        """Sort points into cells: `pos` is an (n, 3) or (n, 4) array of positions, or an MPM whose
        current particle positions (lattice units) are binned in place."""
        if isinstance(pos, MPM):
            check(L.lib().si_spatial_build_mpm(self._h, pos._h))
            self.count = pos.count
            return self
        p = np.asarray(pos, np.float32)
        p = p.reshape(-1, p.shape[-1]) if p.ndim > 1 else p.reshape(-1, 4)
        n = len(p) if count is None else int(count)
        v4 = np.zeros((n, 4), np.float32)
        v4[:, :min(4, p.shape[1])] = p[:n, :4]
        check(L.lib().si_spatial_build(self._h, fptr(v4), n))
        self.count = n
        return self

    def read(self):
        """(order, start) of the last build."""
        order = np.empty(self.count, np.uint32)
        start = np.empty(self.numCells + 1, np.uint32)
        check(L.lib().si_spatial_read(self._h, order.ctypes.data_as(L.c_uint32_p), start.ctypes.data_as(L.c_uint32_p)))
        return order, start

    def gather(self, src):
        """dst[k] = src[order[k]] for an attribute array of `count` rows (float32)."""
        s = np.ascontiguousarray(src, np.float32)
        width = int(np.prod(s.shape[1:])) if s.ndim > 1 else 1
        dst = np.empty_like(s)
        check(L.lib().si_spatial_gather(self._h, fptr(s), fptr(dst), width))
        return dst

    def cell_of(self, p):
        """gridCoord of grid.js:14-16 for one position, in f32 like the kernel."""
        f = np.float32
        inv = f(1.0 / self.cellSize)
        return [int(min(max(math.floor(f(f(p[a]) - f(self.origin[a])) * inv), 0), self.dims[a] - 1)) for a in range(3)]

    def neighbors(self, p, start):
        """The sorted-slot ranges [a, b) of the 27 cells around `p`, as SpatialGrid.neighbors
        (grid.js:97-116) visits them: one range per (y, z) row covering x - 1 .. x + 1."""
        c = self.cell_of(p)
        d = self.dims
        x0, x1 = max(c[0] - 1, 0), min(c[0] + 1, d[0] - 1)
        out = []
        for z in range(max(c[2] - 1, 0), min(c[2] + 1, d[2] - 1) + 1):
            for y in range(max(c[1] - 1, 0), min(c[1] + 1, d[1] - 1) + 1):
                row = d[0] * (y + d[1] * z)
                out.append((int(start[row + x0]), int(start[row + x1 + 1])))
        return out

    def destroy(self):
        if self._h:
            check(L.lib().si_spatial_destroy(self._h))
            self._h = None
            if self._own:
                self.world.destroy()
