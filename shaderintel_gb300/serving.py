"""The served form: simulations resident in HBM, step(dt, K) requests run by continuous batching.

A thin host mirror of the si_server_* entry points of include/si_cuda.h. The server thread lives in
the library: each round runs a few substeps of every resident simulation that has a queued request,
in one launch per phase, and requests that arrive meanwhile join the next round. A simulation is
admitted only if its device footprint fits the HBM budget.
"""
import ctypes

import numpy as np

from . import _lib as L
from ._lib import SIError, check
from .mpm import MPM, World


class Server:
    """Request loop over one World. Use admit() to create resident simulations, submit() to queue
    step(dt, K) on one of them, wait()/poll() for the result, retire() to free one."""

    def __init__(self, world=None, budget_bytes=150 * 10 ** 9):
        self.world = world if world is not None else World()
        self._own_world = world is None
        h = ctypes.c_void_p()
        check(L.lib().si_server_create(self.world._h, int(budget_bytes), ctypes.byref(h)))
        self._h = h
        self.budget_bytes = int(budget_bytes)

    # ---------------------------------------------------------------- admission
    def admit(self, maxParticles=262144, grid=64, size=1, origin=(0, 0, 0), gravity=(0, -9.81, 0), substeps=8,
              timeScale=1, sortEvery=4, ppcAxis=2):
        """A new resident simulation (the options of new MPM(ctx, o)); SIError 'out-of-memory' when
        its footprint does not fit what is left of the budget."""
        d = L.si_mpm_desc()
        L.lib().si_mpm_desc_default(ctypes.byref(d))
        d.max_particles = int(maxParticles)
        d.grid = int(grid)
        sz = list(size) if isinstance(size, (list, tuple)) else [size] * 3
        for a in range(3):
            d.size[a] = float(sz[a])
            d.origin[a] = float(origin[a])
            d.gravity[a] = float(gravity[a])
        d.substeps = int(round(substeps))
        d.time_scale = float(timeScale)
        d.sort_every = int(sortEvery)
        d.ppc_axis = int(ppcAxis)
        h = ctypes.c_void_p()
        check(L.lib().si_server_admit(self._h, ctypes.byref(d), ctypes.byref(h)))
        sim = MPM(self.world, _handle=h)
        sim._server = self
        return sim

    def retire(self, sim):
        """Frees a resident simulation; its queued requests end with status 'destroyed'."""
        check(L.lib().si_server_retire(self._h, sim._h))
        sim.destroyed = True
        if sim in self.world.scenes:
            self.world.scenes.remove(sim)

    # ---------------------------------------------------------------- requests
    def submit(self, sim, dt=None, K=None):
        """Queues step(dt, K) on `sim` (dt None: its current substep; K None: one frame); returns a
        ticket. The request carries the simulation's collider table as step() would upload it, so
        requests queued on one simulation each run with the colliders they were submitted with."""
        rows = np.ascontiguousarray(sim._collider_rows(float(dt) if dt else 0.0), np.float32)
        t = ctypes.c_uint64()
        k = int(K) if K else sim.substeps
        check(L.lib().si_server_submit_colliders(self._h, sim._h, float(dt) if dt else 0.0, k,
                                                 rows.ctypes.data_as(ctypes.c_void_p) if len(rows) else None,
                                                 len(rows), ctypes.byref(t)))
        return t.value

    def poll(self, ticket):
        """(done, status): status 0 when the request ran, else the SI_* code it ended with."""
        done, st = ctypes.c_int32(), ctypes.c_int32()
        check(L.lib().si_server_poll(self._h, ctypes.c_uint64(ticket), ctypes.byref(done), ctypes.byref(st)))
        return bool(done.value), st.value

    def wait(self, ticket, timeout_ms=-1):
        """Blocks until the ticket's substeps have finished on the device; returns its status."""
        st = ctypes.c_int32()
        check(L.lib().si_server_wait(self._h, ctypes.c_uint64(ticket), int(timeout_ms), ctypes.byref(st)))
        return st.value

    def stats(self, reset=False):
        s = L.si_server_stats()
        check(L.lib().si_server_stats_get(self._h, ctypes.byref(s), 1 if reset else 0))
        return {k: getattr(s, k) for k, _ in L.si_server_stats._fields_}

    # ---------------------------------------------------------------- lifetime
    def destroy(self):
        """Stops the loop (requests already on the device finish; queued ones are cancelled)."""
        if self._h:
            check(L.lib().si_server_destroy(self._h))
            self._h = None
            if self._own_world:
                self.world.destroy()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()


__all__ = ["Server", "SIError"]
