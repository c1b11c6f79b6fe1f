"""MPM — the host side of ShaderIntel's MLS-MPM solver object over libsi_cuda.

Mirrors `class MPM` of src/physics/mpm.js (ShaderIntel v0.3.0) member for member: the constructor
options (mpm.js:89-127), add / clear / setColliders / step / p2g / _sort / readPositions / destroy,
the properties count, dims, dx, numNodes, substepDt, stepCount, materials and the setters
substeps / timeScale / sortEvery / gravity. Host arithmetic (material table, shape sampling,
record conversion, collider rows) runs in libsi_cuda's f64 helpers so every host builds the same
scenes; all simulation work runs in the CUDA kernels. There is no CPU path: constructing an MPM
without a GPU raises SIError('no-device').
"""
import ctypes
import json
import math

import numpy as np

from . import _lib as L
from ._lib import SIError, check, dptr, fptr

FLUID, JELLY, SNOW, SAND = 0, 1, 2, 3
MPM_KINDS = {"fluid": FLUID, "jelly": JELLY, "elastic": JELLY, "snow": SNOW, "sand": SAND}
# mpm.js:38-46
MATERIALS = {
    "water": {"kind": FLUID, "density": 1, "stiffness": 1.0, "viscosity": 0.0, "color": [0.12, 0.42, 0.95]},
    "oil": {"kind": FLUID, "density": 0.9, "stiffness": 0.9, "viscosity": 0.3, "color": [0.9, 0.62, 0.12]},
    "honey": {"kind": FLUID, "density": 1.4, "stiffness": 0.9, "viscosity": 1.0, "color": [0.95, 0.6, 0.05]},
    "jelly": {"kind": JELLY, "density": 1, "stiffness": 0.35, "poisson": 0.3, "color": [0.95, 0.3, 0.35]},
    "rubber": {"kind": JELLY, "density": 1.2, "stiffness": 0.7, "poisson": 0.45, "color": [0.25, 0.25, 0.28]},
    "snow": {"kind": SNOW, "density": 0.4, "stiffness": 0.6, "poisson": 0.2, "hardening": 10, "compression": 0.025,
             "stretch": 0.0075, "color": [0.95, 0.96, 1.0]},
    "sand": {"kind": SAND, "density": 1.6, "stiffness": 0.6, "poisson": 0.3, "friction": 33,
             "color": [0.86, 0.68, 0.42]},
}
_NAN = float("nan")


def material_row(defn, ppc_axis=2):
    """One row of the material table (mpm.js:174-195) for a material definition dict."""
    d = L.si_material_def()
    d.kind = int(defn["kind"])
    for f, key in (("density", "density"), ("stiffness", "stiffness"), ("poisson", "poisson"),
                   ("viscosity", "viscosity"), ("hardening", "hardening"), ("compression", "compression"),
                   ("stretch", "stretch"), ("friction_deg", "friction")):
        v = defn.get(key)
        setattr(d, f, _NAN if v is None else float(v))
    row = np.zeros(12, np.float32)
    check(L.lib().si_material_row(ctypes.byref(d), int(ppc_axis), fptr(row)))
    return row


def sample_shape(shape, spacing, jitter, seed):
    """sampleShape of mpm.js:683-714 (xorshift32 jitter); returns world xyz float32 (n, 3)."""
    lib = L.lib()
    if "sdf" in shape:   # an arbitrary Python SDF: same lattice and generator as the reference
        lo, hi = shape["bounds"]
        rnd = (int(seed) & 0xFFFFFFFF) or 1

        def rand():
            nonlocal rnd
            rnd ^= (rnd << 13) & 0xFFFFFFFF
            rnd ^= rnd >> 17
            rnd ^= (rnd << 5) & 0xFFFFFFFF
            return rnd / 4294967296.0
        n = [max(1, math.floor((hi[a] - lo[a]) / spacing)) for a in range(3)]
        out = []
        for z in range(n[2]):
            for y in range(n[1]):
                for x in range(n[0]):
                    p = [lo[0] + (x + 0.5 + (rand() - 0.5) * jitter) * spacing,
                         lo[1] + (y + 0.5 + (rand() - 0.5) * jitter) * spacing,
                         lo[2] + (z + 0.5 + (rand() - 0.5) * jitter) * spacing]
                    if shape["sdf"](p) <= 0:
                        out.append(p)
        return np.asarray(out, np.float32).reshape(-1, 3)
    if "box" in shape:
        kind, a, b, r, h = 0, shape["box"][0], shape["box"][1], 0.0, 0.0
    elif "sphere" in shape:
        kind, a, b, r, h = 1, shape["sphere"][0], (0, 0, 0), float(shape["sphere"][1]), 0.0
    elif "cylinder" in shape:
        c, r, h = shape["cylinder"]
        kind, a, b = 2, c, (0, 0, 0)
    else:
        raise SIError("MPM.add: shape needs box | sphere | cylinder | sdf | points", "invalid-argument")
    cnt = ctypes.c_int64()
    seed32 = (int(seed) & 0xFFFFFFFF)
    check(lib.si_sample_shape(kind, dptr(a), dptr(b), float(r), float(h), float(spacing), float(jitter), seed32,
                              None, 0, ctypes.byref(cnt)))
    out = np.empty((cnt.value, 3), np.float32)
    check(lib.si_sample_shape(kind, dptr(a), dptr(b), float(r), float(h), float(spacing), float(jitter), seed32,
                              fptr(out), cnt.value, ctypes.byref(cnt)))
    return out


SHAPES = {"sphere": 0, "box": 1, "capsule": 2}   # src/physics/rigid-wgsl.js:12


def body_record(position, size, shape="sphere", quaternion=(0, 0, 0, 1), velocity=(0, 0, 0),
                angular_velocity=(0, 0, 0), mass=0.0, friction=0.5, group=1, mask=0xFFFFFFFF, flags=0, radius=None):
    """One Body record of src/physics/rigid-wgsl.js:20-33 (48 floats, world units) for MPM.couple:
    size = sphere (r, r, r), box half extents, capsule (r, half length, r); mass 0 = static;
    radius = bounding radius (default from the shape)."""
    r = np.zeros(48, np.float32)
    sz = np.asarray(size, np.float64)
    k = SHAPES[shape] if isinstance(shape, str) else int(shape)
    if radius is None:
        radius = float(sz[0]) if k == 0 else (float(np.linalg.norm(sz)) if k == 1 else float(sz[0] + sz[1]))
    q = np.asarray(quaternion, np.float64)
    r[0:3], r[3] = position, radius
    r[4:8] = q / np.linalg.norm(q)
    r[8:11], r[11] = velocity, friction
    r[12:15] = angular_velocity
    r[32:35], r[35] = sz, k
    r[36] = mass
    r[44:48] = np.array([group, mask, flags, 0], np.uint64).astype(np.uint32).view(np.float32)
    return r


class World:
    """A CUDA stream and the simulations stepped together on it (the batched form)."""

    def __init__(self, _handle=None):
        if _handle is None:
            h = ctypes.c_void_p()
            check(L.lib().si_world_create(ctypes.byref(h)))
            _handle = h
        self._h = _handle
        self.scenes = []

    def step(self, K):
        """K substeps of every simulation in the world: one launch per phase covers them all."""
        for s in self.scenes:
            if not s.destroyed:
                s._upload_colliders()
        check(L.lib().si_world_step(self._h, int(K)))

    def sync(self):
        check(L.lib().si_world_sync(self._h))

    def set_graphs(self, on):
        check(L.lib().si_world_set_graphs(self._h, 1 if on else 0))

    def set_svd_tolerance(self, on):
        """Snow and sand decompose F to a tolerance (x, v, C, F, J within 1e-5 relative per substep of
        the bit-exact path) instead of bit for bit: faster plasticity. Off by default."""
        check(L.lib().si_world_set_svd_tolerance(self._h, 1 if on else 0))

    def profile(self, enable=True, reset=False):
        """Per-phase GPU ms {'mpm sort', 'mpm p2g', 'mpm grid', 'mpm g2p'} (labels of mpm.js:591-600)."""
        ms = (ctypes.c_double * 4)()
        check(L.lib().si_world_profile(self._h, 1 if enable else 0, ms, 1 if reset else 0))
        return dict(zip(("mpm sort", "mpm p2g", "mpm grid", "mpm g2p"), list(ms)))

    def set_tuning(self, particles_per_cta=256, tile_nodes=2048, flush=0):
        """Particles per CTA, shared tile capacity (nodes) and P2G flush strategy (0 tile, 1 global)."""
        check(L.lib().si_world_set_tuning(self._h, int(particles_per_cta), int(tile_nodes), int(flush)))

    def mark(self, slot):
        """Record timing event `slot` (0..7) on the world's stream."""
        check(L.lib().si_world_mark(self._h, int(slot)))

    def elapsed(self, a, b):
        """GPU ms between marks a and b (waits for b)."""
        ms = ctypes.c_double()
        check(L.lib().si_world_elapsed(self._h, int(a), int(b), ctypes.byref(ms)))
        return ms.value

    def launches(self):
        n = ctypes.c_int64()
        check(L.lib().si_world_launches(self._h, ctypes.byref(n)))
        return n.value

    def destroy(self):
        if self._h:
            for s in self.scenes:
                s.destroyed = True
            check(L.lib().si_world_destroy(self._h))
            self._h = None


class MPM:
    """MLS-MPM continuum simulation (water, oil, honey, jelly, rubber, snow, sand) on the GPU."""

    def __init__(self, world=None, maxParticles=262144, grid=64, size=1, origin=(0, 0, 0), gravity=(0, -9.81, 0),
                 substeps=8, timeScale=1, sortEvery=4, ppcAxis=2, _handle=None):
        lib = L.lib()
        self.world = world
        if _handle is None:
            d = L.si_mpm_desc()
            lib.si_mpm_desc_default(ctypes.byref(d))
            d.max_particles = int(maxParticles or 262144)
            d.grid = int(grid or 64)
            sz = list(size) if isinstance(size, (list, tuple)) else [size or 1] * 3
            for a in range(3):
                d.size[a] = float(sz[a])
                d.origin[a] = float(origin[a])
                d.gravity[a] = float(gravity[a])
            d.substeps = int(round(substeps or 8))
            d.time_scale = float(timeScale)
            d.sort_every = int(sortEvery or 4)
            d.ppc_axis = int(ppcAxis or 2)
            h = ctypes.c_void_p()
            check(lib.si_mpm_create(world._h if world else None, ctypes.byref(d), ctypes.byref(h)))
            self._h = h
        else:
            self._h = _handle
        if world is not None:
            world.scenes.append(self)
        self.destroyed = False
        self.materials = []
        self._material_index = {}
        self.colliders = []
        info = self._info()
        self.maxParticles = info.max_particles
        self.dx = info.dx
        self.dims = list(info.dims)
        self.size = [d * self.dx for d in self.dims]
        self.origin = list(info.origin)
        self._gravity = list(info.gravity)
        self.ppcAxis = info.ppc_axis
        self.bound = info.bound
        self.numNodes = info.num_nodes
        self.numBlocks = info.num_blocks
        self._substeps = info.substeps
        self._timeScale = info.time_scale

    # ---------------------------------------------------------------- properties
    def _info(self):
        i = L.si_mpm_info()
        check(L.lib().si_mpm_get_info(self._h, ctypes.byref(i)))
        return i

    @property
    def count(self):
        return self._info().count

    @property
    def stepCount(self):
        return self._info().step_count

    @property
    def substepDt(self):
        return self._info().substep_dt

    @property
    def substeps(self):
        return self._substeps

    @substeps.setter
    def substeps(self, n):
        self._substeps = max(1, int(round(n)))
        check(L.lib().si_mpm_set_frame(self._h, self._substeps, _NAN))

    @property
    def timeScale(self):
        return self._timeScale

    @timeScale.setter
    def timeScale(self, x):
        self._timeScale = max(1e-6, float(x))
        check(L.lib().si_mpm_set_frame(self._h, 0, self._timeScale))

    @property
    def sortEvery(self):
        return self._info().sort_every

    @sortEvery.setter
    def sortEvery(self, n):
        check(L.lib().si_mpm_set_sort_every(self._h, int(n)))

    @property
    def gravity(self):
        return list(self._gravity)

    @gravity.setter
    def gravity(self, g):
        self._gravity = [float(x) for x in g]
        check(L.lib().si_mpm_set_gravity(self._h, dptr(self._gravity)))

    # ---------------------------------------------------------------- materials (mpm.js:148-199)
    def _material(self, name_or_def):
        if isinstance(name_or_def, str):
            if name_or_def not in MATERIALS:
                raise SIError(f"MPM: unknown material {json.dumps(name_or_def)} (use {', '.join(MATERIALS)} or a "
                              "definition with a kind)", "invalid-argument")
            d = dict(MATERIALS[name_or_def], name=name_or_def)
        else:
            d = dict(name_or_def)
        if d.get("kind") is None:
            raise SIError("MPM: material definition needs a kind", "invalid-argument")
        if isinstance(d["kind"], str):
            if d["kind"] not in MPM_KINDS:
                raise SIError(f'MPM: unknown material kind "{d["kind"]}" (use {", ".join(MPM_KINDS)})',
                              "invalid-argument")
            d["kind"] = MPM_KINDS[d["kind"]]
        row = material_row(d, self.ppcAxis)   # validates kind and density like _material
        key = json.dumps(d, sort_keys=False, default=str)
        if key in self._material_index:
            return self._material_index[key]
        if len(self.materials) >= 8:
            raise SIError("MPM: at most 8 distinct materials at once (clear() frees them)", "invalid-argument")
        idx = len(self.materials)
        self.materials.append(d)
        self._material_index[key] = idx
        self._rows = getattr(self, "_rows", [])[:idx] + [row]
        table = np.stack(self._rows).astype(np.float32)
        check(L.lib().si_mpm_set_materials(self._h, fptr(table), len(self._rows)))
        return idx

    # ---------------------------------------------------------------- emission (mpm.js:207-232)
    def add(self, shape, opts=None, **kw):
        """Fill a shape with ppcAxis^3 jittered particles per cell; returns how many were added."""
        o = dict(opts or {}, **kw)
        mat = self._material(o.get("material") or shape.get("material") or "water")
        vel = o.get("velocity") or shape.get("velocity") or [0, 0, 0]
        count = self.count
        jitter, seed = o.get("jitter"), o.get("seed")
        jitter = 0.6 if jitter is None else float(jitter)
        seed = (count + 1 if seed is None else int(seed)) & 0xFFFFFFFF
        if not o.get("_host") and any(k in shape for k in ("box", "sphere", "cylinder")) and "points" not in shape:
            # sampled on the device: the same records as the host path below, bit for bit
            if "box" in shape:
                k, a, b, r, h = 0, shape["box"][0], shape["box"][1], 0.0, 0.0
            elif "sphere" in shape:
                k, a, b, r, h = 1, shape["sphere"][0], (0, 0, 0), float(shape["sphere"][1]), 0.0
            else:
                c, r, h = shape["cylinder"]
                k, a, b = 2, c, (0, 0, 0)
            added = ctypes.c_int64()
            check(L.lib().si_mpm_emit(self._h, k, dptr(a), dptr(b), float(r), float(h), jitter, seed, mat, dptr(vel),
                                      ctypes.byref(added)))
            return added.value
        if "points" in shape and shape["points"] is not None:
            pts = np.asarray(shape["points"], np.float32).reshape(-1, 3)
        else:
            pts = sample_shape(shape, self.dx / self.ppcAxis, jitter, seed)
        n = min(len(pts), self.maxParticles - count)
        if n <= 0:
            return 0
        pts = np.ascontiguousarray(pts[:n])
        rec = np.empty((n, 32), np.float32)
        check(L.lib().si_make_records(self._h, fptr(pts), n, mat, dptr(vel), 0.0, fptr(rec)))
        added = ctypes.c_int64()
        check(L.lib().si_mpm_add_particles(self._h, fptr(rec), n, ctypes.byref(added)))
        return added.value

    def addRecords(self, records):
        """Append raw particle records (32 floats each, the reference layout) up to the capacity;
        returns how many were taken (the upload half of add(), mpm.js:228-230)."""
        rec = np.ascontiguousarray(records, np.float32).reshape(-1, 32)
        added = ctypes.c_int64()
        check(L.lib().si_mpm_add_particles(self._h, fptr(rec), len(rec), ctypes.byref(added)))
        return added.value

    def clear(self):
        """Remove every particle and forget the materials (mpm.js:238-242)."""
        check(L.lib().si_mpm_clear(self._h))
        self.materials = []
        self._material_index = {}
        self._rows = []

    # ---------------------------------------------------------------- colliders (mpm.js:274-293)
    def setColliders(self, lst):
        self.colliders = list(lst)

    def _collider_rows(self, dt=0.0):
        rows = []
        for c in self.colliders[:16]:
            t = {"sphere": 0, "box": 1, "plane": 2}[c.get("type", "sphere")]
            vec = c.get("normal") if t == 2 else (c.get("half") if t == 1 else None)
            row = np.zeros(12, np.float32)
            check(L.lib().si_collider_row(self._h, t, dptr(c.get("center", [0, 0, 0])),
                                          dptr(vec) if vec is not None else None,
                                          float(c.get("radius", _NAN) if c.get("radius") is not None else _NAN),
                                          float(c.get("friction") if c.get("friction") is not None else _NAN),
                                          dptr(c.get("velocity", [0, 0, 0])), float(dt), fptr(row)))
            rows.append(row)
        return np.stack(rows) if rows else np.zeros((0, 12), np.float32)

    def _upload_colliders(self, dt=0.0):
        rows = np.ascontiguousarray(self._collider_rows(dt))
        check(L.lib().si_mpm_set_colliders(self._h, fptr(rows) if len(rows) else None, len(rows)))

    # ---------------------------------------------------------------- stepping (mpm.js:582-621)
    def step(self, dt=None, K=None):
        """One frame of `substeps` substeps (the reference's step()), or step(dt, K): K substeps of length dt."""
        if self.destroyed:
            raise SIError("MPM.step: it was destroyed", "destroyed")
        d = float(dt) if dt else 0.0
        self._upload_colliders(d)
        check(L.lib().si_mpm_step(self._h, d, int(K or 0)))

    # ---------------------------------------------------------------- rigid coupling (mpm.js:244-259)
    def couple(self, bodies, friction=0.2, band=0.5, mask=0xFFFFFFFF, densityScale=1.0):
        """Two-way coupling with rigid bodies (src/physics/coupling.js): `bodies` is an (n, 48)
        float32 array of the reference's Body records (see body_record). Empty uncouples."""
        b = np.ascontiguousarray(bodies, np.float32).reshape(-1, 48)
        check(L.lib().si_mpm_couple(self._h, fptr(b) if len(b) else None, len(b), float(friction), float(band),
                                    int(mask) & 0xFFFFFFFF, float(densityScale)))
        self._nbodies = len(b)

    def uncouple(self):
        self.couple(np.zeros((0, 48), np.float32))

    def setBodies(self, bodies):
        """New poses and velocities of the coupled bodies (the rigid world stepped)."""
        b = np.ascontiguousarray(bodies, np.float32).reshape(-1, 48)
        check(L.lib().si_mpm_set_bodies(self._h, fptr(b), len(b)))

    def readImpulses(self):
        """The bodies' reaction impulses since the last read, world units: (n, 8) float32 with
        J in [:, 0:3] and L in [:, 4:7] (coupling.finish(), mpm-rigid-apply)."""
        n = getattr(self, "_nbodies", 0)
        out = np.zeros((n, 8), np.float32)
        if n:
            check(L.lib().si_mpm_read_impulses(self._h, fptr(out), n))
        return out

    def p2g(self, forceGlobal=False):
        """Clear the grid and scatter the particles (forceGlobal: skip the shared-memory tile)."""
        check(L.lib().si_mpm_p2g(self._h, 1 if forceGlobal else 0))

    def gridUpdate(self):
        check(L.lib().si_mpm_grid_update(self._h))

    def g2p(self):
        check(L.lib().si_mpm_g2p(self._h))

    def _sort(self):
        check(L.lib().si_mpm_sort(self._h))

    # ---------------------------------------------------------------- readback
    def readPositions(self):
        n = self.count
        out = np.empty((n, 3), np.float32)
        if n:
            check(L.lib().si_mpm_read_positions(self._h, fptr(out), 0, n))
        return out

    def readPositionsAsync(self, out=None):
        """readPositions() as the reference's Promise: queues the copy behind the queued work and
        returns a handle whose wait() gives the (count, 3) array. `out` (pinned memory keeps the
        copy asynchronous) must stay alive until then."""
        n = self.count
        buf = np.empty((n, 3), np.float32) if out is None else out
        t = ctypes.c_uint64()
        check(L.lib().si_mpm_read_positions_async(self._h, fptr(buf), 0, n, ctypes.byref(t)))
        sim = self

        class _Read:
            def wait(self):
                check(L.lib().si_mpm_read_wait(sim._h, t.value))
                return buf[:n]
        return _Read()

    def deviceView(self, which="P0"):
        """Zero-copy read-only view of a device array: "P0".."P7" (the record's eight float4 streams),
        "grid", "keys", "starts". Valid until the next step, sort, add or destroy."""
        return DeviceView(self, which)

    def readInstances(self, solidsOnly=False, size=1.0, matMask=None):
        """The sphere layer's instances as a headless buffer (spheres(), mpm.js:658-679): (count, 8)
        float32 — world xyz, radius (0 = culled by the material mask), world velocity, material id
        (u32 bits). solidsOnly culls the fluid materials like spheres({solidsOnly: true})."""
        mask = (~self.fluidMask() & 0xFFFFFFFF) if solidsOnly else 0xFFFFFFFF
        if matMask is not None:
            mask = int(matMask) & 0xFFFFFFFF
        n = self.count
        out = np.empty((n, 8), np.float32)
        if n:
            check(L.lib().si_mpm_read_instances(self._h, fptr(out), 0, n, mask, float(size)))
        return out

    def readParticles(self, offset=0, n=None):
        n = self.count - offset if n is None else n
        out = np.empty((n, 32), np.float32)
        if n:
            check(L.lib().si_mpm_read_particles(self._h, fptr(out), int(offset), int(n)))
        return out

    def writeParticles(self, records, offset=0):
        rec = np.ascontiguousarray(records, np.float32).reshape(-1, 32)
        check(L.lib().si_mpm_write_particles(self._h, fptr(rec), int(offset), len(rec)))

    def readGrid(self):
        out = np.empty((self.numNodes, 4), np.int32)
        check(L.lib().si_mpm_read_grid(self._h, out.ctypes.data_as(L.c_int32_p)))
        return out

    def readBins(self, keys=True):
        """(keys, starts) of the last sort (mpm.js:122-124). A scene admitted to a server keeps no
        keys: read it with keys=False, which returns (None, starts)."""
        k = np.empty(self.count, np.uint32) if keys else None
        starts = np.empty(self.numBlocks + 1, np.uint32)
        check(L.lib().si_mpm_read_bins(self._h, k.ctypes.data_as(L.c_uint32_p) if keys else None,
                                       starts.ctypes.data_as(L.c_uint32_p)))
        return k, starts

    def sync(self):
        check(L.lib().si_mpm_sync(self._h))

    def palette(self):
        return [m.get("color", [0.7, 0.7, 0.7]) for m in self.materials]

    def fluidMask(self):
        return sum(1 << k for k, d in enumerate(self.materials) if d["kind"] == FLUID)

    @property
    def deviceBytes(self):
        return self._info().device_bytes

    def destroy(self):
        if self.destroyed:
            return
        server = getattr(self, "_server", None)
        if server is not None and server._h:
            server.retire(self)   # a resident simulation leaves through its server
            return
        self.destroyed = True
        check(L.lib().si_mpm_destroy(self._h))

    def __del__(self):
        try:
            if getattr(self, "_h", None) and L._lib is not None and self.world is None:
                L._lib.si_mpm_free(self._h)
                self._h = None
        except Exception:
            pass


class DeviceView:
    """A read-only device array of an MPM scene (si_mpm_device_ptr) with __cuda_array_interface__,
    so torch.as_tensor(view, device="cuda") or another CUDA array library wraps it without a copy."""
    _KINDS = {**{f"P{k}": (k, "<f4", 4) for k in range(8)}, "grid": (8, "<i4", 4), "keys": (9, "<u4", 1),
              "starts": (10, "<u4", 1)}

    def __init__(self, sim, which):
        k, typestr, width = self._KINDS[which]
        ptr, count, stride = ctypes.c_void_p(), ctypes.c_int64(), ctypes.c_int64()
        check(L.lib().si_mpm_device_ptr(sim._h, k, ctypes.byref(ptr), ctypes.byref(count), ctypes.byref(stride)))
        sim.sync()
        shape = (count.value, width) if width > 1 else (count.value,)
        # read-only by contract; the interface's read-only flag is left False because some consumers
        # (torch) refuse it
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr.value or 0, False),
                                         "version": 3, "strides": None}
