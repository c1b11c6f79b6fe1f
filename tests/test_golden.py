"""Parity pin: the oracle, and then the CUDA path, against fixtures made by executing the
reference's own WGSL (src/physics/mpm.js, src/shaders/linalg.js) with tests/golden/wgsl_exec.py.

What the fixtures hold (tests/golden/gen_golden.py makes them, with the reference beside it):
  p2g.npz         a water + rubber scene at grid 16 with random v, C and tau; the mpm-p2g grid sums
                  (the reference's shared-tile and global paths gave the same words)
  grid.npz        that grid after mpm-grid with gravity, walls, floor friction and three colliders
  g2p.npz         water, honey, jelly, snow and sand from a deformed state: mpm-p2g, mpm-grid, mpm-g2p
  sort.npz        mpm-key + scan + mpm-reorder of a shuffled scene at grid 32
  trajectory.npz  12 substeps of step()'s schedule (sort every 4th) for water and honey
  couple.npz      the fluid <-> rigid coupling pass and apply (src/physics/coupling.js) on a pool with
                  five bodies (dynamic sphere and rotated box, static capsule, disabled, masked out)
  retime.npz      mpm-retime (mpm.js:405-413) on a deformed five-material state at k = 0.5, 2 and the
                  k of a substeps change 8 -> 6
  spatial.npz     SpatialGrid.build (src/prims/grid.js:23-96): cells, starts and order of 2,500 points,
                  some outside the box and 40 in one cell

Bar: bit-exact for keys, starts, sorted records, grid sums, the grid update and every particle
field whose computation has no log/exp. log and exp are implementation-defined in WGSL (absolute
error below 2^-21 for log on [0.5, 2], 3 + 2|x| ulp for exp); the fields that pass through them
(tau of jelly, snow and sand; F of sand) are held to 1e-5 relative plus the stress that WGSL's own
log accuracy allows, (2 mu + 3 lambda) 2^-20."""
import os

import numpy as np
import pytest

import si_oracle as O

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TAU = [11, 15, 19, 23, 27, 31]
F_COLS = [20, 21, 22, 24, 25, 26, 28, 29, 30]


def fixture(name):
    return np.load(os.path.join(HERE, name))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def check_g2p(got, want, rec, mats):
    """Asserts the G2P bar above on records `got` against the fixture's `want`."""
    kinds = mats[:, 0].view(np.uint32)
    kind = kinds[bits(rec[:, 3]) & 7]
    exact = np.ones(32, bool)
    exact[TAU] = False
    exact[F_COLS] = False
    assert np.array_equal(bits(got[:, exact]), bits(want[:, exact])), "x, v, J/Jp or C differ"
    plain = kind == 0
    assert np.array_equal(bits(got[plain]), bits(want[plain])), "a fluid record differs"
    no_log_f = kind != 3
    assert np.array_equal(bits(got[no_log_f][:, F_COLS]), bits(want[no_log_f][:, F_COLS]))
    mid = bits(rec[:, 3]) & 7
    mu, la = mats[mid, 2].astype(np.float64), mats[mid, 3].astype(np.float64)
    dtau = np.abs(got[:, TAU].astype(np.float64) - want[:, TAU]).max(1)
    bound = 1e-5 * np.abs(want[:, TAU]).max(1) + (2 * mu + 3 * la) * 2.0 ** -20
    assert np.all(dtau <= bound), f"tau off by {float((dtau / bound).max()):.3g} of its bound"
    sand = kind == 3
    if sand.any():
        dF = np.abs(got[sand][:, F_COLS].astype(np.float64) - want[sand][:, F_COLS]).max(1)
        assert np.all(dF <= 2.0 ** -19 * np.abs(want[sand][:, F_COLS]).max(1))


# ---------------------------------------------------------------------------- the oracle


def test_oracle_p2g_matches_reference_wgsl():
    d = fixture("p2g.npz")
    g = O.p2g(d["rec"], d["dims"], d["mats"], float(d["vol4"]))
    assert np.array_equal(g, d["grid"])
    assert (d["grid"][:, 3] != 0).sum() > 300


def test_oracle_grid_update_matches_reference_wgsl():
    d = fixture("grid.npz")
    g = O.grid_update(d["grid_in"], d["dims"], d["gravity"], d["cols"], int(d["ncol"]))
    assert np.array_equal(g, d["grid_out"])


def test_oracle_g2p_matches_reference_wgsl():
    d = fixture("g2p.npz")
    assert np.array_equal(O.p2g(d["rec"], d["dims"], d["mats"], float(d["vol4"])), d["grid"])
    gv = O.grid_update(d["grid"], d["dims"], d["gravity"], np.zeros((16, 12), np.float32), 0)
    assert np.array_equal(gv, d["gv"])
    got = O.g2p(d["rec"], d["dims"], d["gv"], d["mats"])
    kinds = set((d["mats"][:, 0].view(np.uint32)[bits(d["rec"][:, 3]) & 7]).tolist())
    assert kinds == {0, 1, 2, 3}
    check_g2p(got, d["out"], d["rec"], d["mats"])


def test_oracle_block_sort_matches_reference_wgsl():
    d = fixture("sort.npz")
    dst, keys, starts, _ = O.sort(d["rec"], int(d["num_blocks"]))
    assert np.array_equal(keys, d["keys"])
    assert np.array_equal(starts, d["starts"])
    assert np.array_equal(bits(dst), bits(d["sorted"]))


def test_oracle_substeps_match_reference_wgsl():
    d = fixture("trajectory.npz")
    P, _, sc = O.substeps(d["rec"], d["dims"], d["mats"], d["cols"], int(d["ncol"]), d["gravity"],
                          float(d["vol4"]), int(d["substeps"]), 0, int(d["sort_every"]))
    assert sc == int(d["substeps"])
    assert np.array_equal(bits(P), bits(d["out"]))


def test_planted_mistake_in_oracle_is_caught():
    """A one-ulp change of one particle's position must break the bit-exact trajectory check."""
    d = fixture("trajectory.npz")
    rec = d["rec"].copy()
    rec[17, 1] = np.nextafter(rec[17, 1], np.float32(100))
    P, _, _ = O.substeps(rec, d["dims"], d["mats"], d["cols"], int(d["ncol"]), d["gravity"],
                         float(d["vol4"]), int(d["substeps"]), 0, int(d["sort_every"]))
    assert not np.array_equal(bits(P), bits(d["out"]))


# ---------------------------------------------------------------------------- the CUDA path


MATS_P2G = [dict(kind=0, density=1, stiffness=1.0, viscosity=0.0),
            dict(kind=1, density=1.2, stiffness=0.7, poisson=0.45)]
MATS_G2P = [dict(kind=0, density=1, stiffness=1.0, viscosity=0.0),
            dict(kind=0, density=1.4, stiffness=0.9, viscosity=1.0),
            dict(kind=1, density=1, stiffness=0.35, poisson=0.3),
            dict(kind=2, density=0.4, stiffness=0.6, poisson=0.2, hardening=10, compression=0.025, stretch=0.0075),
            dict(kind=3, density=1.6, stiffness=0.6, poisson=0.3, friction=30)]
MATS_TRAJ = MATS_G2P[:2]
COLS_GRID = [{"type": "sphere", "center": [0.45, 0.45, 0.45], "radius": 0.12, "velocity": [0.3, 0, 0], "friction": 0.5},
             {"type": "box", "center": [0.6, 0.35, 0.5], "half": [0.08, 0.05, 0.1]},
             {"type": "plane", "center": [0, 0.3, 0], "normal": [0.1, 1, 0]}]
COLS_TRAJ = [{"type": "sphere", "center": [0.45, 0.25, 0.45], "radius": 0.1, "velocity": [0.2, 0, 0], "friction": 0.5},
             {"type": "plane", "center": [0, 0.2, 0], "normal": [0.2, 1, 0]}]


def _loaded(d, mats, grid, colliders=()):
    """An MPM holding the fixture's records, with its material table checked against the fixture's."""
    from shaderintel_gb300 import MPM
    sim = MPM(grid=grid, maxParticles=len(d["rec"]) + 64, substeps=8)
    for m in mats:
        sim._material(m)
    assert np.array_equal(bits(np.stack(sim._rows)), bits(d["mats"][:len(mats)]))
    if colliders:
        sim.setColliders(list(colliders))
        rows = sim._collider_rows()
        assert np.array_equal(bits(rows), bits(d["cols"][:len(rows)]))
    assert sim.addRecords(d["rec"]) == len(d["rec"])
    return sim


@pytest.mark.gpu
def test_cuda_p2g_and_grid_update_match_reference_wgsl():
    d, dg = fixture("p2g.npz"), fixture("grid.npz")
    sim = _loaded(d, MATS_P2G, 16)
    for force_global in (False, True):
        sim.p2g(forceGlobal=force_global)
        assert np.array_equal(sim.readGrid(), d["grid"])
    sim.setColliders(COLS_GRID)
    sim._upload_colliders()
    sim.gridUpdate()
    assert np.array_equal(sim.readGrid(), dg["grid_out"])
    sim.destroy()


@pytest.mark.gpu
def test_cuda_g2p_matches_reference_wgsl():
    d = fixture("g2p.npz")
    sim = _loaded(d, MATS_G2P, 16)
    sim.p2g()
    assert np.array_equal(sim.readGrid(), d["grid"])
    sim.gridUpdate()
    assert np.array_equal(sim.readGrid(), d["gv"])
    sim.g2p()
    check_g2p(sim.readParticles(), d["out"], d["rec"], d["mats"])
    sim.destroy()


@pytest.mark.gpu
def test_cuda_block_sort_matches_reference_wgsl():
    d = fixture("sort.npz")
    from shaderintel_gb300 import MPM
    sim = MPM(grid=32, maxParticles=len(d["rec"]), substeps=8)
    sim._material(dict(kind=0, density=1, stiffness=1.0, viscosity=0.0))
    sim.addRecords(d["rec"])
    sim._sort()
    keys, starts = sim.readBins()
    assert np.array_equal(keys, d["keys"])
    assert np.array_equal(starts, d["starts"])
    assert np.array_equal(bits(sim.readParticles()), bits(d["sorted"]))
    sim.destroy()


@pytest.mark.gpu
def test_cuda_substeps_match_reference_wgsl():
    d = fixture("trajectory.npz")
    sim = _loaded(d, MATS_TRAJ, 16, COLS_TRAJ)
    sim.step(dt=sim.substepDt, K=int(d["substeps"]))
    assert np.array_equal(bits(sim.readParticles()), bits(d["out"]))
    sim.destroy()


def test_oracle_coupling_matches_reference_wgsl():
    """mpm-rigid-couple + mpm-rigid-apply (src/physics/coupling.js:83-196) on a water pool with a
    dynamic sphere, a rotated dynamic box, a static capsule, a disabled and a masked-out body."""
    d = fixture("couple.npz")
    g, acc = O.couple(d["grid_in"], d["dims"], d["bodies"], d["params"], int(d["mask"]))
    assert np.array_equal(g, d["grid_out"])
    assert np.array_equal(acc, d["acc"])
    assert (g != d["grid_in"]).any(1).sum() > 20                   # the pass changed nodes
    nz = d["acc"].reshape(-1, 8)[:, [0, 1, 2, 4, 5, 6]].any(1)
    assert nz.tolist() == [True, True, False, False, False]        # static, disabled, masked: none
    ext, rest = O.couple_apply(acc, len(d["bodies"]), float(d["mom_to_world"]), float(d["params"][3]))
    assert np.array_equal(bits(ext), bits(d["ext"]))
    assert not rest.any()


# ---------------------------------------------------------------------------- retime (mpm.js:136-145, 405-413)


def test_oracle_retime_matches_reference_wgsl():
    d = fixture("retime.npz")
    for k, want in zip(d["ks"], d["out"]):
        got = O.retime(d["rec"], float(k))
        assert np.array_equal(bits(got), bits(want)), f"k = {k}"
    assert not np.array_equal(bits(d["out"][0]), bits(d["rec"]))


@pytest.mark.gpu
def test_cuda_retime_matches_reference_wgsl():
    """The substep-length change through the C ABI: si_mpm_set_substep_dt at half and twice the
    substep, and the substeps setter 8 -> 6 (si_mpm_set_frame), each from the fixture's state, equal
    the reference's mpm-retime output and the oracle's sio_retime bit for bit."""
    from shaderintel_gb300 import _lib as L
    d = fixture("retime.npz")
    for case, (k, want) in enumerate(zip(d["ks"], d["out"])):
        sim = _loaded(d, MATS_G2P, 16)
        dt = sim.substepDt
        if case == 0:
            L.check(L.lib().si_mpm_set_substep_dt(sim._h, dt * 0.5))
        elif case == 1:
            L.check(L.lib().si_mpm_set_substep_dt(sim._h, dt * 2.0))
        else:
            sim.substeps = 6
            assert np.float32(sim.substepDt / dt) == k
        got = sim.readParticles()
        assert np.array_equal(bits(got), bits(want)), f"k = {k}: differs from the reference's mpm-retime"
        assert np.array_equal(bits(got), bits(O.retime(d["rec"], float(k)))), f"k = {k}: differs from the oracle"
        sim.destroy()


# ---------------------------------------------------------------------------- SpatialGrid (src/prims/grid.js)


def _cells_from_order(order, start):
    """The cell of every point, read back from a counting-sort result (order, start)."""
    cell = np.empty(len(order), np.int64)
    for c in np.flatnonzero(np.diff(start.astype(np.int64))):
        cell[order[start[c]:start[c + 1]]] = c
    return cell


def _same_cells_as_fixture(order, start, d):
    """Cells and starts bit-exact; the order within each cell as a set (the reference ranks points
    in a cell by atomic arrival, so any order inside a cell is one of its outcomes)."""
    assert np.array_equal(start, d["start"]), "start differs"
    assert np.array_equal(_cells_from_order(order, start), d["cell"].astype(np.int64)), "cells differ"
    for c in np.flatnonzero(np.diff(start.astype(np.int64))):
        a, b = int(start[c]), int(start[c + 1])
        assert sorted(order[a:b].tolist()) == sorted(d["order"][a:b].tolist()), f"cell {c} holds other points"


def test_restatement_spatial_grid_matches_reference_wgsl():
    import host_ref
    d = fixture("spatial.npz")
    cell, order, start = host_ref.spatial_grid(d["pos"], d["lo"], float(d["cell_size"]), list(d["dims"]))
    assert np.array_equal(np.asarray(cell, np.int64), d["cell"].astype(np.int64))
    _same_cells_as_fixture(np.asarray(order), np.asarray(start, np.uint32), d)
    assert np.diff(d["start"].astype(np.int64)).max() >= 40          # the crowded cell


@pytest.mark.gpu
def test_cuda_spatial_grid_matches_reference_wgsl():
    from shaderintel_gb300.spatial import SpatialGrid
    d = fixture("spatial.npz")
    g = SpatialGrid(maxCount=4096, min=list(d["lo"]), max=list(d["hi"]), cellSize=float(d["cell_size"]))
    assert g.dims == list(d["dims"])
    g.build(d["pos"])
    order, start = g.read()
    _same_cells_as_fixture(order, start, d)
    g.destroy()
