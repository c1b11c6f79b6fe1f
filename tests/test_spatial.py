"""SpatialGrid (src/prims/grid.js): the numpy restatement on hand-checked cases (CPU), and the
CUDA build through the C ABI against it (GPU): order and start bit-exact, gather, the 27-cell
neighbour ranges, and binning an MPM scene's particles in place."""
import numpy as np
import pytest

import host_ref

from conftest import mulberry32


def test_restatement_hand_checked():
    # 2 x 3 x 2 cells of size 0.5 from (0, 0, 0); x fastest (grid.js:17-19); outside points clamp
    pts = np.array([[0.1, 0.1, 0.1], [0.7, 0.1, 0.1], [0.1, 1.2, 0.6], [5.0, -3.0, 0.2], [0.6, 0.6, 0.9],
                    [0.2, 0.2, 0.2]], np.float32)
    cell, order, start = host_ref.spatial_grid(pts, [0, 0, 0], 0.5, [2, 3, 2])
    assert cell.tolist() == [0, 1, 10, 1, 9, 0]
    assert order.tolist() == [0, 5, 1, 3, 4, 2]          # stable: index order inside a cell
    assert start.tolist() == [0, 2, 4, 4, 4, 4, 4, 4, 4, 4, 5, 6, 6]
    assert start[-1] == len(pts)


@pytest.mark.gpu
def test_cuda_spatial_grid_matches_restatement():
    from shaderintel_gb300.spatial import SpatialGrid
    R = mulberry32(9)
    n = 50000
    pts = np.array([[R() * 2.4 - 0.2, R() * 1.4 - 0.2, R() * 1.2 - 0.1, 0.0] for _ in range(n)], np.float32)
    g = SpatialGrid(maxCount=60000, min=[0, 0, 0], max=[2.0, 1.0, 1.0], cellSize=0.07)
    assert g.dims == [29, 15, 15]
    g.build(pts)
    order, start = g.read()
    _, want_order, want_start = host_ref.spatial_grid(pts, [0, 0, 0], 0.07, g.dims)
    assert np.array_equal(order, want_order)
    assert np.array_equal(start, want_start)
    attr = np.stack([np.arange(n, dtype=np.float32), -np.arange(n, dtype=np.float32)], 1)
    assert np.array_equal(g.gather(attr), attr[order])
    # neighbour certificate: every point within one cell size of a probe lies in its 27-cell ranges
    sorted_pts = pts[order, :3]
    for k in range(0, n, 997):
        p = pts[k, :3]
        inside = set()
        for a, b in g.neighbors(p, start):
            inside.update(order[a:b].tolist())
        near = np.flatnonzero(np.linalg.norm(pts[:, :3] - p, axis=1) < 0.07)
        near = [j for j in near if all(0 <= pts[j, a] < [2.0, 1.0, 1.0][a] for a in range(3))
                and all(0 <= p[a] < [2.0, 1.0, 1.0][a] for a in range(3))]
        assert set(near) <= inside
    assert sorted_pts.shape == (n, 3)
    g.build(pts[:0])
    order, start = g.read()
    assert len(order) == 0 and not start.any()
    g.destroy()


@pytest.mark.gpu
def test_cuda_spatial_grid_over_mpm_particles():
    from shaderintel_gb300 import MPM, World
    from shaderintel_gb300.spatial import SpatialGrid
    w = World()
    sim = MPM(w, grid=32, maxParticles=40000)
    sim.add({"sphere": [[0.5, 0.5, 0.5], 0.3]}, material="water")
    sim.step()
    g = SpatialGrid(maxCount=40000, min=[0, 0, 0], max=[32, 32, 32], cellSize=2.0, world=w)
    g.build(sim)
    order, start = g.read()
    x = sim.readParticles()[:, :3]
    _, want_order, want_start = host_ref.spatial_grid(x, [0, 0, 0], 2.0, g.dims)
    assert np.array_equal(order, want_order) and np.array_equal(start, want_start)
    g.destroy()
    w.destroy()
