"""The batched form: many scenes of uneven sizes stepped together (one launch per phase for all of
them, replayed from CUDA graphs), against the same scenes stepped alone and against the oracle.

Bar: each scene's particle state after K substeps is the same bits in the batch as alone, for every
tuning setting (particles per CTA, tile capacity, flush strategy) and with graphs on or off."""
import numpy as np
import pytest

import si_oracle as O
from shaderintel_gb300 import MPM, World
from shaderintel_gb300.autotune import autotune

pytestmark = pytest.mark.gpu

# edge, box (cells: lo, size), material, velocity (m/s): uneven sizes, all four models, moving
SPECS = [
    (16, (4, 5, 3), (6, 5, 7), "water", (0.5, -1.0, 0.2)),
    (32, (5, 3, 6), (14, 10, 12), "jelly", (-0.8, 0.0, 0.4)),
    (24, (3, 8, 4), (9, 6, 11), "snow", (0.0, -2.0, 0.0)),
    (48, (10, 3, 12), (20, 16, 18), "sand", (1.0, 0.0, -0.5)),
    (16, (3, 3, 3), (2, 2, 2), "honey", (0.0, 0.0, 0.0)),
    (40, (6, 12, 5), (11, 9, 25), "water", (-1.5, -0.5, 0.0)),
    (32, (20, 4, 3), (7, 20, 8), "rubber", (0.3, 0.3, 0.3)),
]


def make(world, spec, seed_base=0):
    edge, lo, size, mat, vel = spec
    cap = 8 * (size[0] + 1) * (size[1] + 1) * (size[2] + 1)
    sim = MPM(world, grid=edge, maxParticles=cap, substeps=8)
    sim.add({"box": [[x / edge for x in lo], [(x + s) / edge for x, s in zip(lo, size)]]}, material=mat,
            velocity=list(vel), seed=seed_base + 7 * edge + size[0])
    if edge >= 32:
        sim.setColliders([{"type": "sphere", "center": [0.5, 0.3, 0.5], "radius": 0.12, "friction": 0.3}])
    return sim


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def batch(tuning=None, graphs=True):
    w = World()
    w.set_graphs(graphs)
    if tuning:
        w.set_tuning(*tuning)
    return w, [make(w, s) for s in SPECS]


def alone_states(K):
    out = []
    for s in SPECS:
        sim = make(None, s)
        sim.step(dt=sim.substepDt, K=K)
        out.append(sim.readParticles())
        sim.destroy()
    return out


def test_batched_equals_alone_and_oracle():
    K = 13
    w, scenes = batch()
    w.step(K)
    want = alone_states(K)
    for sim, ref in zip(scenes, want):
        assert sim.count == len(ref) > 0
        assert sim.stepCount == K
        assert np.array_equal(bits(sim.readParticles()), bits(ref))
    # one small scene against the CPU oracle from its initial state
    sim0 = make(None, SPECS[0])
    rec0 = sim0.readParticles()
    mats = np.zeros((8, 12), np.float32)
    mats[:len(sim0._rows)] = np.stack(sim0._rows)
    dt = sim0.substepDt
    grav = [np.float32((g * dt * dt) / sim0.dx) for g in sim0.gravity]
    P, _, _ = O.substeps(rec0, sim0.dims, mats, np.zeros((16, 12), np.float32), 0, grav,
                         np.float32(0.5), K, 0, 4, threads=4)
    assert np.array_equal(bits(scenes[0].readParticles()), bits(P))
    sim0.destroy()
    w.destroy()


@pytest.mark.parametrize("tuning", [(512, 2048, 0), (1024, 1331, 0), (256, 343, 0), (256, 2048, 1), (512, 1331, 1)])
def test_tuning_settings_give_the_same_bits(tuning):
    K = 9
    w0, base = batch()
    w0.step(K)
    w1, tuned = batch(tuning)
    w1.step(K)
    for a, b in zip(base, tuned):
        assert np.array_equal(bits(a.readParticles()), bits(b.readParticles()))
        assert np.array_equal(a.readGrid(), b.readGrid())
    w0.destroy()
    w1.destroy()


def test_graphs_on_and_off_and_replays_agree():
    w0, a = batch(graphs=False)
    w1, b = batch(graphs=True)
    for K in (8, 8, 8, 5, 8):   # the 8-substep plan repeats: captured, then replayed
        w0.step(K)
        w1.step(K)
    for x, y in zip(a, b):
        assert np.array_equal(bits(x.readParticles()), bits(y.readParticles()))
    assert w1.launches() > 0
    w0.destroy()
    w1.destroy()


def test_autotuner_picks_a_setting_and_results_stay_exact():
    w, scenes = batch()
    cands = [(256, 2048, 0), (512, 2048, 0), (256, 343, 1)]
    best = autotune(w, substeps=4, repeats=1, cands=cands)
    assert (best["particles_per_cta"], best["tile_nodes"], best["flush"]) in cands
    assert len(best["table"]) == 3 and best["ms_per_substep"] > 0
    total = 4 * 2 * len(cands)          # the tuner's substeps are real substeps
    w.step(7)
    want = alone_states(total + 7)
    for sim, ref in zip(scenes, want):
        assert sim.stepCount == total + 7
        assert np.array_equal(bits(sim.readParticles()), bits(ref))
    w.destroy()


def test_scene_added_and_destroyed_mid_batch():
    """Scenes join and leave a world between steps; the others are unaffected."""
    w, scenes = batch()
    w.step(4)
    late = make(w, SPECS[2], seed_base=99)
    scenes[3].destroy()
    w.step(6)
    ref = make(None, SPECS[2], seed_base=99)
    ref.step(dt=ref.substepDt, K=6)
    assert np.array_equal(bits(late.readParticles()), bits(ref.readParticles()))
    want = alone_states(10)
    for k in (0, 1, 2, 4, 5, 6):
        assert np.array_equal(bits(scenes[k].readParticles()), bits(want[k]))
    ref.destroy()
    w.destroy()


def test_segmented_sort_tile_edges():
    """Scenes whose particle counts sit on either side of the sort's 4096-key tiles (1, 4095, 4096,
    4097, 8193) sorted in one tick: each scene's segment is padded to whole tiles, so every count
    exercises another padding; the records after two sorts equal the scenes stepped alone."""
    src = make(None, (48, (10, 3, 12), (20, 16, 18), "sand", (1.0, 0.0, -0.5)))
    src.step(dt=src.substepDt, K=2)
    rec = src.readParticles()
    src.destroy()
    counts = [1, 4095, 4096, 4097, 8193]

    def scene(world, n):
        sim = MPM(world, grid=48, maxParticles=n, substeps=8)
        sim._material("sand")
        assert sim.addRecords(rec[:n]) == n
        return sim

    w = World()
    batch_sims = [scene(w, n) for n in counts]
    w.step(8)                                   # sorts at the first and fifth substep
    for n, b in zip(counts, batch_sims):
        a = scene(None, n)
        a.step(dt=a.substepDt, K=8)
        assert np.array_equal(bits(a.readParticles()), bits(b.readParticles())), n
        assert all(np.array_equal(x, y) for x, y in zip(a.readBins(), b.readBins())), n
        a.destroy()
    w.destroy()


def _water_records():
    src = make(None, (16, (4, 5, 3), (6, 5, 7), "water", (0.5, -1.0, 0.2)))
    src.step(dt=src.substepDt, K=2)
    rec = src.readParticles()
    src.destroy()
    return rec


def _scene_from(rec, world, n):
    sim = MPM(world, grid=16, maxParticles=max(n, 1), substeps=8)
    sim._material("water")
    if n:
        assert sim.addRecords(rec[:n]) == n
    return sim


def _check_against_alone(rec, counts, sims, which):
    for i in which:
        a = _scene_from(rec, None, counts[i])
        a.step(dt=a.substepDt, K=8)
        assert np.array_equal(bits(a.readParticles()), bits(sims[i].readParticles())), i
        assert all(np.array_equal(x, y) for x, y in zip(a.readBins(), sims[i].readBins())), i
        a.destroy()


def test_more_scenes_than_the_shared_scene_tables():
    """1,100 scenes in one tick, more than the 1,024 that the kernels' shared-memory scene tables
    hold: the G2P and the sort find a chunk's scene in the tick table in global memory, and the grid
    update walks the host's node chunks instead of splitting the regions evenly. Sampled scenes on
    both sides of the table's size equal the same scenes stepped alone after two sorts."""
    rec = _water_records()
    counts = [100 + (i * 37) % (len(rec) - 100) for i in range(1100)]
    w = World()
    sims = [_scene_from(rec, w, n) for n in counts]
    w.step(8)
    _check_against_alone(rec, counts, sims, [0, 1, 511, 1023, 1024, 1025, 1099])
    w.destroy()


def test_even_grid_split_with_an_empty_scene():
    """A tick of six scenes, one without particles (an empty region, no nodes in the evenly split
    grid update) between others of uneven sizes: every scene equals the same scene stepped alone."""
    rec = _water_records()
    counts = [700, 0, 1500, 1, 4096 % len(rec), 333]
    w = World()
    sims = [_scene_from(rec, w, n) for n in counts]
    w.step(8)
    _check_against_alone(rec, counts, sims, range(len(counts)))
    w.destroy()
