"""Fluid <-> rigid coupling (src/physics/coupling.js) on the GPU against the oracle: particle state
after coupled substeps and the bodies' reaction impulses bit-exact, alone and in a batch."""
import numpy as np
import pytest

import si_oracle as O
from shaderintel_gb300 import MPM, World
from shaderintel_gb300.mpm import body_record

pytestmark = pytest.mark.gpu


def bodies():
    s = np.sin(np.pi / 12)
    return np.stack([
        body_record([0.5, 0.3, 0.5], [0.1] * 3, "sphere", velocity=[0.1, -0.2, 0], angular_velocity=[0, 0, 1], mass=2),
        body_record([0.33, 0.28, 0.4], [0.08, 0.05, 0.1], "box", quaternion=[0.2, 0.3, 0.1, 0.93], velocity=[0, 0, 0.3],
                    angular_velocity=[1, 0, 0], mass=1),
        body_record([0.66, 0.25, 0.62], [0.05, 0.08, 0.05], "capsule", quaternion=[0, 0, s, np.cos(np.pi / 12)]),
        body_record([0.3, 0.3, 0.7], [0.06] * 3, "sphere", mass=1, flags=4),
        body_record([0.7, 0.3, 0.3], [0.06] * 3, "sphere", mass=1, group=2)])


def pool(world=None, grid=24):
    sim = MPM(world, grid=grid, maxParticles=120000, substeps=8)
    sim.add({"box": [[0.15, 0.15, 0.15], [0.85, 0.45, 0.85]]}, material="water", velocity=[0.2, -0.5, 0.1])
    sim.couple(bodies(), friction=0.2, band=0.5, mask=1, densityScale=1.0)
    return sim


def oracle_run(sim, rec, K):
    mats = np.zeros((8, 12), np.float32)
    mats[:len(sim._rows)] = np.stack(sim._rows)
    dt = sim.substepDt
    grav = [np.float32((g * dt * dt) / sim.dx) for g in sim.gravity]
    acc = np.zeros(5 * 8, np.int32)
    cpl = {"bodies": bodies(), "params": [0, 0, 0, sim.dx, 1 / sim.dx, 0, dt / sim.dx, 0.2, 0.5], "mask": 1,
           "dt": dt, "acc": acc}
    P, _, _ = O.substeps(rec, sim.dims, mats, np.zeros((16, 12), np.float32), 0, grav, np.float32(0.5), K, 0, 4,
                         threads=8, coupling=cpl)
    ext, _ = O.couple_apply(acc, 5, np.float32(1.0 * sim.dx ** 4 / dt), sim.dx)
    return P, ext


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_coupled_substeps_and_impulses_match_oracle():
    sim = pool()
    rec = sim.readParticles()
    sim.step(dt=sim.substepDt, K=10)
    imp = sim.readImpulses()
    P, ext = oracle_run(sim, rec, 10)
    assert np.array_equal(bits(sim.readParticles()), bits(P))
    assert np.array_equal(bits(imp), bits(ext))
    nz = imp[:, [0, 1, 2, 4, 5, 6]].any(1)
    assert nz.tolist() == [True, True, False, False, False]
    assert not sim.readImpulses().any()          # read restarts the sums
    sim.destroy()


def test_coupled_scene_in_a_batch_equals_alone():
    w = World()
    a = pool(w)
    other = MPM(w, grid=16, maxParticles=20000, substeps=8)
    other.add({"box": [[0.3, 0.3, 0.3], [0.6, 0.6, 0.6]]}, material="jelly")
    w.step(6)
    alone = pool()
    alone.step(dt=alone.substepDt, K=6)
    assert np.array_equal(bits(a.readParticles()), bits(alone.readParticles()))
    assert np.array_equal(bits(a.readImpulses()), bits(alone.readImpulses()))
    a.uncouple()
    w.step(2)
    assert a.stepCount == 8
    alone.destroy()
    w.destroy()


def test_set_bodies_moves_the_boundary():
    sim = pool()
    sim.step(dt=sim.substepDt, K=2)
    sim.readImpulses()
    b = bodies()
    b[0, 0:3] = [0.5, 0.9, 0.5]                  # the sphere leaves the water
    b[1, 0:3] = [0.5, 0.9, 0.2]
    sim.setBodies(b)
    sim.step(dt=sim.substepDt, K=2)
    imp = sim.readImpulses()
    assert not imp[:2].any()
    sim.destroy()


def test_many_bodies_match_oracle():
    """280 bodies: several ballot rounds of the cull, and (130 spheres piled on one spot) tiles whose
    candidates pass the reference's 128-body cap. Particle state and every body's impulses are
    bit-exact to the oracle."""
    rng = np.random.default_rng(17)
    many = np.stack([body_record(list(rng.uniform([0.2, 0.15, 0.2], [0.8, 0.45, 0.8])),
                                 [float(rng.uniform(0.02, 0.05))] * 3, "sphere" if k % 3 else "box",
                                 quaternion=list(rng.normal(size=4)), velocity=list(rng.uniform(-0.3, 0.3, 3)),
                                 angular_velocity=list(rng.uniform(-1, 1, 3)), mass=float(k % 4))
                     for k in range(150)])
    pile = np.stack([body_record([0.5, 0.3, 0.5], [0.04] * 3, "sphere", velocity=[0, -0.1, 0], mass=1.0)
                     for _ in range(130)])
    allb = np.concatenate([many, pile])
    sim = MPM(grid=24, maxParticles=120000, substeps=8)
    sim.add({"box": [[0.15, 0.15, 0.15], [0.85, 0.45, 0.85]]}, material="water", velocity=[0.2, -0.5, 0.1])
    sim.couple(allb, friction=0.2, band=0.5, mask=1, densityScale=1.0)
    rec = sim.readParticles()
    K = 6
    sim.step(dt=sim.substepDt, K=K)
    imp = sim.readImpulses()
    mats = np.zeros((8, 12), np.float32)
    mats[:len(sim._rows)] = np.stack(sim._rows)
    dt = sim.substepDt
    grav = [np.float32((g * dt * dt) / sim.dx) for g in sim.gravity]
    acc = np.zeros(len(allb) * 8, np.int32)
    cpl = {"bodies": allb, "params": [0, 0, 0, sim.dx, 1 / sim.dx, 0, dt / sim.dx, 0.2, 0.5], "mask": 1,
           "dt": dt, "acc": acc}
    P, _, _ = O.substeps(rec, sim.dims, mats, np.zeros((16, 12), np.float32), 0, grav, np.float32(0.5), K, 0, 4,
                         threads=8, coupling=cpl)
    ext, _ = O.couple_apply(acc, len(allb), np.float32(1.0 * sim.dx ** 4 / dt), sim.dx)
    assert np.array_equal(bits(sim.readParticles()), bits(P))
    assert np.array_equal(bits(imp), bits(ext))
    assert imp[:, [0, 1, 2, 4, 5, 6]].any(1).sum() > 50
    sim.destroy()
