"""The served form: resident scenes, step(dt, K) requests from several threads run by continuous
batching, admission by HBM footprint, retirement.

Bar: a scene served among others ends in the same bits as the same scene stepped alone with the same
substeps (requests of different K interleave round by round, so this shows each result is the same
alone and in the mix); admission refuses a scene past the budget and accepts it once memory is
freed; statistics report what ran."""
import random
import threading
import time

import numpy as np
import pytest

from shaderintel_gb300 import MPM, SIError
from shaderintel_gb300.serving import Server

pytestmark = pytest.mark.gpu

SCENES = [
    (16, (4, 5, 3), (6, 5, 7), "water", (0.5, -1.0, 0.2)),
    (32, (5, 3, 6), (14, 10, 12), "jelly", (-0.8, 0.0, 0.4)),
    (24, (3, 8, 4), (9, 6, 11), "snow", (0.0, -2.0, 0.0)),
    (40, (10, 3, 12), (20, 16, 18), "sand", (1.0, 0.0, -0.5)),
    (32, (6, 12, 5), (11, 9, 15), "honey", (-1.5, -0.5, 0.0)),
]


def cap_of(spec):
    _, _, size, _, _ = spec
    return 8 * (size[0] + 1) * (size[1] + 1) * (size[2] + 1)


def fill(sim, spec):
    edge, lo, size, mat, vel = spec
    sim.add({"box": [[x / edge for x in lo], [(x + s) / edge for x, s in zip(lo, size)]]}, material=mat,
            velocity=list(vel), seed=3 + edge)
    return sim


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def alone(spec, plan):
    """The scene stepped alone: the same (dt, K) requests in order, as step(dt, K) calls."""
    sim = fill(MPM(None, grid=spec[0], maxParticles=cap_of(spec), substeps=8), spec)
    for dt, K in plan:
        sim.step(dt=dt, K=K)
    out = sim.readParticles()
    sim.destroy()
    return out


@pytest.mark.parametrize("budget", [4 * 10 ** 9, 6 * 10 ** 7])
def test_served_results_equal_alone(budget):
    """Served scenes keep one particle buffer (their sort substeps read a gathered copy of the old
    state). With the small budget the sort scratch reserve (budget / 32) holds about 20,000 particles,
    so a tick whose scenes sort together runs as several groups of scenes: the bits do not change."""
    srv = Server(budget_bytes=budget)
    sims = [fill(srv.admit(grid=s[0], maxParticles=cap_of(s), substeps=8), s) for s in SCENES]
    dt0 = sims[0].substepDt
    rng = random.Random(5)
    plans = [[] for _ in SCENES]
    for k in range(len(SCENES)):
        for _ in range(rng.randint(3, 6)):
            plans[k].append((dt0, rng.randint(1, 12)))
    plans[2][1] = (dt0 * 0.5, plans[2][1][1])   # one request at another dt: the retime path
    tickets = []
    lock = threading.Lock()

    def client(ids, seed):
        r = random.Random(seed)
        for k in ids:
            for dt, K in plans[k]:
                t = srv.submit(sims[k], dt=dt, K=K)
                with lock:
                    tickets.append(t)
                time.sleep(r.uniform(0, 0.003))

    threads = [threading.Thread(target=client, args=(ids, 11 + j)) for j, ids in enumerate(([0, 3], [1, 4], [2]))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for t in tickets:
        assert srv.wait(t, timeout_ms=120000) == 0
    st = srv.stats()
    assert st["requests_done"] == len(tickets)
    assert st["substeps_done"] > 0 and st["p99_ms"] >= st["p50_ms"] > 0
    assert st["resident_scenes"] == len(SCENES)
    for k, spec in enumerate(SCENES):
        assert sims[k].stepCount == sum(K for _, K in plans[k])
        assert np.array_equal(bits(sims[k].readParticles()), bits(alone(spec, plans[k])))
    srv.destroy()


def test_admission_by_footprint_and_retire():
    one = Server(budget_bytes=10 ** 12)
    reserve = one.stats()["resident_bytes"]        # the sort scratch reserve: min(2 GiB, budget / 32)
    assert reserve == min(2 << 30, 10 ** 12 // 32)
    probe = one.admit(grid=32, maxParticles=100000)
    fp = one.stats()["resident_bytes"] - reserve
    one.destroy()
    # one particle buffer (128 B a particle), two grids, no key buffers: not two particle buffers
    assert 100000 * 128 + 32 ** 3 * 32 <= fp < 100000 * 136 + 32 ** 3 * 32

    budget = int(fp * 1.5 * 32 / 31)               # a reserve of budget / 32 leaves room for 1.5 scenes
    srv = Server(budget_bytes=budget)
    a = srv.admit(grid=32, maxParticles=100000)
    with pytest.raises(SIError) as e:
        srv.admit(grid=32, maxParticles=100000)
    assert e.value.code == "out-of-memory"
    assert srv.stats()["resident_scenes"] == 1
    fill(a, SCENES[1])
    t = srv.submit(a, K=6)
    srv.retire(a)                  # queued or running, the request ends (done or destroyed)
    st = srv.wait(t, timeout_ms=60000)
    assert st in (0, 3)
    b = srv.admit(grid=32, maxParticles=100000)   # the freed budget admits the next scene
    fill(b, SCENES[1])
    assert srv.wait(srv.submit(b, K=3), timeout_ms=60000) == 0
    assert b.stepCount == 3
    assert srv.stats()["resident_scenes"] == 1
    srv.destroy()
    del probe


def test_poll_and_edits_while_serving():
    """Resident scenes can be edited between rounds; a poll reports progress."""
    srv = Server(budget_bytes=4 * 10 ** 9)
    s0 = fill(srv.admit(grid=SCENES[0][0], maxParticles=cap_of(SCENES[0]) * 2), SCENES[0])
    t = srv.submit(s0, K=20)
    n_before = s0.count
    s0.add({"box": [[0.6, 0.6, 0.6], [0.7, 0.7, 0.7]]}, material="water")   # lands between rounds
    assert s0.count > n_before
    deadline = time.time() + 60
    done = False
    while time.time() < deadline and not done:
        done, status = srv.poll(t)
        time.sleep(0.002)
    assert done and status == 0
    assert s0.stepCount == 20
    x = s0.readPositions()
    assert np.isfinite(x).all()
    srv.destroy()


def test_destroyed_server_rejects_work():
    srv = Server(budget_bytes=10 ** 9)
    s = fill(srv.admit(grid=16, maxParticles=cap_of(SCENES[0])), SCENES[0])
    srv.wait(srv.submit(s, K=2), timeout_ms=30000)
    srv.destroy()
    with pytest.raises(SIError):
        s.step()   # the world and its scenes went with the server it owned


def test_queued_requests_keep_their_own_colliders():
    """A sphere moved between submits: requests queued on one scene each run with the collider
    table they were submitted with, as the same step(dt, K) calls with setColliders in between."""
    spec = (32, (4, 3, 5), (20, 12, 18), "water", (1.0, 0.0, 0.5))
    centers = [(0.40, 0.20, 0.45), (0.46, 0.22, 0.47), (0.52, 0.24, 0.49), (0.58, 0.26, 0.51)]
    Ks = [5, 3, 7, 4]

    def sphere(c):
        return [{"type": "sphere", "center": list(c), "radius": 0.12, "velocity": [0.3, 0.1, 0.1]}]

    srv = Server(budget_bytes=4 * 10 ** 9)
    big = fill(srv.admit(grid=64, maxParticles=400000), (64, (3, 3, 3), (50, 20, 50), "sand", (0, 0, 0)))
    sim = fill(srv.admit(grid=spec[0], maxParticles=cap_of(spec)), spec)
    dt = sim.substepDt
    tb = srv.submit(big, dt=dt, K=16)      # keeps the rounds busy while the others queue
    tickets = []
    for c, K in zip(centers, Ks):
        sim.setColliders(sphere(c))
        tickets.append(srv.submit(sim, dt=dt, K=K))
    sim.setColliders([])                   # the queued requests keep their tables
    for t in tickets + [tb]:
        assert srv.wait(t, timeout_ms=120000) == 0
    served = sim.readParticles()
    srv.destroy()

    ref = fill(MPM(None, grid=spec[0], maxParticles=cap_of(spec), substeps=8), spec)
    for c, K in zip(centers, Ks):
        ref.setColliders(sphere(c))
        ref.step(dt=dt, K=K)
    want = ref.readParticles()
    ref.destroy()
    assert np.array_equal(bits(served), bits(want))

    # and the colliders matter here: the same steps without them end elsewhere
    free = fill(MPM(None, grid=spec[0], maxParticles=cap_of(spec), substeps=8), spec)
    for K in Ks:
        free.step(dt=dt, K=K)
    assert not np.array_equal(bits(free.readParticles()), bits(want))
    free.destroy()


def test_explicit_sort_of_a_served_scene():
    """_sort() of a one-buffer scene reorders into a fresh buffer; the records equal those of the
    same scene with two buffers."""
    srv = Server(budget_bytes=4 * 10 ** 9)
    spec = SCENES[3]
    a = fill(srv.admit(grid=spec[0], maxParticles=cap_of(spec), substeps=8), spec)
    assert srv.wait(srv.submit(a, K=5), timeout_ms=60000) == 0
    b = fill(MPM(None, grid=spec[0], maxParticles=cap_of(spec), substeps=8), spec)
    b.step(dt=b.substepDt, K=5)
    a._sort()                                  # between rounds: the world's lock serialises it
    b._sort()
    assert np.array_equal(bits(a.readParticles()), bits(b.readParticles()))
    assert np.array_equal(a.readBins(keys=False)[1], b.readBins()[1])
    with pytest.raises(SIError):   # a served scene keeps no block keys
        a.readBins()
    srv.destroy()
    b.destroy()
