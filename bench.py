#!/usr/bin/env python3
"""bench.py — MLS-MPM particle-substeps/s on one GB300 through libsi_cuda.

Workload (default, `--config mixed`): the single large mixed-material scene — 128^3 grid, a
64^3-cell water block at the floor corner plus a 24^3-cell neo-Hookean jelly cube whose top is
at y = 90 cells, 8 particles per cell (2,207,744 particles), the reference's defaults
(8 substeps per 1/60 s frame, sort every 4 substeps, gravity -9.81). Inputs are seeded synthetic
lattices (the reference's own jittered sampler); no dataset is involved.

One bench step = one frame = the reference's MPM.step() = 8 substeps. `value` is device-timed
with CUDA events on the library's stream, state resident in HBM (282.6 MB of particle state,
larger than the 129 MB L2, so no flush is needed between steps). `e2e` is the same metric through
the public API with host buffers, on a fresh copy of the scene with the same warm-up (so the same
frames): every frame uploads the 16-row collider table the reference uploads each step and reads
every particle position back into pinned host memory.

The same line carries the batched form (256 seeded scenes of uneven sizes and materials, one launch
per phase, autotuned, against the same scenes stepped one by one), the served form (Poisson
arrivals of step(dt, K) over resident scenes: small scenes at 2,000 and 8,000 requests/s, and
1 M-particle plasticity scenes under a 150 GB admission budget at 2,000 and 200 requests/s), a
conservation run of the dam break and a few host-side costs.

`--impl reference` times the reference algorithm on the host cores instead: the CPU restatement
(oracle/, the reference's WGSL runs only in a browser), all threads, one substep of the same
scene per step (a bounded sample).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "mixed": {"grid": 128, "substeps": 8, "blocks": [
        ("water", [3, 3, 3], [67, 67, 67], [0, 0, 0]),
        ("jelly", [72, 66, 52], [96, 90, 76], [0, 0, 0])],
        "desc": "mixed_128: 128^3 grid, 64^3-cell water block at the floor corner + 24^3-cell neo-Hookean "
                "jelly cube (top at y=90 cells), 8 ppc"},
    "dam_break": {"grid": 32, "substeps": 8, "blocks": [("water", [3, 3, 3], [19, 19, 19], [0, 0, 0])],
                  "desc": "dam_break_32: 32^3 grid, 16^3-cell water block at the corner, 8 ppc"},
    "plasticity": {"grid": 96, "substeps": 8, "blocks": [
        ("snow", [3, 3, 3], [93, 20, 45], [0, 0, 0]),
        ("sand30", [25, 3, 52], [65, 50, 86], [0, 0, 0])],
        "desc": "plasticity_96: 96^3 grid, 90x17x42-cell snow slab + 40x47x34-cell Drucker-Prager sand column "
                "(friction 30 deg), 8 ppc"},
}
SAND30 = {"kind": 3, "density": 1.6, "stiffness": 0.6, "poisson": 0.3, "friction": 30}


def material_def(name):
    from shaderintel_gb300 import MATERIALS
    return dict(SAND30) if name == "sand30" else dict(MATERIALS[name])


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- clocks
class Clocks:
    """nvidia-smi sampled every 50 ms from before the timed region to after it. start() and stop()
    bracket the timed region, and only the samples stamped inside it are reported (all of them if
    none is, with `in_window` 0)."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.idx = gpu_index
        self.t0 = self.t1 = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)   # let the sampler start before the timed region does
        except OSError:
            self.proc = None

    def start(self):
        self.t0 = time.time()

    def stop(self):
        self.t1 = time.time()
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.1)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        import datetime
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(f[2]), float(f[3]), [n for n, v in zip(names, f[6:10]) if v.lower() == "active"]))
            except ValueError:
                continue
        lo = (self.t0 if self.t0 is not None else 0.0) - 0.05
        inside = [r for r in rows if lo <= r[0] <= self.t1 + 0.05]
        use = inside or rows
        sm = [r[1] for r in use]
        reasons = sorted({n for r in use for n in r[3]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": use[-1][2] if use else None,
                "samples": len(use), "in_window": len(inside), "reasons": reasons}


# ----------------------------------------------------------------------------- scenes
def build_gpu(cfg, world):
    from shaderintel_gb300 import MPM
    c = CONFIGS[cfg]
    g = c["grid"]
    n_est = sum(8 * (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]) for _, lo, hi, _ in c["blocks"])
    sim = MPM(world, grid=g, maxParticles=n_est, substeps=c["substeps"])
    for name, lo, hi, vel in c["blocks"]:
        sim.add({"box": [[x / g for x in lo], [x / g for x in hi]]}, material=material_def(name), velocity=vel)
    return sim


def build_cpu(cfg):
    """The same scene for the CPU restatement (oracle emission, no GPU library involved)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import host_ref
    import si_oracle as O
    c = CONFIGS[cfg]
    g = c["grid"]
    geo = host_ref.geometry(g)
    dt = 1 / 60 / c["substeps"]
    recs, mats = [], np.zeros((8, 12), np.float32)
    for k, (name, lo, hi, vel) in enumerate(c["blocks"]):
        mats[k] = host_ref.material_row(material_def(name))
        seed = sum(len(r) for r in recs) + 1
        recs.append(O.emit_box([x / g for x in lo], [x / g for x in hi], geo["dx"] / 2, 0.6, seed, k, vel,
                               geo["dims"], geo["dx"], [0, 0, 0], dt))
    rec = np.concatenate(recs)
    grav = [np.float32(0.0), np.float32((-9.81 * dt * dt) / geo["dx"]), np.float32(0.0)]
    return rec, mats, geo, grav, np.float32(4 * (1 / 2 ** 3)), c["substeps"]


def cpu_measure(cfg, target_s, steps=None, warmup=0):
    """Times the oracle (all host threads) on the scene; returns (particle-substeps/s, substeps, threads)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import si_oracle as O
    rec, mats, geo, grav, vol4, _ = build_cpu(cfg)
    threads = os.cpu_count() or 1
    cols = np.zeros((16, 12), np.float32)
    P, sc = rec, 0
    if warmup:
        P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, warmup, sc, threads=threads)
    if steps is None:
        t = time.perf_counter()
        P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, 1, sc, threads=threads)
        t1 = time.perf_counter() - t
        steps = max(1, min(16, int(target_s / max(t1, 1e-6))))
    t = time.perf_counter()
    P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, steps, sc, threads=threads)
    el = time.perf_counter() - t
    return len(rec) * steps / el, steps, threads, len(rec), el


# ----------------------------------------------------------------------------- pinned host memory
def pinned_floats(n):
    import numpy as np
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            rt = None
    if rt is not None:
        p = ctypes.c_void_p()
        if rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(max(n, 1) * 4), 1) == 0:
            buf = (ctypes.c_float * max(n, 1)).from_address(p.value)
            return np.ctypeslib.as_array(buf)[:n], True
    return np.empty(n, np.float32), False


# ----------------------------------------------------------------------------- arms
def run_ours(a, rank):
    import numpy as np
    from shaderintel_gb300 import World
    from shaderintel_gb300 import _lib as L
    lib = L.lib()
    c = CONFIGS[a.config]
    world = World()
    sim = build_gpu(a.config, world)
    n_p = sim.count
    nodes = sim.numNodes
    subs = c["substeps"]
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))   # sampling before the warm-up
    for _ in range(a.warmup):
        sim.step()
    world.sync()
    l0 = world.launches()
    clocks.start()
    world.mark(0)
    for _ in range(a.steps):
        sim.step()
    world.mark(1)
    ms = world.elapsed(0, 1)
    clk = clocks.stop()
    launches = world.launches() - l0
    value = n_p * subs * a.steps / (ms / 1e3)

    # per-phase kernel times (events around each phase on the launching stream)
    world.profile(enable=True, reset=True)
    pf = 4
    for _ in range(pf):
        sim.step()
    ph = world.profile(enable=False, reset=True)
    launches_g2p = pf * subs
    g2p_ms = ph["mpm g2p"] / launches_g2p
    b_alg = 256 * n_p + 32 * nodes          # algorithmic bytes per substep (one k_g2p launch)
    peak, peak_kind = load_peaks()
    achieved = b_alg / (g2p_ms / 1e3) / 1e9

    # end to end through the public API with host buffers: every frame uploads the collider table and
    # reads every position back, as readPositions()' Promise: frame k's positions are copied into one
    # of two pinned buffers while frame k+1 runs, and the loop waits for frame k before queueing k+2.
    # It runs on a fresh copy of the scene with the same warm-up, so it times the same frames of the
    # simulation as `value` (a frame's cost changes as the scene evolves)
    sim.destroy()
    sim = build_gpu(a.config, world)
    for _ in range(a.warmup):
        sim.step()
    world.sync()
    bufs = [pinned_floats(n_p * 3) for _ in range(2)]
    pinned = bufs[0][1]
    cols, _ = pinned_floats(16 * 12)
    cols[:] = 0
    h = sim._h
    ticket = ctypes.c_uint64()
    pending = []
    t = time.perf_counter()
    for k in range(a.steps):
        lib.si_mpm_set_colliders(h, L.fptr(cols), 0)   # the per-step collider table upload (mpm.js:586)
        L.check(lib.si_mpm_step(h, 0.0, 0))
        if len(pending) == 2:
            L.check(lib.si_mpm_read_wait(h, pending.pop(0)))
        L.check(lib.si_mpm_read_positions_async(h, L.fptr(bufs[k % 2][0]), 0, n_p, ctypes.byref(ticket)))
        pending.append(ticket.value)
    for tk in pending:
        L.check(lib.si_mpm_read_wait(h, tk))
    e2e_s = time.perf_counter() - t
    e2e = n_p * subs * a.steps / e2e_s

    out = {
        "metric": METRIC,
        "value": value, "unit": "particle-substeps/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded jittered lattice of the reference sampler)",
        "config": run_config(c, n_p, nodes),
        "roofline": {"kernel": "k_g2p (G2P + constitutive + fused next-substep P2G)", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic_per_launch(a.config),
                     "algorithmic_bytes_per_launch": b_alg, "avg_launch_ms": g2p_ms},
        "substep_roofline": {"achieved": b_alg * subs * a.steps / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                             "frac": b_alg * subs * a.steps / (ms / 1e3) / 1e9 / peak},
        "phases_ms_per_substep": {k: v / launches_g2p for k, v in ph.items()},
        "e2e": {"value": e2e, "unit": "particle-substeps/s", "h2d_bytes_per_step": 1200,
                "d2h_bytes_per_step": n_p * 12, "pinned": pinned},
        "gpu_launches": launches,
        "clocks": clk,
    }
    if rank == 0 and not a.no_cpu:
        v, st, th, n, el = cpu_measure(a.config, a.cpu_seconds)
        out["cpu_baseline"] = {"value": v, "unit": "particle-substeps/s", "cores": th, "kind": "port",
                               "sample": f"{st} substeps of the full {n}-particle scene from its initial state "
                                         f"({el:.1f} s, oracle/ C restatement, OpenMP {th} threads)"}
    world.destroy()
    return out


# ----------------------------------------------------------------------------- batched and served forms
BATCH_EDGES = (16, 32, 48, 64)
BATCH_MATERIALS = ("water", "jelly", "snow", "sand")


def scene_specs(n, seed):
    """Scenes drawn as the batched workload: grid edge uniform in {16,32,48,64}, particle count
    log-uniform in [2k, 260k] capped by 8 ppc of the interior (edge - 6)^3 cells, material uniform
    over water/jelly/snow/sand, a box of that many cells at a random place, a random velocity."""
    import math
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        edge = rng.choice(BATCH_EDGES)
        inner = edge - 6
        target = min(math.exp(rng.uniform(math.log(2000), math.log(260000))), 8 * inner ** 3)
        cells = target / 8
        sx = sy = max(1, min(inner, round(cells ** (1 / 3))))
        sz = max(1, min(inner, round(cells / (sx * sy))))
        lo = [3 + rng.randrange(0, inner - d + 1) for d in (sx, sy, sz)]
        vel = [rng.uniform(-1, 1), rng.uniform(-1, 0.5), rng.uniform(-1, 1)]
        out.append({"edge": edge, "lo": lo, "size": [sx, sy, sz], "material": rng.choice(BATCH_MATERIALS),
                    "vel": vel, "seed": rng.randrange(1, 1 << 30)})
    return out


def spec_capacity(s):
    return 8 * (s["size"][0] + 1) * (s["size"][1] + 1) * (s["size"][2] + 1)


def fill_scene(sim, s):
    e = s["edge"]
    sim.add({"box": [[x / e for x in s["lo"]], [(x + d) / e for x, d in zip(s["lo"], s["size"])]]},
            material=s["material"], velocity=s["vel"], seed=s["seed"])
    return sim


def plasticity_specs(n, seed):
    """Scenes drawn as the plasticity workload: 96^3 grid, a snow slab on the floor (z below 47) and a
    Drucker-Prager sand column (friction 30 deg, z from 50) beside it, sizes and x/z placement
    seeded, 8 ppc: 0.67-1.27 M particles, about 0.94 M on average, half snow and half sand."""
    import random
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        slab = [rng.randint(80, 90), rng.randint(14, 20), rng.randint(38, 44)]
        col = [rng.randint(34, 44), rng.randint(40, 50), rng.randint(30, 36)]
        lo_s = [3 + rng.randint(0, 90 - slab[0]), 3, 3 + rng.randint(0, 44 - slab[2])]
        lo_c = [3 + rng.randint(0, 90 - col[0]), 3, 50 + rng.randint(0, 43 - col[2])]
        out.append({"edge": 96, "blocks": [("snow", lo_s, slab), ("sand30", lo_c, col)],
                    "seeds": [rng.randrange(1, 1 << 30), rng.randrange(1, 1 << 30)]})
    return out


def box_count(lo, size, edge, ppc=2):
    """Particles add() emits for a box of `size` cells at cell `lo` of a grid of `edge` cells (size 1):
    the lattice extent floor((hi - lo) / spacing) per axis in f64, as the emitter computes it, every
    point kept (a box's inside test is always true)."""
    import math
    sp = (1.0 / edge) / ppc
    n = 1
    for x, d in zip(lo, size):
        n *= max(1, math.floor(((x + d) / edge - x / edge) / sp))
    return n


def plasticity_capacity(s):
    """maxParticles of a plasticity scene: exactly the particles its two blocks emit."""
    return sum(box_count(lo, d, s["edge"]) for _, lo, d in s["blocks"])


def fill_plasticity(sim, s):
    e = s["edge"]
    for (name, lo, size), seed in zip(s["blocks"], s["seeds"]):
        sim.add({"box": [[x / e for x in lo], [(x + d) / e for x, d in zip(lo, size)]]},
                material=material_def(name), seed=seed)
    return sim


def b_alg(sims):
    """Algorithmic bytes of one substep of these scenes: 256 B per particle + 32 B per node."""
    return sum(256 * s.count + 32 * s.numNodes for s in sims)


SVD_TOL = "snow and sand decompose F to a tolerance (si_world_set_svd_tolerance): particle x, v, C, F, J " \
          "within 1e-5 relative per substep of the bit-exact path, binning and grid sums exact"


def run_batched(a, log, svd_tol=True, tune=None):
    """256 scenes in one world: one launch per phase for all of them, CUDA graphs, autotuned; against
    the same scenes each stepped alone (the plain single-scene path) one after another."""
    from shaderintel_gb300 import MPM, World
    from shaderintel_gb300.autotune import autotune
    specs = scene_specs(a.batch_scenes, 4242)
    world = World()
    world.set_svd_tolerance(svd_tol)
    sims = [fill_scene(MPM(world, grid=s["edge"], maxParticles=spec_capacity(s), substeps=8), s) for s in specs]
    n_total = sum(s.count for s in sims)
    K = a.batch_substeps
    if tune is not None:
        world.set_tuning(tune["particles_per_cta"], tune["tile_nodes"], tune["flush"])
    elif a.no_autotune:
        tune = {"particles_per_cta": 256, "tile_nodes": 2048, "flush": 0, "autotuned": False}
    else:
        tune = autotune(world, substeps=4, repeats=2)
        log(f"batched: autotune chose {tune['particles_per_cta']}/{tune['tile_nodes']}/{tune['flush']}")
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))   # sampling before the warm-up
    for _ in range(a.warmup):
        world.step(K)
    world.sync()
    l0 = world.launches()
    clocks.start()
    world.mark(2)
    for _ in range(a.batch_steps):
        world.step(K)
    world.mark(3)
    ms = world.elapsed(2, 3)
    clk = clocks.stop()
    launches = world.launches() - l0
    value = n_total * K * a.batch_steps / (ms / 1e3)
    # the plain path: each scene alone, K substeps, scene after scene (warmed up the same way)
    for _ in range(2):
        for s in sims:
            s.step(dt=s.substepDt, K=K)
    world.mark(4)
    for s in sims:
        s.step(dt=s.substepDt, K=K)
    world.mark(5)
    plain_ms = world.elapsed(4, 5)
    plain = n_total * K / (plain_ms / 1e3)
    peak, peak_kind = load_peaks()
    bytes_substep = b_alg(sims)
    achieved = bytes_substep * K * a.batch_steps / (ms / 1e3) / 1e9
    out = {"workload": f"batched: {len(sims)} scenes, edge in {{16,32,48,64}}, N log-uniform 2k-260k capped by "
                       "8 ppc of the interior, water/jelly/snow/sand, random box placement (seed 4242), "
                       f"{K} substeps per step",
           "scenes": len(sims), "particles": n_total, "grid_nodes": sum(s.numNodes for s in sims),
           "substeps_per_step": K, "steps": a.batch_steps, "ms_per_step": ms / a.batch_steps,
           "value": value, "unit": "particle-substeps/s",
           "plain_value": plain, "plain_ms_per_step": plain_ms, "vs_plain": value / plain,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "peak_source": peak_kind, "algorithmic_bytes_per_substep": bytes_substep},
           "tuning": tune, "gpu_launches": launches, "clocks": clk,
           "svd": SVD_TOL if svd_tol else "bit-exact",
           "l2": f"inputs larger than L2 ({n_total * 128 / 1e6:.0f} MB particle state)"}
    world.destroy()
    return out


def run_served(a, log, scenes="batched"):
    """Continuous batching over up to `serve_resident` resident scenes drawn as the batched workload
    (`scenes="batched"`) or as the plasticity workload (`scenes="plasticity"`, about 1 M particles
    each, so the 150 GB budget is what limits residency): Poisson arrivals of step(dt, K) with K
    uniform in 1..32, admission by a 150 GB budget, scenes retired after 500 substeps and replaced
    by new ones. Arrivals stop after `serve_seconds`; every request issued is then waited for."""
    import collections
    import random
    from shaderintel_gb300 import SIError
    from shaderintel_gb300.serving import Server
    rng = random.Random(77)
    if scenes == "plasticity":
        spec_iter = iter(plasticity_specs(1 << 14, 5151))
        cap_of, fill_of = plasticity_capacity, fill_plasticity
        drawn = "the plasticity workload (96^3 grid, snow slab + sand column, 0.67-1.27 M particles)"
    else:
        spec_iter = iter(scene_specs(1 << 20, 9191))
        cap_of, fill_of = spec_capacity, fill_scene
        drawn = "the batched workload"
    srv = Server(budget_bytes=150 * 10 ** 9)
    srv.world.set_svd_tolerance(True)
    peak, _ = load_peaks()
    resident, given, size_of, outstanding = [], {}, {}, collections.defaultdict(list)
    retiring = []
    refused = admitted = retired = 0

    def admit_one():
        nonlocal refused, admitted
        s = next(spec_iter)
        try:
            sim = srv.admit(grid=s["edge"], maxParticles=cap_of(s), substeps=8)
        except SIError as e:
            if e.code != "out-of-memory":   # only a full budget is an admission refusal
                raise
            refused += 1
            return None
        fill_of(sim, s)
        admitted += 1
        # particles and algorithmic bytes per substep, read once: the properties take the world's
        # lock, which a round holds while it is enqueued
        size_of[sim] = (sim.count, 256 * sim.count + 32 * sim.numNodes)
        given[sim] = 0
        resident.append(sim)
        return sim

    for _ in range(a.serve_resident):
        admit_one()
    log(f"served ({scenes}): {len(resident)} resident scenes, {sum(s.count for s in resident)} particles, "
        f"{refused} refused by the budget")
    resident_particles = sum(size_of[s][0] for s in resident)
    issued = 0
    srv.stats(reset=True)
    # the client's own pauses would bunch the Poisson arrivals: no garbage collection while it runs
    import gc
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    next_t = t0
    n_sub = 0
    bytes_done = 0
    all_tickets = []
    while True:
        now = time.perf_counter()
        if now - t0 >= a.serve_seconds:
            break
        if now < next_t:
            time.sleep(min(next_t - now, 0.0005))
            continue
        next_t += rng.expovariate(a.serve_rate)
        sim = resident[rng.randrange(len(resident))]
        K = rng.randint(1, 32)
        t = srv.submit(sim, K=K)
        all_tickets.append(t)
        outstanding[sim].append(t)
        issued += 1
        given[sim] += K
        n_sub += K
        bytes_done += K * size_of[sim][1]
        if given[sim] >= 500:            # retire after 500 substeps: no more requests, then replace
            resident.remove(sim)
            retiring.append(sim)
            admit_one()
        for r in list(retiring):         # retire those whose last request has finished
            done, _ = srv.poll(outstanding[r][-1])
            if done:
                outstanding[r].pop()
                for tk in outstanding.pop(r):
                    srv.wait(tk, timeout_ms=60000)
                srv.retire(r)
                retiring.remove(r)
                retired += 1
    offered = n_sub * (resident_particles / max(1, len(resident))) / max(1e-9, time.perf_counter() - t0)
    gc.enable()
    for sim, tks in outstanding.items():
        for tk in tks:
            srv.wait(tk, timeout_ms=600000)
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.destroy()
    thr = st["particle_substeps"] / wall
    return {"workload": f"served: Poisson arrivals {a.serve_rate:g}/s for {a.serve_seconds:g} s over up to "
                        f"{a.serve_resident} resident scenes drawn as {drawn}, K uniform 1..32, "
                        "150 GB admission budget, retire after 500 substeps",
            "resident_scenes": len(resident), "resident_particles": resident_particles,
            "offered_particle_substeps_per_s": offered, "requests_issued": issued,
            "requests": st["requests_done"], "substeps": st["substeps_done"], "wall_s": wall,
            "value": thr, "unit": "particle-substeps/s", "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
            "mean_ms": st["mean_ms"], "max_ms": st["max_ms"], "busy_s": st["busy_s"],
            "admitted": admitted, "retired": retired, "refused": refused,
            "roofline": {"bound": "hbm", "achieved": bytes_done / wall / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": bytes_done / wall / 1e9 / peak},
            "resident_peak_bytes": st["resident_bytes"], "budget_bytes": st["budget_bytes"], "svd": SVD_TOL}


def run_conservation(substeps=200):
    """The correctness gates reported beside the throughput: the 32^3 dam break (32,768 particles)
    stepped `substeps` substeps through the same library; particle count and particle mass are
    exact, the grid's fixed-point mass after P2G is compared with the particles' mass, and the
    momentum sum and the energy (kinetic + gravitational, lattice units) are reported at the start
    and the end."""
    import numpy as np
    from shaderintel_gb300 import World
    world = World()
    sim = build_gpu("dam_break", world)
    rows = np.stack(sim._rows)
    g = sim.gravity[1] * sim.substepDt ** 2 / sim.dx            # cells / substep^2

    def state():
        P = sim.readParticles()
        m = rows[P.view(np.uint32)[:, 3] & 7, 1].astype(np.float64)
        v = P[:, 4:7].astype(np.float64)
        y = P[:, 1].astype(np.float64)
        sim.p2g()
        grid_mass = float(sim.readGrid()[:, 3].astype(np.int64).sum()) / 4194304.0
        return {"particles": len(P), "mass": float(m.sum()), "grid_mass": grid_mass,
                "momentum": (m[:, None] * v).sum(0).tolist(),
                "energy": float((0.5 * m * (v * v).sum(1)).sum() - (m * g * y).sum())}

    s0 = state()
    devs = [abs(s0["grid_mass"] / s0["mass"] - 1)]
    frames = substeps // sim.substeps
    for _ in range(frames):
        sim.step()
        devs.append(abs(state()["grid_mass"] / s0["mass"] - 1))
    s1 = state()
    world.destroy()
    return {"workload": CONFIGS["dam_break"]["desc"] + f", {frames * 8} substeps",
            "particles_start": s0["particles"], "particles_end": s1["particles"],
            "particle_mass": s0["mass"], "particle_mass_end": s1["mass"],
            "grid_mass_rel_dev_max": max(devs),
            "momentum_start": s0["momentum"], "momentum_end": s1["momentum"],
            "energy_start": s0["energy"], "energy_end": s1["energy"],
            "energy_drift_rel": (s1["energy"] - s0["energy"]) / abs(s0["energy"]) if s0["energy"] else None}


def run_extras():
    """Costs of the added rows on the mixed 128^3 scene: add() sampled on the device against the host
    sampler (wall time, same particles), and the coupling pass with 32 rigid bodies per substep."""
    import numpy as np
    from shaderintel_gb300 import MPM, World
    from shaderintel_gb300.mpm import body_record
    c = CONFIGS["mixed"]
    g = c["grid"]
    out = {}
    for label, host in (("device", False), ("host", True)):
        sim = MPM(None, grid=g, maxParticles=2300000, substeps=8)
        sim.add({"box": [[0.4, 0.4, 0.4], [0.41, 0.41, 0.41]]}, material="water")   # warm the path
        sim.clear()
        sim.sync()
        t = time.perf_counter()
        for name, lo, hi, vel in c["blocks"]:
            sim.add({"box": [[x / g for x in lo], [x / g for x in hi]]}, material=material_def(name), velocity=vel,
                    _host=host)
        sim.sync()
        el = time.perf_counter() - t
        out[f"add_{label}_ms"] = el * 1e3
        out["add_particles"] = sim.count
        sim.destroy()
    rng = np.random.default_rng(3)
    bodies = np.stack([body_record(rng.uniform(0.1, 0.9, 3), [rng.uniform(0.03, 0.08)] * 3,
                                   "sphere" if k % 2 else "box", quaternion=rng.normal(size=4),
                                   velocity=rng.uniform(-0.5, 0.5, 3), mass=1.0) for k in range(32)])
    times = {}
    for coupled in (False, True):
        w = World()
        sim = build_gpu("mixed", w)
        if coupled:
            sim.couple(bodies)
        for _ in range(3):
            sim.step()
        w.mark(0)
        for _ in range(10):
            sim.step()
        w.mark(1)
        times[coupled] = w.elapsed(0, 1) / (10 * c["substeps"])
        w.destroy()
    out["couple_bodies"] = 32
    out["substep_ms_uncoupled"] = times[False]
    out["substep_ms_coupled"] = times[True]
    out["couple_us_per_substep"] = (times[True] - times[False]) * 1e3
    return out


def traffic_per_launch(cfg):
    """DRAM bytes per k_g2p launch from the committed ncu summary, if one exists for this workload."""
    p = os.path.join(ROOT, "profiles", f"g2p_{cfg}_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("bytes_per_launch"):
            return float(line.split("=")[1])
    return None


METRIC = "MPM particle-substeps/s, plain single-scene form"
REF_BUDGET_S = 200.0   # the reference arm's timed CPU work stays within a few minutes


def run_config(c, n_p, nodes):
    """The workload's config dict, identical in both arms."""
    return {"workload": c["desc"], "particles": n_p, "grid_nodes": nodes, "substeps_per_step": c["substeps"],
            "sort_every": 4, "l2": f"inputs larger than L2 ({n_p * 128 / 1e6:.1f} MB particle state)"}


def run_reference(a):
    """The reference algorithm on the host cores (the oracle's C restatement, all threads) over the
    frames the GPU arm times: `warmup` frames, then `steps` frames of `substeps` substeps each. If
    that would take longer than REF_BUDGET_S, each step times a bounded sample of its frame's
    substeps (stated in `sample`); the metric is per substep either way."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import si_oracle as O
    c = CONFIGS[a.config]
    subs = c["substeps"]
    rec, mats, geo, grav, vol4, _ = build_cpu(a.config)
    n = len(rec)
    nodes = int(np.prod(geo["dims"]))
    threads = os.cpu_count() or 1
    cols = np.zeros((16, 12), np.float32)
    P, sc = rec, 0
    P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, a.warmup * subs, sc, threads=threads)
    t = time.perf_counter()
    P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, 1, sc, threads=threads)
    t1 = time.perf_counter() - t
    per_step = max(1, min(subs, int(REF_BUDGET_S / max(t1 * a.steps, 1e-9))))
    timed = 0.0
    for _ in range(a.steps):
        t = time.perf_counter()
        P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, per_step, sc, threads=threads)
        timed += time.perf_counter() - t
        if per_step < subs:   # skip the rest of the frame untimed, so each step starts on its own frame
            P, _, sc = O.substeps(P, geo["dims"], mats, cols, 0, grav, vol4, subs - per_step, sc, threads=threads)
    v = n * per_step * a.steps / timed
    frames = f"{a.steps} frames of {subs} substeps" if per_step == subs else \
        f"the first {per_step} of the {subs} substeps of each of {a.steps} frames"
    sample = (f"{frames} of the full {n}-particle scene after {a.warmup} warm-up frames (the frames the GPU "
              f"arm times; {timed:.1f} s timed, oracle/ C restatement, OpenMP {threads} threads). The "
              "reference's WGSL needs a browser WebGPU stack, unavailable on this box")
    return {
        "impl": "reference", "metric": METRIC,
        "value": v, "unit": "particle-substeps/s", "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": timed * 1e3 / a.steps * (subs / per_step), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice of the reference sampler)",
        "config": run_config(c, n, nodes),
        "cpu_baseline": {"value": v, "unit": "particle-substeps/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def with_summary(out):
    """The line with the headline of the batched/served metric placed early (right after the plain
    value), so that a reader of the line's first fields sees it: the batched value, its ratio to the
    same scenes stepped one by one, its roofline fraction, and served p50/p99 step latency."""
    summ = {}
    b = out.get("batched")
    if b:
        summ["batched_value"] = b["value"]
        summ["batched_vs_plain"] = b["vs_plain"]
        summ["batched_roofline_frac"] = b["roofline"]["frac"]
        if "bit_exact" in b:
            summ["batched_bit_exact_value"] = b["bit_exact"]["value"]
            summ["batched_bit_exact_vs_plain"] = b["bit_exact"]["vs_plain"]
            summ["batched_bit_exact_roofline_frac"] = b["bit_exact"]["roofline_frac"]
    sv = out.get("served")
    if sv:
        summ["served_value"] = sv["value"]
        summ["served_p50_ms"] = sv["p50_ms"]
        summ["served_p99_ms"] = sv["p99_ms"]
    ss = out.get("served_saturated")
    if ss:
        summ["served_saturated_value"] = ss["value"]
        if b:   # the plain aggregate of scenes drawn from the same distribution, stepped one by one
            summ["served_saturated_vs_plain"] = ss["value"] / b["plain_value"]
    spl = out.get("served_plasticity") or []
    if spl:
        summ["served_plasticity_resident_scenes"] = spl[0]["resident_scenes"]
        summ["served_plasticity_capacity"] = spl[0]["value"]
        if len(spl) > 1:   # the run at the rate the GPU sustains
            summ["served_plasticity_sustained_rate_per_s"] = spl[1].get("rate_per_s")
            summ["served_plasticity_sustained_p50_ms"] = spl[1]["p50_ms"]
            summ["served_plasticity_sustained_p99_ms"] = spl[1]["p99_ms"]
    head = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config")
    first = {k: out[k] for k in head if k in out}
    return {**first, **summ, **{k: v for k, v in out.items() if k not in first}}


def reduce_replicas(out, world_size, substeps):
    """Independent replicas (one scene per GPU, no device collective): the job's time per step is
    the maximum over ranks, its value the particle-substeps of all ranks over that time. Needs an
    initialised process group (gloo: host tensors only)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([out["ms_per_step"]], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out = dict(out)
    out["ms_per_step"] = float(t[0])
    out["value"] = out["config"]["particles"] * substeps * world_size / (float(t[0]) / 1e3)
    out["config"] = dict(out["config"], parallelism=f"replicas x{world_size}")
    return out


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", choices=list(CONFIGS), default="mixed")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-batched", action="store_true", help="skip the batched-form leg")
    p.add_argument("--batch-scenes", type=int, default=256)
    p.add_argument("--batch-substeps", type=int, default=100)
    p.add_argument("--batch-steps", type=int, default=3)
    p.add_argument("--no-served", action="store_true", help="skip the served-form leg")
    p.add_argument("--serve-seconds", type=float, default=10.0)
    p.add_argument("--serve-rate", type=float, default=2000.0)
    p.add_argument("--serve-resident", type=int, default=1000)
    p.add_argument("--no-served-plasticity", action="store_true",
                   help="skip the served leg over 1 M-particle plasticity scenes")
    p.add_argument("--serve-p-seconds", type=float, default=2.0,
                   help="arrival window of each served-plasticity run (every request is then waited for)")
    p.add_argument("--serve-p-rates", default="2000,sustain,200",
                   help="arrival rates (requests/s) of the served-plasticity runs; 'sustain' = 85 %% of the "
                        "capacity the previous run measured, in requests of mean K over the mean resident scene")
    p.add_argument("--only-batched", action="store_true",
                   help="run the batched leg alone (its line carries the batched metric), e.g. under a profiler")
    p.add_argument("--no-autotune", action="store_true", help="batched leg with the default tuning")
    a = p.parse_args()
    if a.warmup < 3:
        a.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    if world_size > 1 and "CUDA_VISIBLE_DEVICES" not in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", "0")
    if a.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(a)))
        return
    if a.only_batched:
        b = run_batched(a, lambda m: print(m, file=sys.stderr, flush=True))
        print(json.dumps({"metric": "MPM particle-substeps/s on 1 GB300 (batched form)", "value": b["value"],
                          "unit": "particle-substeps/s", "n_gpus": 1, "steps": a.batch_steps, "warmup": a.warmup,
                          "ms_per_step": b["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                          "vs_baseline": None, "dtype": "f32", "data": "synthetic", "batched": b}))
        return
    out = run_ours(a, rank)
    log = lambda m: print(m, file=sys.stderr, flush=True)   # noqa: E731
    if world_size == 1 and not a.no_batched:
        out["batched"] = run_batched(a, log)
        # the same leg with every field bit-identical to the CPU restatement, beside it
        ex = run_batched(a, log, svd_tol=False, tune=out["batched"]["tuning"])
        out["batched"]["bit_exact"] = {k: ex[k] for k in ("value", "plain_value", "vs_plain", "ms_per_step")}
        out["batched"]["bit_exact"]["roofline_frac"] = ex["roofline"]["frac"]
    if world_size == 1 and not a.no_served:
        out["served"] = run_served(a, log)
        # the same loop offered more than it can run: its capacity (latency is then queueing)
        import types
        sat = types.SimpleNamespace(serve_rate=max(8000.0, 4 * a.serve_rate), serve_seconds=min(5.0, a.serve_seconds),
                                    serve_resident=a.serve_resident)
        out["served_saturated"] = run_served(sat, log)
    if world_size == 1 and not a.no_served and not a.no_served_plasticity:
        import types
        out["served_plasticity"] = []
        for tok in (x for x in a.serve_p_rates.split(",") if x):
            if tok == "sustain":
                prev = out["served_plasticity"][-1] if out["served_plasticity"] else None
                if not prev:
                    continue
                per_request = 16.5 * prev["resident_particles"] / max(1, prev["resident_scenes"])   # K uniform 1..32
                rate = round(0.85 * prev["value"] / per_request)
            else:
                rate = float(tok)
            sp = types.SimpleNamespace(serve_rate=rate, serve_seconds=a.serve_p_seconds, serve_resident=1000)
            out["served_plasticity"].append(run_served(sp, log, scenes="plasticity"))
            out["served_plasticity"][-1]["rate_per_s"] = rate
    if world_size == 1:
        out["conservation"] = run_conservation()
        out["extras"] = run_extras()
    out = with_summary(out)
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        out = reduce_replicas(out, world_size, CONFIGS[a.config]["substeps"])
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
