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
the public API with host buffers: every frame uploads the 16-row collider table the reference
uploads each step and reads every particle position back into pinned host memory.

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
        ("snow", [3, 3, 3], [93, 15, 45], [0, 0, 0]),
        ("sand30", [20, 3, 55], [70, 40, 80], [0, 0, 0])],
        "desc": "plasticity_96: 96^3 grid, snow slab + Drucker-Prager sand column (friction 30 deg), 8 ppc"},
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
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.idx = gpu_index
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


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
    for _ in range(a.warmup):
        sim.step()
    world.sync()
    l0 = world.launches()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
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

    # end to end through the public API with host buffers
    xyz, pinned = pinned_floats(n_p * 3)
    cols, _ = pinned_floats(16 * 12)
    cols[:] = 0
    h = sim._h
    t = time.perf_counter()
    for _ in range(a.steps):
        lib.si_mpm_set_colliders(h, L.fptr(cols), 0)   # the per-step collider table upload (mpm.js:586)
        L.check(lib.si_mpm_step(h, 0.0, 0))
        L.check(lib.si_mpm_read_positions(h, L.fptr(xyz), 0, n_p))
    e2e_s = time.perf_counter() - t
    e2e = n_p * subs * a.steps / e2e_s

    out = {
        "metric": "MPM particle-substeps/s on 1 GB300 (plain single-scene form)",
        "value": value, "unit": "particle-substeps/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded jittered lattice of the reference sampler)",
        "config": {"workload": c["desc"], "particles": n_p, "grid_nodes": nodes, "substeps_per_step": subs,
                   "sort_every": 4, "l2": f"inputs larger than L2 ({n_p * 128 / 1e6:.1f} MB particle state)",
                   "parallelism": "replicas" if a.gpus > 1 else "single"},
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


def traffic_per_launch(cfg):
    """DRAM bytes per k_g2p launch from the committed ncu summary, if one exists for this workload."""
    p = os.path.join(ROOT, "profiles", f"g2p_{cfg}_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("bytes_per_launch"):
            return float(line.split("=")[1])
    return None


def run_reference(a):
    v, st, th, n, el = cpu_measure(a.config, 0, steps=a.steps, warmup=a.warmup)
    c = CONFIGS[a.config]
    return {
        "impl": "reference", "metric": "MPM particle-substeps/s on 1 GB300 (plain single-scene form)",
        "value": v, "unit": "particle-substeps/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": el * 1e3 / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded jittered lattice of the reference sampler)",
        "config": {"workload": c["desc"], "particles": n, "substeps_per_step": 1},
        "cpu_baseline": {"value": v, "unit": "particle-substeps/s", "cores": th, "kind": "port",
                         "sample": f"{st} substeps (one per step) of the full {n}-particle scene after {a.warmup} "
                                   "warm-up substeps; the reference's WGSL needs a browser WebGPU stack, so its "
                                   "CPU restatement (oracle/) runs instead"},
        "e2e": {"value": v, "unit": "particle-substeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", choices=list(CONFIGS), default="mixed")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
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
    out = run_ours(a, rank)
    if world_size > 1:   # independent replicas: the job value is the sum, the time the max over ranks
        import torch.distributed as dist
        dist.init_process_group("gloo")
        import torch
        t = torch.tensor([out["ms_per_step"]], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        out["ms_per_step"] = float(t[0])
        out["value"] = out["config"]["particles"] * CONFIGS[a.config]["substeps"] * world_size / (t[0].item() / 1e3)
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
