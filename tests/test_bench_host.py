"""Host-side parts of bench.py, on CPU: the reference arm's JSON line (the CPU restatement timed on
the host cores, as `bench.py --impl reference` prints it) and the seeded workload generators of
the batched and served legs (every block inside the walls, snow and sand apart, capacity enough
for the emitted lattice)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
                        "dam_break", "--steps", "2", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and "GB300" not in d["metric"] and "n_gpus" not in d
    assert d["unit"] == "particle-substeps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert d["config"]["particles"] == 32768
    # the GPU arm's config dict, key for key: the same workload and the same frames
    assert d["config"] == bench.run_config(bench.CONFIGS["dam_break"], 32768, 32 ** 3)
    assert d["config"]["substeps_per_step"] == 8 and d["config"]["sort_every"] == 4
    assert "2 frames of 8 substeps" in cb["sample"] and "after 3 warm-up frames" in cb["sample"]


def test_summary_keys_come_first():
    out = {"metric": "m", "value": 1.0, "unit": "u", "n_gpus": 1, "config": {}, "roofline": {},
           "batched": {"value": 6.0, "vs_plain": 5.0, "plain_value": 1.2, "roofline": {"frac": 0.3}},
           "served": {"value": 2.0, "p50_ms": 1.0, "p99_ms": 4.0}, "served_saturated": {"value": 4.8}}
    s = bench.with_summary(out)
    keys = list(s)
    assert keys.index("batched_value") < keys.index("roofline") < keys.index("batched")
    assert s["batched_vs_plain"] == 5.0 and s["served_p99_ms"] == 4.0
    assert abs(s["served_saturated_vs_plain"] - 4.0) < 1e-12


def _cells(lo, size):
    return [(lo[a], lo[a] + size[a]) for a in range(3)]


def test_batched_scene_draws_stay_inside_the_walls():
    specs = bench.scene_specs(512, 4242)
    assert specs == bench.scene_specs(512, 4242)          # seeded
    for s in specs:
        e = s["edge"]
        assert e in bench.BATCH_EDGES and s["material"] in bench.BATCH_MATERIALS
        for lo, hi in _cells(s["lo"], s["size"]):
            assert 3 <= lo < hi <= e - 3                   # bound = 3 cells (mpm.js:103)
        n = 8 * s["size"][0] * s["size"][1] * s["size"][2]
        assert 0 < n <= bench.spec_capacity(s)


def test_plasticity_scene_draws_match_the_workload():
    specs = bench.plasticity_specs(2000, 5151)
    assert specs == bench.plasticity_specs(2000, 5151)
    counts = []
    for s in specs:
        assert s["edge"] == 96
        (m0, lo0, d0), (m1, lo1, d1) = s["blocks"]
        assert (m0, m1) == ("snow", "sand30")
        box0, box1 = _cells(lo0, d0), _cells(lo1, d1)
        for lo, hi in box0 + box1:
            assert 3 <= lo < hi <= 93
        assert box0[1][0] == 3 and box1[1][0] == 3       # both on the floor
        assert box0[2][1] < box1[2][0]                    # the slab and the column do not overlap (z)
        n = 8 * (d0[0] * d0[1] * d0[2] + d1[0] * d1[1] * d1[2])
        assert n - 8 * 100 ** 2 <= bench.plasticity_capacity(s) <= n   # the lattice, to within its edge rounding
        counts.append(n)
    assert 0.6e6 < min(counts) and max(counts) < 1.3e6
    assert 0.85e6 < sum(counts) / len(counts) < 1.05e6   # about 1 M particles, as the workload asks


def test_plasticity_capacity_is_the_emitted_count():
    """The served plasticity scenes are sized to exactly the particles add() emits for their boxes:
    the library's host sampler (si_sample_shape, the reference's sampleShape restated) counts them."""
    import ctypes
    from shaderintel_gb300 import _lib as L
    for s in bench.plasticity_specs(3, 5151):
        e = s["edge"]
        total = 0
        for (name, lo, d), seed in zip(s["blocks"], s["seeds"]):
            a = L.dptr([x / e for x in lo])
            b = L.dptr([(x + k) / e for x, k in zip(lo, d)])
            n = ctypes.c_int64()
            L.check(L.lib().si_sample_shape(0, a, b, 0.0, 0.0, (1.0 / e) / 2, 0.6, seed, None, 0, ctypes.byref(n)))
            assert n.value == bench.box_count(lo, d, e)
            total += n.value
        assert total == bench.plasticity_capacity(s)
