"""CPU tests of the oracle itself: its math against float64, the reference's invariants
(tests/physics.test.js:6-59, src/verify/index.js:19-62,175-191, tests/core.test.js:72-110) and
its determinism. No GPU."""
import numpy as np
import pytest

import host_ref
import si_oracle as O
from conftest import mulberry32


def _ulps(got, ref):
    ref32 = np.float32(ref)
    return np.abs(got.astype(np.float64) - ref) / np.spacing(np.abs(ref32)).astype(np.float64)


def test_log_exp_within_2_ulp():
    L = O.lib()
    rng = np.random.default_rng(7)
    xs = np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 20000)).astype(np.float32)
    xs = np.concatenate([xs, np.float32([1.0, 0.05, 1e-4, 0.6, 20.0])])
    got = np.array([L.sio_logf(float(x)) for x in xs], np.float32)
    assert _ulps(got, np.log(xs.astype(np.float64))).max() <= 2.0
    ys = rng.uniform(-87, 88, 20000).astype(np.float32)
    got = np.array([L.sio_expf(float(y)) for y in ys], np.float32)
    assert _ulps(got, np.exp(ys.astype(np.float64))).max() <= 2.0
    assert L.sio_expf(-200.0) == 0.0 and np.isinf(L.sio_expf(100.0))


def test_svd3_reconstructs():
    rng = np.random.default_rng(3)
    for _ in range(200):
        F = (np.eye(3) + rng.normal(0, 0.3, (3, 3))).astype(np.float32)
        Fc = np.ascontiguousarray(F.T)   # column-major
        U = np.empty(9, np.float32); s = np.empty(3, np.float32); V = np.empty(9, np.float32)
        O.lib().sio_svd3(O._f(Fc.ravel()), O._f(U), O._f(s), O._f(V))
        Um, Vm = U.reshape(3, 3).T, V.reshape(3, 3).T
        rec = Um @ np.diag(s) @ Vm.T
        assert np.abs(rec - F).max() < 2e-4 * max(1.0, np.abs(F).max())
        assert abs(np.linalg.det(Um) - 1) < 1e-4 and abs(np.linalg.det(Vm) - 1) < 1e-4
        assert s[0] >= s[1] >= abs(s[2]) - 1e-6


def _water_block(grid=48, lo=(0.2, 0.2, 0.2), hi=(0.7, 0.6, 0.7), seed=None):
    g = host_ref.geometry(grid)
    pts = host_ref.sample_shape({"box": [list(lo), list(hi)]}, g["dx"] / 2, 0.6, 1 if seed is None else seed)
    dt = 1 / 60 / 4
    rec = host_ref.make_records(pts, 0, [0, 0, 0], g["dims"], g["dx"], [0, 0, 0], dt)
    mats = np.zeros((8, 12), np.float32)
    mats[0] = host_ref.material_row({"kind": 0, "density": 1, "stiffness": 1.0, "viscosity": 0.0})
    return g, rec, mats


def _randomise(rec, seed=3):
    """Random v, C and tau as in tests/physics.test.js:10-17 (mulberry32)."""
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


def test_p2g_conserves_mass_and_momentum():
    """tests/physics.test.js:6-32 on the oracle (small box)."""
    g, rec, mats = _water_block(grid=24, lo=(0.3, 0.3, 0.3), hi=(0.6, 0.55, 0.6))
    rec = _randomise(rec)
    grid = O.p2g(rec, g["dims"], mats, 4 / 8)
    FP = 2.0 ** 22
    mass = 1 / 8
    gm = grid[:, 3].astype(np.int64).sum() / FP
    gp = grid[:, :3].astype(np.int64).sum(0) / FP
    pm = mass * len(rec)
    pp = mass * rec[:, 4:7].astype(np.float64).sum(0)
    assert abs(gm - pm) / pm < 1e-4
    assert np.abs(gp - pp).max() < 1e-3 * max(1, np.linalg.norm(pp)) + len(rec) * 27 * 4 / FP


def test_p2g_order_independent():
    """The fixed-point grid is the same for any particle order (bench/suite.js:284-290)."""
    g, rec, mats = _water_block(grid=24, lo=(0.3, 0.3, 0.3), hi=(0.6, 0.5, 0.6))
    rec = _randomise(rec, 5)
    a = O.p2g(rec, g["dims"], mats, 0.5)
    perm = np.random.default_rng(11).permutation(len(rec))
    b = O.p2g(rec[perm], g["dims"], mats, 0.5, threads=4)
    assert np.array_equal(a, b)


def test_sort_certificates():
    """checkSorted / checkPermutation / checkScan of src/verify/index.js:19-62 on the oracle sort."""
    g, rec, _ = _water_block(grid=32)
    rng = np.random.default_rng(2)
    rec = rec[rng.permutation(len(rec))]
    nb = O.num_blocks(g["dims"])
    assert nb == g["num_blocks"]
    dst, keys, starts, perm = O.sort(rec, nb)
    skeys = O.keys(dst, nb)
    assert np.all(skeys[:-1] <= skeys[1:])                      # sorted
    assert np.array_equal(np.sort(perm), np.arange(len(rec)))   # a permutation
    counts = np.bincount(keys, minlength=nb + 1)
    assert starts[0] == 0 and np.array_equal(np.diff(starts.astype(np.int64)), counts[:nb])
    assert starts[nb] == len(rec)
    for k in np.unique(keys):                                    # stable inside each block
        seg = perm[starts[k]:starts[k + 1]]
        assert np.all(seg[:-1] < seg[1:])


@pytest.mark.parametrize("n", [0, 1, 3, 17, 4097])
def test_bins_edge_sizes(n):
    """Exclusive-scan semantics of the block counts for ragged sizes (tests/core.test.js:72-110)."""
    rng = np.random.default_rng(n)
    rec = np.zeros((n, 32), np.float32)
    rec[:, :3] = rng.uniform(3, 29, (n, 3))
    nb = O.num_blocks([32, 32, 32])
    keys = O.keys(rec, nb)
    starts = np.empty(nb + 1, np.uint32)
    O.lib().sio_bins(O._u(keys), n, nb, O._u(starts))
    ref = np.concatenate([[0], np.cumsum(np.bincount(keys, minlength=nb))]).astype(np.uint32)
    assert np.array_equal(starts, ref)


def test_dam_break_stable_and_volume():
    """tests/physics.test.js:43-59 on the oracle, scaled down (24^3, 40 frames)."""
    g = host_ref.geometry(24)
    dt = 1 / 60 / 8
    pw = host_ref.sample_shape({"box": [[0.05, 0.05, 0.05], [0.4, 0.6, 0.95]]}, g["dx"] / 2, 0.6, 1)
    pj = host_ref.sample_shape({"sphere": [[0.7, 0.4, 0.5], 0.12]}, g["dx"] / 2, 0.6, len(pw) + 1)
    rec = np.concatenate([host_ref.make_records(pw, 0, [0, 0, 0], g["dims"], g["dx"], [0, 0, 0], dt),
                          host_ref.make_records(pj, 1, [0, 0, 0], g["dims"], g["dx"], [0, 0, 0], dt)])
    mats = np.zeros((8, 12), np.float32)
    mats[0] = host_ref.material_row({"kind": 0, "density": 1, "stiffness": 1.0, "viscosity": 0.0})
    mats[1] = host_ref.material_row({"kind": 1, "density": 1, "stiffness": 0.35, "poisson": 0.3})
    grav = [np.float32(-9.81 * dt * dt / g["dx"]) * (a == 1) for a in range(3)]
    P, _, sc = O.substeps(rec, g["dims"], mats, np.zeros((16, 12), np.float32), 0, grav, 0.5, 320, threads=8)
    assert sc == 320
    x = P[:, :3]
    assert np.isfinite(x).all()
    assert ((x >= 1) & (x <= np.array(g["dims"]) - 1)).all()
    water = P.view(np.uint32)[:, 3] == 0
    assert abs(P[water, 7].mean() - 1) < 0.05
