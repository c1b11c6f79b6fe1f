"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE: used only by tests/, the smoke check and
the CPU-baseline leg of bench.py, as the checker — never by the product path)."""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libsi_oracle.so")
_L = None

f_p = ctypes.POINTER(ctypes.c_float)
i32_p = ctypes.POINTER(ctypes.c_int32)
u32_p = ctypes.POINTER(ctypes.c_uint32)
i64_p = ctypes.POINTER(ctypes.c_int64)


class CoupleParams(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_float * 3), ("dx", ctypes.c_float), ("inv_dx", ctypes.c_float),
                ("lead", ctypes.c_float), ("vel_to_lattice", ctypes.c_float), ("friction", ctypes.c_float),
                ("band", ctypes.c_float), ("mask", ctypes.c_uint32)]


class Params(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int32 * 3), ("num_blocks", ctypes.c_uint32), ("gravity", ctypes.c_float * 3),
                ("bound", ctypes.c_float), ("floor_friction", ctypes.c_float), ("vmax", ctypes.c_float),
                ("vol4", ctypes.c_float), ("sort_every", ctypes.c_int32), ("ncol", ctypes.c_int32),
                ("mats", f_p), ("cols", f_p), ("bodies", f_p), ("nbodies", ctypes.c_int32),
                ("couple", CoupleParams), ("substep_dt", ctypes.c_double), ("body_acc", i32_p)]


def lib():
    global _L
    if _L is None:
        src = os.path.join(HERE, "si_oracle.c")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", HERE], check=True)
        L = ctypes.CDLL(LIB)
        L.sio_morton3.restype = ctypes.c_uint32
        L.sio_morton3.argtypes = [ctypes.c_uint32] * 3
        L.sio_num_blocks.restype = ctypes.c_uint32
        L.sio_num_blocks.argtypes = [i32_p]
        L.sio_keys.argtypes = [f_p, ctypes.c_int64, ctypes.c_uint32, u32_p]
        L.sio_bins.argtypes = [u32_p, ctypes.c_int64, ctypes.c_uint32, u32_p]
        L.sio_sort.argtypes = [f_p, f_p, ctypes.c_int64, ctypes.c_uint32, u32_p, u32_p, u32_p]
        L.sio_p2g.argtypes = [f_p, ctypes.c_int64, i32_p, f_p, ctypes.c_float, i32_p, ctypes.c_int]
        L.sio_grid_update.argtypes = [i32_p, i32_p, f_p, ctypes.c_float, f_p, ctypes.c_int, ctypes.c_float,
                                      ctypes.c_int]
        L.sio_g2p.argtypes = [f_p, ctypes.c_int64, i32_p, i32_p, f_p, ctypes.c_float, ctypes.c_float, ctypes.c_int]
        L.sio_retime.argtypes = [f_p, ctypes.c_int64, ctypes.c_float]
        L.sio_substeps.argtypes = [f_p, f_p, ctypes.c_int64, i32_p, ctypes.POINTER(Params), i64_p, ctypes.c_int,
                                   ctypes.c_int]
        L.sio_logf.restype = ctypes.c_float
        L.sio_logf.argtypes = [ctypes.c_float]
        L.sio_expf.restype = ctypes.c_float
        L.sio_expf.argtypes = [ctypes.c_float]
        L.sio_svd3.argtypes = [f_p, f_p, f_p, f_p]
        L.sio_couple.argtypes = [i32_p, i32_p, f_p, ctypes.c_int32, ctypes.POINTER(CoupleParams), i32_p]
        L.sio_couple_apply.argtypes = [i32_p, f_p, ctypes.c_int32, ctypes.c_float, ctypes.c_float]
        d3 = ctypes.POINTER(ctypes.c_double)
        L.sio_emit_box.restype = ctypes.c_int64
        L.sio_emit_box.argtypes = [d3, d3, ctypes.c_double, ctypes.c_double, ctypes.c_uint32, ctypes.c_uint32, d3,
                                   i32_p, ctypes.c_double, d3, ctypes.c_double, f_p, ctypes.c_int64]
        _L = L
    return _L


def _f(a):
    return a.ctypes.data_as(f_p)


def _i(a):
    return a.ctypes.data_as(i32_p)


def _u(a):
    return a.ctypes.data_as(u32_p)


def emit_box(lo, hi, spacing, jitter, seed, material, vel, dims, dx, origin, substep_dt):
    """Records of add({box}) (sampleShape + conversion, mpm.js:683-714, 213-227)."""
    D = lambda v: (ctypes.c_double * 3)(*[float(x) for x in v])  # noqa: E731
    args = [D(lo), D(hi), spacing, jitter, seed, material, D(vel), _i(dims_arr(dims)), dx, D(origin), substep_dt]
    n = lib().sio_emit_box(*args, None, 0)
    out = np.empty((n, 32), np.float32)
    lib().sio_emit_box(*args, _f(out), n)
    return out


def dims_arr(dims):
    return np.ascontiguousarray(dims, np.int32)


def num_blocks(dims):
    return int(lib().sio_num_blocks(_i(dims_arr(dims))))


def keys(P, nb):
    P = np.ascontiguousarray(P, np.float32)
    out = np.empty(len(P), np.uint32)
    lib().sio_keys(_f(P), len(P), nb, _u(out))
    return out


def sort(P, nb):
    """Stable block sort: returns (sorted records, keys (pre-sort order), starts, perm)."""
    P = np.ascontiguousarray(P, np.float32)
    n = len(P)
    dst = np.empty_like(P)
    k = np.empty(n, np.uint32)
    st = np.empty(nb + 1, np.uint32)
    perm = np.empty(n, np.uint32)
    lib().sio_sort(_f(P), _f(dst), n, nb, _u(k), _u(st), _u(perm))
    return dst, k, st, perm


def p2g(P, dims, mats, vol4, threads=1):
    P = np.ascontiguousarray(P, np.float32)
    d = dims_arr(dims)
    grid = np.empty((int(np.prod(dims)), 4), np.int32)
    lib().sio_p2g(_f(P), len(P), _i(d), _f(np.ascontiguousarray(mats, np.float32)), vol4, _i(grid), threads)
    return grid


def grid_update(grid, dims, gravity, cols, ncol, bound=3.0, floor_friction=0.4, threads=1):
    g = np.array(grid, np.int32, copy=True)
    lib().sio_grid_update(_i(g), _i(dims_arr(dims)), _f(np.ascontiguousarray(gravity, np.float32)), bound,
                          _f(np.ascontiguousarray(cols, np.float32)), ncol, floor_friction, threads)
    return g


def g2p(P, dims, grid, mats, bound=3.0, vmax=0.9, threads=1):
    P = np.array(P, np.float32, copy=True)
    lib().sio_g2p(_f(P), len(P), _i(dims_arr(dims)), _i(np.ascontiguousarray(grid, np.int32)),
                  _f(np.ascontiguousarray(mats, np.float32)), bound, vmax, threads)
    return P


def retime(P, k):
    P = np.array(P, np.float32, copy=True)
    lib().sio_retime(_f(P), len(P), k)
    return P


def substeps(P, dims, mats, cols, ncol, gravity, vol4, K, step_count=0, sort_every=4, threads=1,
             bound=3.0, floor_friction=0.4, vmax=0.9, coupling=None):
    """K substeps of mpm.js:590-602 on records P; returns (P, grid i32 words, step_count)."""
    P = np.array(P, np.float32, copy=True)
    scratch = np.empty_like(P)
    grid = np.empty((int(np.prod(dims)), 4), np.int32)
    mats = np.ascontiguousarray(mats, np.float32)
    cols = np.ascontiguousarray(cols, np.float32)
    prm = Params()
    for a in range(3):
        prm.dims[a] = int(dims[a])
        prm.gravity[a] = float(gravity[a])
    prm.num_blocks = num_blocks(dims)
    prm.bound, prm.floor_friction, prm.vmax, prm.vol4 = bound, floor_friction, vmax, vol4
    prm.sort_every, prm.ncol = sort_every, ncol
    prm.mats, prm.cols = _f(mats), _f(cols)
    keep = []
    if coupling is not None:   # dict(bodies, params (9 floats: origin xyz dx inv_dx - vel friction band), mask, dt, acc)
        b = np.ascontiguousarray(coupling["bodies"], np.float32).reshape(-1, 48)
        acc = coupling["acc"]
        keep += [b, acc]
        prm.bodies, prm.nbodies, prm.body_acc = _f(b), len(b), _i(acc)
        q = coupling["params"]
        for k in range(3):
            prm.couple.origin[k] = float(q[k])
        prm.couple.dx, prm.couple.inv_dx, _, prm.couple.vel_to_lattice, prm.couple.friction, prm.couple.band = \
            [float(x) for x in q[3:9]]
        prm.couple.mask = int(coupling["mask"])
        prm.substep_dt = float(coupling["dt"])
    sc = ctypes.c_int64(step_count)
    lib().sio_substeps(_f(P), _f(scratch), len(P), _i(grid), ctypes.byref(prm), ctypes.byref(sc), K, threads)
    return P, grid, sc.value


def couple(grid, dims, bodies, params, mask):
    """The coupling pass of one substep (coupling.js:83-186) on a grid of vec4f(v, m) bits.
    params: origin xyz, dx, inv_dx, lead, vel_to_lattice, friction, band. Returns (grid, acc)."""
    g = np.array(grid, np.int32, copy=True)
    b = np.ascontiguousarray(bodies, np.float32).reshape(-1, 48)
    acc = np.zeros(len(b) * 8, np.int32)
    cp = CoupleParams()
    for k in range(3):
        cp.origin[k] = float(params[k])
    cp.dx, cp.inv_dx, cp.lead, cp.vel_to_lattice, cp.friction, cp.band = [float(x) for x in params[3:9]]
    cp.mask = int(mask)
    lib().sio_couple(_i(g), _i(dims_arr(dims)), _f(b), len(b), ctypes.byref(cp), _i(acc))
    return g, acc


def couple_apply(acc, n, mom_to_world, dx):
    """mpm-rigid-apply (coupling.js:188-196): world impulses (n x 8) from the fixed-point sums."""
    a = np.array(acc, np.int32, copy=True)
    ext = np.zeros(n * 8, np.float32)
    lib().sio_couple_apply(_i(a), _f(ext), n, mom_to_world, dx)
    return ext.reshape(n, 8), a
