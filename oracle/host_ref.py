"""Pure-Python restatement of the reference's host-side JavaScript (TEST INFRASTRUCTURE).

Python floats are IEEE doubles like JavaScript Numbers, and np.float32(x) rounds to nearest even
like a Float32Array store, so these functions give the bits the reference would upload:
  _uploadMaterials row ..... src/physics/mpm.js:170-199 (with the checks of _material, :148-168)
  sampleShape .............. mpm.js:683-714 (xorshift32: rnd ^= rnd<<13; ^= rnd>>>17; ^= rnd<<5)
  add() records ............ mpm.js:213-227
  _uploadColliders row ..... mpm.js:276-293
  constructor geometry ..... mpm.js:91-121
Used to check libsi_cuda's C++ host helpers bit for bit; never used by the product.
"""
import math

import numpy as np

C_MAX = 0.4


def js_round(x):
    f = math.floor(x)
    return f + 1 if x - f >= 0.5 else f


def geometry(grid=64, size=1, max_particles=262144):
    size = list(size) if isinstance(size, (list, tuple)) else [size] * 3
    dx = max(size) / grid
    dims = [max(8, js_round(s / dx)) for s in size]
    bmax = max(math.ceil(d / 4) for d in dims)
    bpow = 1 << math.ceil(math.log2(bmax))
    return {"dx": dx, "dims": dims, "num_blocks": bpow ** 3}


def material_row(m, ppc_axis=2):
    """mpm.js:174-195 for one material dict (keys as in MATERIALS; missing = JavaScript default)."""
    kind = m["kind"]
    density = m.get("density", 1)
    if kind not in (0, 1, 2, 3):
        raise ValueError("kind")
    if not (density > 0 and density <= 50):
        raise ValueError("density")
    vol = 1 / ppc_axis ** 3
    mass = density * vol
    rho = mass / vol
    c = C_MAX * min(1, max(0.01, m.get("stiffness", 1)))
    nu = min(0.49, max(0, m.get("poisson", 0.3)))
    Mmod = rho * c * c
    mu = Mmod * (1 - 2 * nu) / (2 * (1 - nu))
    la = Mmod * nu / (1 - nu)
    row = np.zeros(12, np.float32)
    row.view(np.uint32)[0] = kind
    row[1] = np.float32(mass)
    row[2] = np.float32(rho * c * c if kind == 0 else mu)
    row[3] = np.float32(la)
    row[4] = np.float32(min(4, max(0, m.get("viscosity", 0))) * 0.05 * rho)
    row[5] = np.float32(m.get("hardening", 10))
    row[6] = np.float32(m.get("compression", 0.025))
    row[7] = np.float32(m.get("stretch", 0.0075))
    phi = (m.get("friction", 33) * math.pi) / 180
    sinp = math.sin(phi)
    row[8] = np.float32(math.sqrt(2 / 3) * (2 * sinp) / (3 - sinp))
    return row


def sample_shape(shape, spacing, jitter, seed):
    rnd = (int(seed) & 0xFFFFFFFF) or 1

    def rand():
        nonlocal rnd
        rnd ^= (rnd << 13) & 0xFFFFFFFF
        rnd ^= rnd >> 17
        rnd ^= (rnd << 5) & 0xFFFFFFFF
        return rnd / 4294967296

    if "box" in shape:
        lo, hi = shape["box"]
        inside = lambda p: True  # noqa: E731
    elif "sphere" in shape:
        c, r = shape["sphere"]
        lo = [x - r for x in c]
        hi = [x + r for x in c]
        inside = lambda p: (p[0] - c[0]) ** 2 + (p[1] - c[1]) ** 2 + (p[2] - c[2]) ** 2 <= r * r  # noqa: E731
    elif "cylinder" in shape:
        c, r, h = shape["cylinder"]
        lo = [c[0] - r, c[1] - h, c[2] - r]
        hi = [c[0] + r, c[1] + h, c[2] + r]
        inside = lambda p: (p[0] - c[0]) ** 2 + (p[2] - c[2]) ** 2 <= r * r  # noqa: E731
    else:
        raise ValueError("shape")
    n = [max(1, math.floor((hi[a] - lo[a]) / spacing)) for a in range(3)]
    out = []
    for z in range(n[2]):
        for y in range(n[1]):
            for x in range(n[0]):
                p = [lo[0] + (x + 0.5 + (rand() - 0.5) * jitter) * spacing,
                     lo[1] + (y + 0.5 + (rand() - 0.5) * jitter) * spacing,
                     lo[2] + (z + 0.5 + (rand() - 0.5) * jitter) * spacing]
                if inside(p):
                    out.extend(p)
    return np.asarray(out, np.float32).reshape(-1, 3)


def js_max(a, b):
    return math.nan if (a != a or b != b) else max(a, b)


def js_min(a, b):
    return math.nan if (a != a or b != b) else min(a, b)


def make_records(pts, mat, velocity, dims, dx, origin, substep_dt, bound=3):
    n = len(pts)
    data = np.zeros((n, 32), np.float32)
    s = substep_dt / dx
    lo = bound
    for k in range(n):
        for a in range(3):
            x = (float(pts[k][a]) - origin[a]) / dx
            data[k, a] = np.float32(js_min(dims[a] - bound - 1e-3, js_max(lo + 1e-3, x)))
        data[k].view(np.uint32)[3] = mat
        for a in range(3):
            data[k, 4 + a] = np.float32(velocity[a] * s)
        data[k, 7] = 1
        data[k, 20] = data[k, 25] = data[k, 30] = 1
    return data


def collider_row(c, dx, origin, substep_dt):
    row = np.zeros(12, np.float32)
    s = substep_dt / dx
    t = c.get("type", "sphere")
    row.view(np.uint32)[0] = {"sphere": 0, "box": 1, "plane": 2}[t]
    ctr = c.get("center", [0, 0, 0])
    for a in range(3):
        row[1 + a] = np.float32((ctr[a] - origin[a]) / dx)
    if t == "plane":
        nrm = c.get("normal", [0, 1, 0])
        row[4:7] = np.float32(nrm)
    elif t == "box":
        h = c.get("half", [0.1, 0.1, 0.1])
        for a in range(3):
            row[4 + a] = np.float32(h[a] / dx)
    else:
        row[4] = np.float32(c.get("radius", 0.1) / dx)
    row[7] = np.float32(c.get("friction", 0.3))
    v = c.get("velocity", [0, 0, 0])
    for a in range(3):
        row[8 + a] = np.float32(v[a] * s)
    return row


def spatial_grid(pos, origin, cell_size, dims):
    """SpatialGrid.build of src/prims/grid.js:14-20, 69-76 in numpy (f32 cell arithmetic): cells,
    order (stable: index order within a cell) and start (numCells + 1)."""
    p = np.asarray(pos, np.float32)[:, :3]
    o = np.asarray(origin, np.float32)
    inv = np.float32(1.0 / cell_size)
    c = np.floor((p - o) * inv)
    c = np.clip(c, -2 ** 31, 2 ** 31 - 1).astype(np.int64)
    c = np.minimum(np.maximum(c, 0), np.asarray(dims) - 1)
    cell = (c[:, 0] + dims[0] * (c[:, 1] + dims[1] * c[:, 2])).astype(np.uint32)
    order = np.argsort(cell, kind="stable").astype(np.uint32)
    n_cells = int(dims[0]) * int(dims[1]) * int(dims[2])
    start = np.searchsorted(cell[order], np.arange(n_cells + 1), side="left").astype(np.uint32)
    return cell, order, start
