"""Makes the golden fixtures of tests/golden/ by executing the reference's own WGSL (TEST INFRASTRUCTURE).

Run with the path of a reference checkout (v0.3.0) as the argument, or in SI_REFERENCE_DIR:
    python tests/golden/gen_golden.py <reference checkout> [--couple | --retime | --spatial]
It reads src/physics/mpm.js and src/shaders/linalg.js (and, for the extra fixtures,
src/physics/coupling.js, src/physics/rigid-wgsl.js, src/shaders/math.js, src/prims/grid.js), builds each MPM kernel the way the
reference's Kernel class wraps it (src/core/kernel.js:83-104: `let wgi = wid.x + wid.y * nwg.x;
let i = wgi * WG + lidx;` and the `i >= u.n` guard), with the template values of a device without
subgroups and with 16 KB of workgroup memory (tileCap = (16384 - 512) / 16 = 992, mpm.js:302), and
runs them with wgsl_exec on small seeded scenes. Inputs are built with oracle/host_ref.py (the
reference's host JavaScript restated). The outputs are committed as .npz files; the tests never need
the reference.
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [HERE, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
import host_ref  # noqa: E402
import wgsl_exec as W  # noqa: E402
from conftest import mulberry32  # noqa: E402

WG = 256
TILE_CAP = 992
PPT = 2


def kernel_sources(ref):
    mpm = open(os.path.join(ref, "src/physics/mpm.js")).read()
    lin = open(os.path.join(ref, "src/shaders/linalg.js")).read()
    mods = W.field_template(lin, "defineModule('linalg'", "code") + "\n" + W.field_template(mpm, "defineModule('mpm'", "code")

    def tpl(expr):
        if expr.startswith("sg ?"):
            return "{"                    # the portable path (no subgroups)
        return {"this.tileCap": str(TILE_CAP), "this.tileCap * 4": str(TILE_CAP * 4), "PPT": str(PPT)}[expr]

    class Values(dict):
        def __contains__(self, k):
            return True

        def __getitem__(self, k):
            return tpl(k)

    out = {}
    for name in ("mpm-p2g", "mpm-grid", "mpm-g2p", "mpm-key", "mpm-reorder", "mpm-retime"):
        anchor = f"name: '{name}'"
        start = mpm.index(anchor)
        nxt = mpm.find("ctx.kernel({", start)
        seg = mpm[start: nxt if nxt > 0 else len(mpm)]
        shared = W.substitute(W.field_template(mpm, anchor, "shared"), Values()) if "shared:" in seg else ""
        code = W.substitute(W.field_template(mpm, anchor, "code"), Values())
        out[name] = (shared, code)
    return mods, out


def compile_kernel(mods, shared, code, dims, guard):
    consts = f"const WG = {WG}u;\nconst DIMS = vec3u({dims[0]}u, {dims[1]}u, {dims[2]}u);\n"
    pre = "let i = wgi * WG + lidx;\n" + ("if (i >= u.n) { return; }\n" if guard else "")
    ns = W.compile_module(consts + mods + "\n" + shared, pre + code)
    return ns


def particle_buffer(rec):
    return W.Buffer(np.ascontiguousarray(rec, np.float32).copy(), "f32", 32,
                    struct=["x", "v", "c0", "c1", "c2", "f0", "f1", "f2"])


def scene_records(grid, shapes, substeps=8):
    g = host_ref.geometry(grid)
    dt = 1 / 60 / substeps
    recs, mats, count = [], np.zeros((8, 12), np.float32), 0
    for k, (shape, mat, vel) in enumerate(shapes):
        pts = host_ref.sample_shape(shape, g["dx"] / 2, 0.6, count + 1)
        recs.append(host_ref.make_records(pts, k, vel, g["dims"], g["dx"], [0, 0, 0], dt))
        mats[k] = host_ref.material_row(mat)
        count += len(pts)
    return g, np.concatenate(recs), mats, dt


def randomise(rec, seed, scale=1.0, deform=False):
    R = mulberry32(seed)
    for k in range(len(rec)):
        for a in range(3):
            rec[k, 4 + a] = (R() - 0.5) * 0.4 * scale
        for c in range(3):
            for a in range(3):
                rec[k, 8 + 4 * c + a] = (R() - 0.5) * 0.2 * scale
        for o in (11, 15, 19, 23, 27, 31):
            rec[k, o] = (R() - 0.5) * 0.3 * scale
        if deform:
            for c in range(3):
                for a in range(3):
                    rec[k, 20 + 4 * c + a] = (1.0 if a == c else 0.0) + (R() - 0.5) * 0.3
        rec[k, 7] = 1.0 + (R() - 0.5) * 0.2
    return rec


def p2g(kern, mods, rec, dims, mats, vol4, force_global):
    shared, code = kern["mpm-p2g"]
    ns = compile_kernel(mods, shared, code, dims, guard=False)
    nodes = int(np.prod(dims))
    grid = W.Buffer(np.zeros(nodes * 4, np.int32), "i32", 1)
    groups = math.ceil(len(rec) / (WG * PPT))
    W.dispatch(ns, groups, WG, {"P": particle_buffer(rec), "grid": grid, "MATS": W.Buffer(mats.reshape(24, 4).copy(), "f32", 4)},
               {"n": np.uint32(len(rec)), "vol4": np.float32(vol4), "forceGlobal": np.uint32(1 if force_global else 0)})
    return grid.arr.reshape(nodes, 4).copy()


def grid_update(kern, mods, g, dims, gravity, cols, ncol):
    shared, code = kern["mpm-grid"]
    ns = compile_kernel(mods, shared, code, dims, guard=True)
    nodes = int(np.prod(dims))
    buf = W.Buffer(g.copy(), "i32", 4)
    W.dispatch(ns, math.ceil(nodes / WG), WG, {"grid": buf, "COL": W.Buffer(cols.reshape(48, 4).copy(), "f32", 4)},
               {"n": np.uint32(nodes), "gravity": W.Vec(np.array(gravity, np.float32)), "bound": np.float32(3.0),
                "numColliders": np.uint32(ncol), "floorFriction": np.float32(0.4)})
    return buf.arr.copy()


def g2p(kern, mods, rec, dims, gv, mats):
    shared, code = kern["mpm-g2p"]
    ns = compile_kernel(mods, shared, code, dims, guard=True)
    P = particle_buffer(rec)
    W.dispatch(ns, math.ceil(len(rec) / WG), WG,
               {"P": P, "GV": W.Buffer(gv.view(np.float32).copy(), "f32", 4), "MATS": W.Buffer(mats.reshape(24, 4).copy(), "f32", 4)},
               {"n": np.uint32(len(rec)), "bound": np.float32(3.0), "vmax": np.float32(0.9)})
    return P.arr.copy()


def sort(kern, mods, rec, dims, num_blocks):
    """_sort(), mpm.js:614-621: keys + atomic ranks, exclusive scan of the counts, reorder."""
    shared, code = kern["mpm-key"]
    ns = compile_kernel(mods, shared, code, dims, guard=True)
    n = len(rec)
    key = W.Buffer(np.zeros(n, np.uint32), "u32", 1)
    rank = W.Buffer(np.zeros(n, np.uint32), "u32", 1)
    cnt = W.Buffer(np.zeros(num_blocks + 1, np.uint32), "u32", 1)
    W.dispatch(ns, math.ceil(n / WG), WG, {"P": particle_buffer(rec), "key": key, "rank": rank, "cnt": cnt},
               {"n": np.uint32(n)})
    counts = cnt.arr.copy()
    starts = np.concatenate([[0], np.cumsum(counts[:-1])]).astype(np.uint32)   # Scan.run semantics, scan.js:288-306
    shared, code = kern["mpm-reorder"]
    ns = compile_kernel(mods, shared, code, dims, guard=True)
    dst = particle_buffer(np.zeros_like(rec))
    W.dispatch(ns, math.ceil(n / WG), WG, {"src": particle_buffer(rec), "dst": dst, "key": key, "rank": rank,
                                            "start": W.Buffer(starts.copy(), "u32", 1)}, {"n": np.uint32(n)})
    return key.arr.copy(), starts, dst.arr.copy()


def main(ref):
    mods, kern = kernel_sources(ref)
    out = os.path.join(HERE)
    # ---- P2G (tile and global paths) with randomised v, C, tau: tests/physics.test.js:6-17
    g, rec, mats, dt = scene_records(16, [({"box": [[0.3, 0.3, 0.3], [0.62, 0.6, 0.55]]}, dict(kind=0, density=1, stiffness=1.0, viscosity=0.0), [0, 0, 0]),
                                          ({"sphere": [[0.55, 0.5, 0.6], 0.1]}, dict(kind=1, density=1.2, stiffness=0.7, poisson=0.45), [0, 0, 0])])
    rec = randomise(rec, 3)
    vol4 = np.float32(4 * (1 / 2 ** 3))
    g_tile = p2g(kern, mods, rec, g["dims"], mats, vol4, False)
    g_glob = p2g(kern, mods, rec, g["dims"], mats, vol4, True)
    assert np.array_equal(g_tile, g_glob), "the reference's tile and global paths disagree"
    np.savez_compressed(os.path.join(out, "p2g.npz"), rec=rec, mats=mats, dims=np.array(g["dims"]), vol4=vol4, grid=g_tile)
    print("p2g", rec.shape, int((g_tile[:, 3] != 0).sum()), "nodes")
    # ---- grid update with walls, floor friction and three collider kinds
    cols = np.zeros((16, 12), np.float32)
    cl = [{"type": "sphere", "center": [0.45, 0.45, 0.45], "radius": 0.12, "velocity": [0.3, 0, 0], "friction": 0.5},
          {"type": "box", "center": [0.6, 0.35, 0.5], "half": [0.08, 0.05, 0.1]},
          {"type": "plane", "center": [0, 0.3, 0], "normal": [0.1, 1, 0]}]
    for k, c in enumerate(cl):
        cols[k] = host_ref.collider_row(c, g["dx"], [0, 0, 0], dt)
    grav = [np.float32(0), np.float32((-9.81 * dt * dt) / g["dx"]), np.float32(0)]
    gu = grid_update(kern, mods, g_tile, g["dims"], grav, cols, len(cl))
    np.savez_compressed(os.path.join(out, "grid.npz"), grid_in=g_tile, dims=np.array(g["dims"]), gravity=np.array(grav),
                        cols=cols, ncol=len(cl), grid_out=gu.reshape(-1, 4))
    print("grid", int((gu != 0).any(1).sum()), "nodes")
    # ---- G2P for water, honey, jelly, snow, sand from a deformed state
    g2, rec2, mats2, _ = scene_records(16, [
        ({"box": [[0.3, 0.3, 0.3], [0.45, 0.45, 0.45]]}, dict(kind=0, density=1, stiffness=1.0, viscosity=0.0), [0, 0, 0]),
        ({"box": [[0.5, 0.3, 0.3], [0.62, 0.42, 0.42]]}, dict(kind=0, density=1.4, stiffness=0.9, viscosity=1.0), [0, 0, 0]),
        ({"box": [[0.3, 0.5, 0.3], [0.42, 0.62, 0.42]]}, dict(kind=1, density=1, stiffness=0.35, poisson=0.3), [0, 0, 0]),
        ({"box": [[0.5, 0.5, 0.3], [0.62, 0.62, 0.42]]}, dict(kind=2, density=0.4, stiffness=0.6, poisson=0.2, hardening=10, compression=0.025, stretch=0.0075), [0, 0, 0]),
        ({"box": [[0.4, 0.4, 0.5], [0.52, 0.52, 0.62]]}, dict(kind=3, density=1.6, stiffness=0.6, poisson=0.3, friction=30), [0, 0, 0])])
    rec2 = randomise(rec2, 7, scale=0.5, deform=True)
    gsum = p2g(kern, mods, rec2, g2["dims"], mats2, vol4, False)
    gv = grid_update(kern, mods, gsum, g2["dims"], grav, np.zeros((16, 12), np.float32), 0)
    out2 = g2p(kern, mods, rec2, g2["dims"], gv, mats2)
    np.savez_compressed(os.path.join(out, "g2p.npz"), rec=rec2, mats=mats2, dims=np.array(g2["dims"]), grid=gsum, gv=gv,
                        gravity=np.array(grav), vol4=vol4, out=out2)
    print("g2p", rec2.shape)
    # ---- block sort of a stirred state
    g3, rec3, mats3, _ = scene_records(32, [({"box": [[0.1, 0.1, 0.1], [0.4, 0.3, 0.35]]}, dict(kind=0, density=1, stiffness=1.0, viscosity=0.0), [0, 0, 0])])
    rng = np.random.default_rng(5)
    rec3 = rec3[rng.permutation(len(rec3))]
    key, starts, dst = sort(kern, mods, rec3, g3["dims"], g3["num_blocks"])
    np.savez_compressed(os.path.join(out, "sort.npz"), rec=rec3, dims=np.array(g3["dims"]), num_blocks=g3["num_blocks"],
                        keys=key, starts=starts, sorted=dst)
    print("sort", rec3.shape, g3["num_blocks"])
    # ---- whole substeps in step()'s schedule (mpm.js:590-602): sort every 4th, P2G, grid, G2P.
    # Water and honey only (no log/exp on their path), falling onto a sphere and a plane collider.
    g4, rec4, mats4, dt4 = scene_records(16, [
        ({"box": [[0.2, 0.35, 0.25], [0.5, 0.7, 0.6]]}, dict(kind=0, density=1, stiffness=1.0, viscosity=0.0), [0.5, -1.0, 0]),
        ({"sphere": [[0.65, 0.6, 0.5], 0.12]}, dict(kind=0, density=1.4, stiffness=0.9, viscosity=1.0), [-0.5, 0, 0.3])])
    cl4 = [{"type": "sphere", "center": [0.45, 0.25, 0.45], "radius": 0.1, "velocity": [0.2, 0, 0], "friction": 0.5},
           {"type": "plane", "center": [0, 0.2, 0], "normal": [0.2, 1, 0]}]
    cols4 = np.zeros((16, 12), np.float32)
    for k, c in enumerate(cl4):
        cols4[k] = host_ref.collider_row(c, g4["dx"], [0, 0, 0], dt4)
    grav4 = [np.float32(0), np.float32((-9.81 * dt4 * dt4) / g4["dx"]), np.float32(0)]
    K, P = 12, rec4.copy()
    for s in range(K):
        if s % 4 == 0:
            _, _, P = sort(kern, mods, P, g4["dims"], g4["num_blocks"])
        gs4 = p2g(kern, mods, P, g4["dims"], mats4, vol4, False)
        gv4 = grid_update(kern, mods, gs4, g4["dims"], grav4, cols4, len(cl4))
        P = g2p(kern, mods, P, g4["dims"], gv4, mats4)
    np.savez_compressed(os.path.join(out, "trajectory.npz"), rec=rec4, mats=mats4, dims=np.array(g4["dims"]),
                        num_blocks=g4["num_blocks"], cols=cols4, ncol=len(cl4), gravity=np.array(grav4), vol4=vol4,
                        substeps=K, sort_every=4, out=P)
    print("trajectory", rec4.shape, K)





# ============================================================================ fluid <-> rigid coupling
BODY_FIELDS = ["x", "q", "v", "w", "x0", "q0", "y", "qy", "size", "mass", "props", "info"]


def coupling_sources(ref):
    """The coupling module and kernels of src/physics/coupling.js with the parts of the rigid and
    math modules they use (Body, its flags and shapeOf from src/physics/rigid-wgsl.js:20-37,75;
    qmat from src/shaders/math.js:56-62)."""
    cpl = open(os.path.join(ref, "src/physics/coupling.js")).read()
    rig = open(os.path.join(ref, "src/physics/rigid-wgsl.js")).read()
    mth = open(os.path.join(ref, "src/shaders/math.js")).read()
    a = rig.index("struct Body {")
    body = rig[a:rig.index("}", a) + 1]
    flags = "\n".join(l for l in rig.splitlines() if l.startswith("const F_"))
    a = rig.index("fn shapeOf(")
    shape = rig[a:rig.index("\n", a)]
    a = mth.index("fn qmat(")
    qmat = mth[a:mth.index("\n}\n", a) + 2]
    mods = "\n".join([body, flags, shape, qmat, W.field_template(cpl, "defineModule('coupling'", "code")])
    vals = {"MAX_CAND": "128", "MAX_CAND * 3": "384", "FPJ": "16384", "FPL": "1024"}
    couple = (W.substitute(W.field_template(cpl, "name: 'mpm-rigid-couple'", "shared"), vals),
              W.substitute(W.field_template(cpl, "name: 'mpm-rigid-couple'", "code"), vals))
    apply = W.substitute(W.field_template(cpl, "name: 'mpm-rigid-apply'", "code"), vals)
    return mods, couple, apply


def body_record(pos, quat, vel, angvel, shape, size, mass, radius, group=1, mask=0xFFFFFFFF, flags=0):
    r = np.zeros(48, np.float32)
    r[0:3], r[3] = pos, radius
    q = np.asarray(quat, np.float64)
    r[4:8] = q / np.linalg.norm(q)
    r[8:11], r[11] = vel, 0.5
    r[12:15] = angvel
    r[32:35], r[35] = size, shape
    r[36] = mass
    r[44:48] = np.array([group, mask, flags, 0], np.uint32).view(np.float32)
    return r


def couple_case(ref, kern, mods):
    cmods, (cshared, ccode), acode = coupling_sources(ref)
    g, rec, mats, dt = scene_records(16, [({"box": [[0.2, 0.2, 0.2], [0.8, 0.5, 0.8]]},
                                           dict(kind=0, density=1, stiffness=1.0, viscosity=0.0), [0, 0, 0])])
    rec = randomise(rec, 11, scale=0.5)
    vol4 = np.float32(4 * (1 / 2 ** 3))
    gs = p2g(kern, mods, rec, g["dims"], mats, vol4, False)
    grav = [np.float32(0), np.float32((-9.81 * dt * dt) / g["dx"]), np.float32(0)]
    gv = grid_update(kern, mods, gs, g["dims"], grav, np.zeros((16, 12), np.float32), 0)
    s30 = np.sin(np.pi / 12)
    bodies = np.stack([
        body_record([0.5, 0.35, 0.5], [0, 0, 0, 1], [0.1, -0.2, 0], [0, 0, 1.0], 0, [0.1, 0.1, 0.1], 2.0, 0.1),
        body_record([0.35, 0.3, 0.4], [0.2, 0.3, 0.1, 0.93], [0, 0, 0.3], [1.0, 0, 0], 1, [0.08, 0.05, 0.1], 1.0, 0.137),
        body_record([0.65, 0.3, 0.62], [0, 0, s30, np.cos(np.pi / 12)], [0, 0, 0], [0, 0, 0], 2, [0.05, 0.08, 0.05], 0.0, 0.13),
        body_record([0.3, 0.4, 0.7], [0, 0, 0, 1], [0, 0, 0], [0, 0, 0], 0, [0.06, 0.06, 0.06], 1.0, 0.06, flags=4),
        body_record([0.7, 0.4, 0.3], [0, 0, 0, 1], [0, 0, 0], [0, 0, 0], 0, [0.06, 0.06, 0.06], 1.0, 0.06, group=2)])
    dts, dx = float(dt), float(g["dx"])
    prm = {"nBodies": np.uint32(len(bodies)), "mask": np.uint32(1), "origin": W.Vec(np.zeros(3, np.float32)),
           "dx": np.float32(dx), "invDx": np.float32(1 / dx), "lead": np.float32(1.5 * dts),
           "velToLattice": np.float32(dts / dx), "friction": np.float32(0.2), "band": np.float32(0.5)}
    dims = g["dims"]
    consts = f"const WG = 64u;\nconst DIMS = vec3u({dims[0]}u, {dims[1]}u, {dims[2]}u);\n"
    ns = W.compile_module(consts + cmods + "\n" + cshared, "let wgi = wid.x + wid.y * nwg.x;\nlet p = gid;\n" + ccode)
    grid = W.Buffer(gv.copy(), "i32", 4)
    gacc = W.Buffer(np.zeros(len(bodies) * 8, np.int32), "i32", 1)
    B = W.Buffer(bodies.copy(), "f32", 48, struct=BODY_FIELDS, struct_types={"info": "u32"})
    W.dispatch3(ns, [math.ceil(d / 4) for d in dims], (4, 4, 4), {"grid": grid, "B": B, "gacc": gacc}, prm)
    acc = gacc.arr.copy()
    ns2 = W.compile_module(f"const WG = {WG}u;\n" + cmods, "let i = wgi * WG + lidx;\nif (i >= u.n) { return; }\n" + acode)
    ext = W.Buffer(np.zeros((len(bodies) * 2, 4), np.float32), "f32", 4)
    accb = W.Buffer(acc.reshape(-1, 4).copy(), "i32", 4)
    m2w = np.float32(1.0 * dx ** 4 / dts)
    W.dispatch(ns2, 1, WG, {"acc": accb, "ext": ext}, {"n": np.uint32(len(bodies)), "momToWorld": m2w, "dx": np.float32(dx)})
    return {"rec": rec, "mats": mats, "dims": np.array(dims), "grid_in": gv, "bodies": bodies,
            "params": np.array([0, 0, 0, dx, 1 / dx, 1.5 * dts, dts / dx, 0.2, 0.5], np.float32), "mask": 1,
            "grid_out": grid.arr.copy(), "acc": acc, "mom_to_world": m2w, "ext": ext.arr.reshape(-1, 8).copy()}


def main_couple(ref):
    mods, kern = kernel_sources(ref)
    out = couple_case(ref, kern, mods)
    np.savez_compressed(os.path.join(HERE, "couple.npz"), **out)
    moved = int((out["grid_out"] != out["grid_in"]).any(1).sum())
    print("couple", moved, "nodes changed; acc", out["acc"].reshape(-1, 8)[:, [0, 1, 2, 4, 5, 6]].tolist())


# ============================================================================ retime (mpm-retime)
def main_retime(ref):
    """rescaleK of mpm.js:405-413 (run by _retime, mpm.js:140-145) on a deformed five-material state,
    from the same state at k = 0.5, k = 2 and the k of a substeps change 8 -> 6 (f64 ratio of the
    two substepDt values, rounded to f32 as the uniform is)."""
    mods, kern = kernel_sources(ref)
    shared, code = kern["mpm-retime"]
    g, rec, mats, _ = scene_records(16, [
        ({"box": [[0.3, 0.3, 0.3], [0.45, 0.45, 0.45]]}, dict(kind=0, density=1, stiffness=1.0, viscosity=0.0), [0, 0, 0]),
        ({"box": [[0.5, 0.3, 0.3], [0.62, 0.42, 0.42]]}, dict(kind=0, density=1.4, stiffness=0.9, viscosity=1.0), [0, 0, 0]),
        ({"box": [[0.3, 0.5, 0.3], [0.42, 0.62, 0.42]]}, dict(kind=1, density=1, stiffness=0.35, poisson=0.3), [0, 0, 0]),
        ({"box": [[0.5, 0.5, 0.3], [0.62, 0.62, 0.42]]}, dict(kind=2, density=0.4, stiffness=0.6, poisson=0.2, hardening=10, compression=0.025, stretch=0.0075), [0, 0, 0]),
        ({"box": [[0.4, 0.4, 0.5], [0.52, 0.52, 0.62]]}, dict(kind=3, density=1.6, stiffness=0.6, poisson=0.3, friction=30), [0, 0, 0])])
    rec = randomise(rec, 13, scale=0.7, deform=True)
    ns = compile_kernel(mods, shared, code, g["dims"], guard=True)
    k86 = ((1 / 60) * 1 / 6) / ((1 / 60) * 1 / 8)
    ks = np.array([0.5, 2.0, k86], np.float32)
    outs = []
    for k in ks:
        P = W.Buffer(np.ascontiguousarray(rec, np.float32).reshape(-1, 4).copy(), "f32", 4)
        W.dispatch(ns, math.ceil(len(rec) / WG), WG, {"P": P}, {"n": np.uint32(len(rec)), "k": np.float32(k)})
        outs.append(P.arr.reshape(-1, 32).copy())
    np.savez_compressed(os.path.join(HERE, "retime.npz"), rec=rec, mats=mats, dims=np.array(g["dims"]), ks=ks,
                        out=np.stack(outs))
    print("retime", rec.shape, ks.tolist())


# ============================================================================ SpatialGrid (grid.js)
def main_spatial(ref):
    """SpatialGrid.build of src/prims/grid.js:23-96: grid-count (gridCoord / gridIndex of the 'grid'
    module, atomic ranks), the exclusive scan of the counts with the total in element numCells
    (scan.js:288-306), grid-scatter. Points include some outside the box (gridCoord clamps them)."""
    src = open(os.path.join(ref, "src/prims/grid.js")).read()
    mod = W.field_template(src, "defineModule('grid'", "code")
    count_code = W.field_template(src, "name: 'grid-count'", "code")
    scatter_code = W.field_template(src, "name: 'grid-scatter'", "code")
    rng = np.random.default_rng(21)
    lo, hi, cell = [-1.0, 0.0, 0.5], [1.0, 1.5, 1.7], 0.125
    dims = [max(1, math.ceil((hi[a] - lo[a]) / cell)) for a in range(3)]
    cells = dims[0] * dims[1] * dims[2]
    n = 2500
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(np.array(lo) - 0.1, np.array(hi) + 0.1, (n, 3)).astype(np.float32)
    pos[:40, :3] = pos[0, :3]                              # one crowded cell
    uni = {"n": np.uint32(n), "gridOrigin": W.Vec(np.array(lo, np.float32)), "gridInv": np.float32(1 / cell),
           "gridDims": W.Vec(np.array(dims, np.uint32)), "gridCells": np.uint32(cells)}
    pre = "let i = wgi * WG + lidx;\nif (i >= u.n) { return; }\n"
    ns = W.compile_module(f"const WG = {WG}u;\n" + mod, pre + count_code)
    cellb = W.Buffer(np.zeros(n, np.uint32), "u32", 1)
    rankb = W.Buffer(np.zeros(n, np.uint32), "u32", 1)
    cnt = W.Buffer(np.zeros(cells + 1, np.uint32), "u32", 1)
    W.dispatch(ns, math.ceil(n / WG), WG, {"pos": W.Buffer(pos.copy(), "f32", 4), "cell": cellb, "rank": rankb,
                                           "count": cnt}, uni)
    counts = cnt.arr.copy()
    start = np.concatenate([[0], np.cumsum(counts[:-1])]).astype(np.uint32)
    ns2 = W.compile_module(f"const WG = {WG}u;\n", pre + scatter_code)
    order = W.Buffer(np.zeros(n, np.uint32), "u32", 1)
    W.dispatch(ns2, math.ceil(n / WG), WG, {"cell": cellb, "rank": rankb, "start": W.Buffer(start.copy(), "u32", 1),
                                            "order": order}, {"n": np.uint32(n)})
    np.savez_compressed(os.path.join(HERE, "spatial.npz"), pos=pos, lo=np.array(lo), hi=np.array(hi), cell_size=cell,
                        dims=np.array(dims), cell=cellb.arr.copy(), start=start, order=order.arr.copy())
    print("spatial", n, "points", cells, "cells")


if __name__ == "__main__":
    ref_dir = next((a for a in sys.argv[1:] if not a.startswith("--")), os.environ.get("SI_REFERENCE_DIR"))
    if not ref_dir:
        sys.exit("usage: gen_golden.py <reference checkout> [--couple|--retime|--spatial] (or set SI_REFERENCE_DIR)")
    if "--couple" in sys.argv:
        main_couple(ref_dir)
    elif "--retime" in sys.argv:
        main_retime(ref_dir)
    elif "--spatial" in sys.argv:
        main_spatial(ref_dir)
    else:
        main(ref_dir)
        main_couple(ref_dir)
        main_retime(ref_dir)
        main_spatial(ref_dir)
