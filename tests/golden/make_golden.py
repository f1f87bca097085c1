"""Generates the golden fixtures in this directory from the REFERENCE ODE 0.12
(built from its own sources by `make -C oracle ref` into oracle/_ref/,
double precision, driven through its public C API by oracle/ref_harness.cpp).

Run from the repository root where the reference sources are present:
    make -C oracle ref && python tests/golden/make_golden.py
Each .npz holds the scene arrays (so no generator has to be re-run), the
reference's per-step contact counts, contact records, RNG seeds, body states
at selected steps, and joint feedback. collider_kats.npz holds single dCollide
calls on seeded near-contact poses for every collider on the path.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from odegpu import scene as S  # noqa: E402
import oracle_lib as O  # noqa: E402

SCENES = {
    "box_drop": (lambda: S.box_drop(seed=0), 80),
    "batched": (lambda: S.batched_worlds(n_worlds=6, seed=7), 60),
    "hinge": (lambda: S.hinge_chains(n_worlds=3, steps=60), 60),
    "stack": (lambda: S.box_stack(n_worlds=2, height=5), 100),
    "capsule": (lambda: S.capsule_mix(seed=6), 80),
    "vehicles": (lambda: S.vehicles(n_worlds=3, steps=60, hf_samples=64), 60),
    "capsule_pile": (lambda: S.capsule_pile(), 120),
    "mechanisms": (lambda: S.mechanisms(n_worlds=3, steps=80), 80),
    "cylinder_pile": (lambda: S.cylinder_pile(), 120),
}
KEEP = 10  # keep the state every KEEP steps


# dWorldStep (the exact stepper, ode/src/step.cpp + lcp.cpp) on the same scenes
EXACT_SCENES = ["box_drop", "batched", "mechanisms", "vehicles", "cylinder_pile"]


def make_scene(name, exact=False):
    mk, steps = SCENES[name]
    sc = mk()
    ref = O.ref("d")
    ref.ref_set_stepper(1 if exact else 0)
    out = dict(sc.to_arrays())
    out["n_steps"] = np.int64(steps)
    for w in range(sc.n_worlds):
        r = O.run_world(ref.ref_run_world, sc, w, steps, max_rec=96, feedback=True)
        out[f"w{w}_ncontacts"] = r["ncontacts"]
        out[f"w{w}_contacts"] = r["contacts"][:, :64].astype(np.float64)
        out[f"w{w}_seeds"] = r["seeds"]
        out[f"w{w}_state"] = r["state"][::KEEP]
        out[f"w{w}_final"] = r["state"][-1]
        out[f"w{w}_feedback"] = r["feedback"]
    ref.ref_set_stepper(0)
    np.savez_compressed(os.path.join(HERE, f"{'exact_' if exact else ''}{name}.npz"), **out)


def rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                     [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                     [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])


def make_collider_kats(n=120, seed=123):
    """Random near-contact poses for each class pair, both argument orders."""
    import ctypes as C
    rng = np.random.Generator(np.random.PCG64(seed))
    ref = O.ref("d")
    pairs = [(0, 0), (0, 1), (1, 0), (0, 4), (4, 0), (1, 1), (1, 4), (4, 1), (2, 4), (4, 2),
             (2, 0), (0, 2), (2, 1), (1, 2), (2, 2)]
    recs = []
    for (t1, t2) in pairs:
        for _ in range(n):
            def params(t):
                if t == 0:
                    return np.array([rng.uniform(0.1, 0.6), 0, 0, 0])
                if t == 1:
                    return np.concatenate([rng.uniform(0.2, 1.2, 3), [0]])
                if t == 2:
                    return np.array([rng.uniform(0.1, 0.4), rng.uniform(0.2, 1.0), 0, 0])
                nrm = rng.normal(size=3)
                nrm /= np.linalg.norm(nrm)
                return np.concatenate([nrm, [rng.uniform(-0.3, 0.3)]])
            p1, p2 = params(t1), params(t2)
            pos1 = rng.uniform(-0.6, 0.6, 3)
            pos2 = rng.uniform(-0.6, 0.6, 3)
            R1, R2 = rot(rng), rot(rng)
            flags = int(rng.choice([1, 2, 3, 4, 8]))
            out = np.zeros((16, 9))
            P = C.POINTER(C.c_double)
            args = [np.ascontiguousarray(a, dtype=np.float64) for a in
                    (p1, pos1, R1.ravel(), p2, pos2, R2.ravel())]
            nc = ref.ref_collide(t1, args[0].ctypes.data_as(P), args[1].ctypes.data_as(P),
                                 args[2].ctypes.data_as(P), t2, args[3].ctypes.data_as(P),
                                 args[4].ctypes.data_as(P), args[5].ctypes.data_as(P), flags,
                                 out.ctypes.data_as(P))
            recs.append((t1, t2, flags, p1, pos1, R1.ravel(), p2, pos2, R2.ravel(), nc, out[:8]))
    np.savez_compressed(
        os.path.join(HERE, "collider_kats.npz"),
        t1=np.array([r[0] for r in recs]), t2=np.array([r[1] for r in recs]),
        flags=np.array([r[2] for r in recs]),
        p1=np.array([r[3] for r in recs]), pos1=np.array([r[4] for r in recs]),
        R1=np.array([r[5] for r in recs]), p2=np.array([r[6] for r in recs]),
        pos2=np.array([r[7] for r in recs]), R2=np.array([r[8] for r in recs]),
        nc=np.array([r[9] for r in recs]), out=np.array([r[10] for r in recs]))


def make_hf_kats(n=150, seed=321):
    """dCollide(heightfield, geom) on a seeded 33 x 29 fractal field placed with
    its up axis along world z, for spheres, boxes and capsules in random poses
    near the surface and random contact limits."""
    import ctypes as C
    rng = np.random.Generator(np.random.PCG64(seed))
    ref = O.ref("d")
    f = ref.ref_collide_hf
    P = C.POINTER(C.c_double)
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, P, P, P, C.c_int, P]
    nx, nz, sp = 33, 29, 0.5
    h = np.ascontiguousarray(S.fractal_heights(64, 0.3, seed=seed)[:nz, :nx])
    Rh = np.array(S.HF_Z_UP)
    pos_h = np.array([0.4, -0.3, 0.2])
    H = S.Heightfield()
    H.nx, H.nz = nx, nz
    H.width, H.depth = sp * (nx - 1), sp * (nz - 1)
    H.scale, H.offset, H.thickness, H.wrap = 1.0, 0.0, 1.0, 0
    H.heights = h.ctypes.data_as(P)
    H.pos[:] = list(pos_h)
    H.R[:] = list(Rh.ravel())
    recs = []
    for t2 in (0, 1, 2):
        for _ in range(n):
            if t2 == 0:
                p2 = np.array([rng.uniform(0.2, 0.5), 0, 0, 0])
            elif t2 == 1:
                p2 = np.concatenate([rng.uniform(0.3, 2.0, 3), [0]])
            else:
                p2 = np.array([rng.uniform(0.1, 0.3), rng.uniform(0.2, 1.0), 0, 0])
            local = np.array([rng.uniform(-0.45, 0.45) * H.width, 0.0, rng.uniform(-0.45, 0.45) * H.depth])
            ix = int(np.clip(round((local[0] + H.width / 2) / sp), 0, nx - 1))
            iz = int(np.clip(round((local[2] + H.depth / 2) / sp), 0, nz - 1))
            local[1] = h[iz, ix] + rng.uniform(-0.3, 0.6)
            pos2 = Rh @ local + pos_h
            R2 = rot(rng) if rng.uniform() < 0.8 else np.eye(3)
            flags = int(rng.choice([1, 2, 3, 4, 8]))
            out = np.zeros((64, 9))
            args = [np.ascontiguousarray(a, dtype=np.float64) for a in (p2, pos2, R2.ravel())]
            nc = f(C.byref(H), t2, args[0].ctypes.data_as(P), args[1].ctypes.data_as(P),
                   args[2].ctypes.data_as(P), flags, out.ctypes.data_as(P))
            recs.append((t2, flags, p2, pos2, R2.ravel(), nc, out[:8]))
    np.savez_compressed(
        os.path.join(HERE, "hf_kats.npz"), heights=h, spacing=sp, hf_pos=pos_h, hf_R=Rh.ravel(),
        t2=np.array([r[0] for r in recs]), flags=np.array([r[1] for r in recs]),
        p2=np.array([r[2] for r in recs]), pos2=np.array([r[3] for r in recs]),
        R2=np.array([r[4] for r in recs]), nc=np.array([r[5] for r in recs]),
        out=np.array([r[6] for r in recs]))


def make_hf_big_kats(n=40, seed=909):
    """dCollide(heightfield, geom) for geoms that cover more than 10 x 10
    samples (zones of up to ~60 samples per axis): a seeded 96 x 80 fractal
    field at 0.25 m spacing, spheres, boxes, capsules and cylinders of several
    metres near its surface, random contact limits; the dDOUBLE build's
    outputs (nc / out) and the dSINGLE build's (nc_s / out_s)."""
    import ctypes as C
    rng = np.random.Generator(np.random.PCG64(seed))
    P = C.POINTER(C.c_double)
    nx, nz, sp = 96, 80, 0.25
    h = np.ascontiguousarray(S.fractal_heights(128, 0.4, seed=seed)[:nz, :nx])
    Rh = np.array(S.HF_Z_UP)
    pos_h = np.array([-0.7, 0.5, 0.1])
    H = S.Heightfield()
    H.nx, H.nz = nx, nz
    H.width, H.depth = sp * (nx - 1), sp * (nz - 1)
    H.scale, H.offset, H.thickness, H.wrap = 1.0, 0.0, 1.0, 0
    H.heights = h.ctypes.data_as(P)
    H.pos[:] = list(pos_h)
    H.R[:] = list(Rh.ravel())
    fd, fs = O.ref("d").ref_collide_hf, O.ref("s").ref_collide_hf
    for f in (fd, fs):
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.c_int, P, P, P, C.c_int, P]
    recs = []
    for t2 in (0, 1, 2, 3):
        for _ in range(n):
            if t2 == 0:
                p2 = np.array([rng.uniform(1.3, 3.5), 0, 0, 0])
                down = p2[0]
            elif t2 == 1:
                p2 = np.concatenate([rng.uniform(2.5, 8.0, 3), [0]])
                down = 0.3 * np.linalg.norm(p2[:3])
            elif t2 == 2:
                p2 = np.array([rng.uniform(0.8, 1.5), rng.uniform(3.0, 8.0), 0, 0])
                down = p2[0] + 0.2 * p2[1]
            else:
                p2 = np.array([rng.uniform(1.0, 2.5), rng.uniform(2.0, 5.0), 0, 0])
                down = 0.5 * p2[0] + 0.3 * p2[1]
            local = np.array([rng.uniform(-0.3, 0.3) * H.width, 0.0, rng.uniform(-0.3, 0.3) * H.depth])
            ix = int(np.clip(round((local[0] + H.width / 2) / sp), 0, nx - 1))
            iz = int(np.clip(round((local[2] + H.depth / 2) / sp), 0, nz - 1))
            local[1] = h[iz, ix] + down + rng.uniform(-0.6, 0.3)
            pos2 = Rh @ local + pos_h
            R2 = rot(rng) if rng.uniform() < 0.8 else np.eye(3)
            flags = int(rng.choice([1, 2, 4, 8]))
            args = [np.ascontiguousarray(a, dtype=np.float64) for a in (p2, pos2, R2.ravel())]
            res = []
            for f in (fd, fs):
                out = np.zeros((64, 9))
                nc = f(C.byref(H), t2, *(a.ctypes.data_as(P) for a in args), flags, out.ctypes.data_as(P))
                res.append((nc, out[:8]))
            recs.append((t2, flags, p2, pos2, R2.ravel(), res[0][0], res[0][1], res[1][0], res[1][1]))
    np.savez_compressed(
        os.path.join(HERE, "hf_big_kats.npz"), heights=h, spacing=sp, hf_pos=pos_h, hf_R=Rh.ravel(),
        t2=np.array([r[0] for r in recs]), flags=np.array([r[1] for r in recs]),
        p2=np.array([r[2] for r in recs]), pos2=np.array([r[3] for r in recs]),
        R2=np.array([r[4] for r in recs]), nc=np.array([r[5] for r in recs]),
        out=np.array([r[6] for r in recs]), nc_s=np.array([r[7] for r in recs]),
        out_s=np.array([r[8] for r in recs]))


def frame_with_z(d):
    """A rotation whose third column is the unit vector d (a ray geom points
    along column 2 of its rotation, ode/src/ray.cpp:115-136)."""
    d = d / np.linalg.norm(d)
    a = np.array([1.0, 0, 0]) if abs(d[0]) < 0.9 else np.array([0, 1.0, 0])
    x = np.cross(a, d)
    x /= np.linalg.norm(x)
    y = np.cross(d, x)
    return np.stack([x, y, d], axis=1)


def make_ray_kats(n=150, seed=555):
    """Rays (ODE's dRayClass) through dCollide: against sphere / box / capsule /
    plane in both argument orders, and against the placeable fractal field of
    hf_kats.npz. Starts are spread around the target, inside it for some, and
    directions aim near it so that most calls hit."""
    import ctypes as C
    rng = np.random.Generator(np.random.PCG64(seed))
    ref = O.ref("d")
    P = C.POINTER(C.c_double)
    recs = []
    for (t1, t2) in [(5, 0), (0, 5), (5, 1), (1, 5), (5, 2), (2, 5), (5, 4), (4, 5), (5, 5)]:
        other = t2 if t1 == 5 else t1
        for _ in range(n):
            if other == 0:
                po = np.array([rng.uniform(0.1, 0.6), 0, 0, 0])
            elif other == 1:
                po = np.concatenate([rng.uniform(0.2, 1.2, 3), [0]])
            elif other == 2:
                po = np.array([rng.uniform(0.1, 0.4), rng.uniform(0.2, 1.0), 0, 0])
            elif other == 4:
                nrm = rng.normal(size=3)
                nrm /= np.linalg.norm(nrm)
                po = np.concatenate([nrm, [rng.uniform(-0.3, 0.3)]])
            else:
                po = np.array([rng.uniform(0.2, 2.0), 0, 0, 0])
            pos_o = rng.uniform(-0.3, 0.3, 3)
            Ro = rot(rng)
            start = pos_o + rng.normal(size=3) * rng.uniform(0.0, 1.5)
            aim = pos_o + rng.normal(size=3) * 0.3 - start
            if rng.uniform() < 0.2 or np.linalg.norm(aim) < 1e-6:
                aim = rng.normal(size=3)
            pr = np.array([rng.uniform(0.2, 3.0), 0, 0, 0])
            Rr = frame_with_z(aim)
            if t1 == 5:
                p1, pos1, R1, p2, pos2, R2 = pr, start, Rr, po, pos_o, Ro
            else:
                p1, pos1, R1, p2, pos2, R2 = po, pos_o, Ro, pr, start, Rr
            flags = int(rng.choice([1, 2, 4]))
            out = np.zeros((16, 9))
            args = [np.ascontiguousarray(a, dtype=np.float64) for a in
                    (p1, pos1, R1.ravel(), p2, pos2, R2.ravel())]
            nc = ref.ref_collide(t1, args[0].ctypes.data_as(P), args[1].ctypes.data_as(P),
                                 args[2].ctypes.data_as(P), t2, args[3].ctypes.data_as(P),
                                 args[4].ctypes.data_as(P), args[5].ctypes.data_as(P), flags,
                                 out.ctypes.data_as(P))
            recs.append((t1, t2, flags, p1, pos1, R1.ravel(), p2, pos2, R2.ravel(), nc, out[:8]))
    # rays against the heightfield of hf_kats.npz, mostly downwards (wheel probes)
    g = np.load(os.path.join(HERE, "hf_kats.npz"))
    h = np.ascontiguousarray(g["heights"])
    sp = float(g["spacing"])
    nz, nx = h.shape
    Rh = g["hf_R"].reshape(3, 3)
    pos_h = g["hf_pos"]
    H = S.Heightfield()
    H.nx, H.nz = nx, nz
    H.width, H.depth = sp * (nx - 1), sp * (nz - 1)
    H.scale, H.offset, H.thickness, H.wrap = 1.0, 0.0, 1.0, 0
    H.heights = h.ctypes.data_as(P)
    H.pos[:] = list(pos_h)
    H.R[:] = list(Rh.ravel())
    f = ref.ref_collide_hf
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, P, P, P, C.c_int, P]
    hrecs = []
    for _ in range(2 * n):
        local = np.array([rng.uniform(-0.45, 0.45) * H.width, 0.0, rng.uniform(-0.45, 0.45) * H.depth])
        ix = int(np.clip(round((local[0] + H.width / 2) / sp), 0, nx - 1))
        iz = int(np.clip(round((local[2] + H.depth / 2) / sp), 0, nz - 1))
        local[1] = h[iz, ix] + rng.uniform(-0.3, 1.5)
        d_local = np.array([rng.normal() * 0.3, -1.0, rng.normal() * 0.3])
        if rng.uniform() < 0.15:
            d_local[1] = 1.0
        pos2 = Rh @ local + pos_h
        R2 = frame_with_z(Rh @ d_local)
        p2 = np.array([rng.uniform(0.3, 2.0), 0, 0, 0])
        flags = int(rng.choice([1, 2, 4]))
        out = np.zeros((64, 9))
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in (p2, pos2, R2.ravel())]
        nc = f(C.byref(H), 5, args[0].ctypes.data_as(P), args[1].ctypes.data_as(P),
               args[2].ctypes.data_as(P), flags, out.ctypes.data_as(P))
        hrecs.append((flags, p2, pos2, R2.ravel(), nc, out[:8]))
    np.savez_compressed(
        os.path.join(HERE, "ray_kats.npz"),
        t1=np.array([r[0] for r in recs]), t2=np.array([r[1] for r in recs]),
        flags=np.array([r[2] for r in recs]),
        p1=np.array([r[3] for r in recs]), pos1=np.array([r[4] for r in recs]),
        R1=np.array([r[5] for r in recs]), p2=np.array([r[6] for r in recs]),
        pos2=np.array([r[7] for r in recs]), R2=np.array([r[8] for r in recs]),
        nc=np.array([r[9] for r in recs]), out=np.array([r[10] for r in recs]),
        hf_flags=np.array([r[0] for r in hrecs]), hf_p2=np.array([r[1] for r in hrecs]),
        hf_pos2=np.array([r[2] for r in hrecs]), hf_R2=np.array([r[3] for r in hrecs]),
        hf_nc=np.array([r[4] for r in hrecs]), hf_out=np.array([r[5] for r in hrecs]))


def _axis_rot(rng):
    """A rotation about a random coordinate axis by a multiple of 90 degrees
    (exactly representable), for the aligned cases of the cylinder colliders."""
    R = np.eye(3)
    k = int(rng.integers(0, 3))
    for _ in range(int(rng.integers(0, 4))):
        Q = np.zeros((3, 3))
        a, b = [(1, 2), (0, 2), (0, 1)][k]
        Q[k, k] = 1
        Q[a, b], Q[b, a] = -1, 1
        R = Q @ R
    return R


def make_cylinder_kats(n=150, seed=777):
    """Cylinders (dCylinderClass) through dCollide: with sphere, box and plane
    in both argument orders, rays into cylinders, cylinder against cylinder
    and capsule (no collider without libccd), and dCollide(heightfield,
    cylinder) on the field of hf_kats.npz. A fifth of the poses are axis
    aligned (the parallel-disc and box-face clipping branches)."""
    import ctypes as C
    rng = np.random.Generator(np.random.PCG64(seed))
    ref = O.ref("d")
    P = C.POINTER(C.c_double)

    def params(t):
        if t == 0:
            return np.array([rng.uniform(0.1, 0.6), 0, 0, 0])
        if t == 1:
            return np.concatenate([rng.uniform(0.2, 1.2, 3), [0]])
        if t == 2:
            return np.array([rng.uniform(0.1, 0.4), rng.uniform(0.2, 1.0), 0, 0])
        if t == 3:
            return np.array([rng.uniform(0.1, 0.5), rng.uniform(0.2, 1.2), 0, 0])
        if t == 5:
            return np.array([rng.uniform(0.2, 3.0), 0, 0, 0])
        nrm = rng.normal(size=3) if rng.uniform() < 0.7 else np.eye(3)[int(rng.integers(0, 3))]
        nrm = nrm / np.linalg.norm(nrm)
        return np.concatenate([nrm, [rng.uniform(-0.3, 0.3)]])

    recs = []
    for (t1, t2) in [(3, 0), (0, 3), (3, 1), (1, 3), (3, 4), (4, 3), (5, 3), (3, 5), (3, 3), (2, 3), (3, 2)]:
        for _ in range(n):
            p1, p2 = params(t1), params(t2)
            aligned = rng.uniform() < 0.2
            pos1 = rng.uniform(-0.5, 0.5, 3)
            pos2 = rng.uniform(-0.5, 0.5, 3)
            R1 = _axis_rot(rng) if aligned else rot(rng)
            R2 = _axis_rot(rng) if aligned else rot(rng)
            if 5 in (t1, t2):
                start = (pos2 if t1 == 5 else pos1) + rng.normal(size=3) * rng.uniform(0.0, 1.5)
                aim = (pos1 if t1 == 5 else pos2) + rng.normal(size=3) * 0.2 - start
                if aligned:   # along the cylinder's axis
                    Rc = R2 if t1 == 5 else R1
                    aim = Rc[:, 2] * rng.choice([-1.0, 1.0])
                    start = (pos2 if t1 == 5 else pos1) + Rc[:, 0] * rng.uniform(-0.3, 0.3) - aim * 1.0
                Rr = frame_with_z(aim)
                if t1 == 5:
                    pos1, R1 = start, Rr
                else:
                    pos2, R2 = start, Rr
            flags = int(rng.choice([1, 2, 3, 4, 8]))
            out = np.zeros((16, 9))
            args = [np.ascontiguousarray(a, dtype=np.float64) for a in
                    (p1, pos1, R1.ravel(), p2, pos2, R2.ravel())]
            nc = ref.ref_collide(t1, args[0].ctypes.data_as(P), args[1].ctypes.data_as(P),
                                 args[2].ctypes.data_as(P), t2, args[3].ctypes.data_as(P),
                                 args[4].ctypes.data_as(P), args[5].ctypes.data_as(P), flags,
                                 out.ctypes.data_as(P))
            recs.append((t1, t2, flags, p1, pos1, R1.ravel(), p2, pos2, R2.ravel(), nc, out[:8]))
    g = np.load(os.path.join(HERE, "hf_kats.npz"))
    h = np.ascontiguousarray(g["heights"])
    sp = float(g["spacing"])
    nz, nx = h.shape
    Rh = g["hf_R"].reshape(3, 3)
    pos_h = g["hf_pos"]
    H = S.Heightfield()
    H.nx, H.nz = nx, nz
    H.width, H.depth = sp * (nx - 1), sp * (nz - 1)
    H.scale, H.offset, H.thickness, H.wrap = 1.0, 0.0, 1.0, 0
    H.heights = h.ctypes.data_as(P)
    H.pos[:] = list(pos_h)
    H.R[:] = list(Rh.ravel())
    f = ref.ref_collide_hf
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, P, P, P, C.c_int, P]
    hrecs = []
    for _ in range(2 * n):
        p2 = np.array([rng.uniform(0.1, 0.6), rng.uniform(0.2, 1.5), 0, 0])
        local = np.array([rng.uniform(-0.45, 0.45) * H.width, 0.0, rng.uniform(-0.45, 0.45) * H.depth])
        ix = int(np.clip(round((local[0] + H.width / 2) / sp), 0, nx - 1))
        iz = int(np.clip(round((local[2] + H.depth / 2) / sp), 0, nz - 1))
        local[1] = h[iz, ix] + rng.uniform(-0.3, 0.6)
        pos2 = Rh @ local + pos_h
        R2 = rot(rng) if rng.uniform() < 0.8 else np.eye(3)
        flags = int(rng.choice([1, 2, 3, 4, 8]))
        out = np.zeros((64, 9))
        args = [np.ascontiguousarray(a, dtype=np.float64) for a in (p2, pos2, R2.ravel())]
        nc = f(C.byref(H), 3, args[0].ctypes.data_as(P), args[1].ctypes.data_as(P),
               args[2].ctypes.data_as(P), flags, out.ctypes.data_as(P))
        hrecs.append((flags, p2, pos2, R2.ravel(), nc, out[:8]))
    np.savez_compressed(
        os.path.join(HERE, "cylinder_kats.npz"),
        t1=np.array([r[0] for r in recs]), t2=np.array([r[1] for r in recs]),
        flags=np.array([r[2] for r in recs]),
        p1=np.array([r[3] for r in recs]), pos1=np.array([r[4] for r in recs]),
        R1=np.array([r[5] for r in recs]), p2=np.array([r[6] for r in recs]),
        pos2=np.array([r[7] for r in recs]), R2=np.array([r[8] for r in recs]),
        nc=np.array([r[9] for r in recs]), out=np.array([r[10] for r in recs]),
        hf_flags=np.array([r[0] for r in hrecs]), hf_p2=np.array([r[1] for r in hrecs]),
        hf_pos2=np.array([r[2] for r in hrecs]), hf_R2=np.array([r[3] for r in hrecs]),
        hf_nc=np.array([r[4] for r in hrecs]), hf_out=np.array([r[5] for r in hrecs]))


def add_single_outputs(name, hf_class=None):
    """Adds the reference's dSINGLE (FP32) outputs of the same dCollide calls to
    a known-answer fixture (nc_s / out_s, and hf_nc_s / hf_out_s for its
    heightfield calls): the bar for the FP32 path, whose colliders keep the
    FP32 build's tolerances (collision_cylinder_*.cpp "toleranz", dEpsilon)."""
    import ctypes as C
    path = os.path.join(HERE, f"{name}.npz")
    g = dict(np.load(path))
    ref = O.ref("s")
    P = C.POINTER(C.c_double)
    n = len(g["t1"]) if "t1" in g else 0
    nc_s, out_s = np.zeros(n, np.int64), np.zeros((n, 8, 9))
    # and every contact the collider can give (16 asked for): where a tie
    # picks which of several equally deep points come first, the FP32 path
    # may return other points of the same set
    nc_all, out_all = np.zeros(n, np.int64), np.zeros((n, 16, 9))
    for k in range(n):
        out = np.zeros((16, 9))
        args = [np.ascontiguousarray(g[x][k], dtype=np.float64) for x in ("p1", "pos1", "R1", "p2", "pos2", "R2")]
        nc_s[k] = ref.ref_collide(int(g["t1"][k]), *(a.ctypes.data_as(P) for a in args[:3]), int(g["t2"][k]),
                                  *(a.ctypes.data_as(P) for a in args[3:]), int(g["flags"][k]), out.ctypes.data_as(P))
        out_s[k] = out[:8]
        out = np.zeros((16, 9))
        nc_all[k] = ref.ref_collide(int(g["t1"][k]), *(a.ctypes.data_as(P) for a in args[:3]), int(g["t2"][k]),
                                    *(a.ctypes.data_as(P) for a in args[3:]), (int(g["flags"][k]) & ~0xffff) | 16,
                                    out.ctypes.data_as(P))
        out_all[k] = out
    if n:
        g["nc_s"], g["out_s"] = nc_s, out_s
        g["nc_s_all"], g["out_s_all"] = nc_all, out_all
    hkey = "hf_nc" if "hf_nc" in g else ("nc" if name == "hf_kats" else None)
    if hkey:
        pre = "hf_" if hkey == "hf_nc" else ""
        hg = np.load(os.path.join(HERE, "hf_kats.npz"))
        h = np.ascontiguousarray(hg["heights"])
        sp = float(hg["spacing"])
        H = S.Heightfield()
        H.nz, H.nx = h.shape
        H.width, H.depth = sp * (H.nx - 1), sp * (H.nz - 1)
        H.scale, H.offset, H.thickness, H.wrap = 1.0, 0.0, 1.0, 0
        H.heights = h.ctypes.data_as(P)
        H.pos[:] = [float(x) for x in hg["hf_pos"]]
        H.R[:] = [float(x) for x in hg["hf_R"]]
        f = ref.ref_collide_hf
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.c_int, P, P, P, C.c_int, P]
        m = len(g[hkey])
        hn, ho = np.zeros(m, np.int64), np.zeros((m, 8, 9))
        for k in range(m):
            out = np.zeros((64, 9))
            t2 = hf_class if hf_class is not None else int(g["t2"][k])
            args = [np.ascontiguousarray(g[pre + x][k], dtype=np.float64) for x in ("p2", "pos2", "R2")]
            hn[k] = f(C.byref(H), t2, *(a.ctypes.data_as(P) for a in args), int(g[pre + "flags"][k]),
                      out.ctypes.data_as(P))
            ho[k] = out[:8]
        g[pre + "nc_s"], g[pre + "out_s"] = hn, ho
    np.savez_compressed(path, **g)


def make_tower():
    """Non-chaotic stacks (boxes of decreasing size, aligned): FP64 reference
    states after 200 steps plus the reference's own FP32 (dSINGLE) build on the
    same scene, whose drift from FP64 sets the achievable FP32 bar."""
    sc = S.box_tower(n_worlds=6, yaw=0.0, spacing=0.0)
    out = dict(sc.to_arrays())
    out["n_steps"] = np.int64(200)
    for w in range(sc.n_worlds):
        d = O.run_world(O.ref("d").ref_run_world, sc, w, 200)
        s_ = O.run_world(O.ref("s").ref_run_world, sc, w, 200)
        out[f"w{w}_final_d"] = d["state"][-1]
        out[f"w{w}_final_s"] = s_["state"][-1]
        out[f"w{w}_ncontacts"] = d["ncontacts"]
    np.savez_compressed(os.path.join(HERE, "tower.npz"), **out)


def make_space_order(seeds=range(8), n_steps=6):
    """The reference's dSINGLE build through its public space API
    (tests/space_program.py step_program): per step, the simple space's member
    order and the near-callback's pairs, with the geoms of every stepped body
    notified in island order by dWorldQuickStep and by dWorldStep."""
    import ctypes as C
    import space_program as SP
    lib = SP.bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))
    out = {"seeds": np.array(list(seeds)), "n_steps": np.int64(n_steps)}
    for st in ("dWorldQuickStep", "dWorldStep"):
        for s in seeds:
            out[f"{st}_{s}"] = SP.step_program(lib, s, n_steps, st)
    np.savez_compressed(os.path.join(HERE, "space_order.npz"), **out)


def make_body_step_options(seeds=(1, 2, 3), n_steps=30):
    """The reference's dSINGLE build through its public API
    (tests/body_step_program.py): damping, the angular speed cap and finite
    rotation over a smooth 30-step flight, the getters, and the moved
    callbacks' order, for dWorldQuickStep and dWorldStep; and the island
    program (null joints, disabled bodies): RNG seeds, enabled flags, states."""
    import ctypes as C
    import body_step_program as BP
    lib = BP.bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))
    out = {"seeds": np.array(seeds), "n_steps": np.int64(n_steps)}
    for st in ("dWorldQuickStep", "dWorldStep"):
        for s in seeds:
            g, x, m = BP.program(lib, s, n_steps, st)
            out[f"{st}_{s}_getters"], out[f"{st}_{s}_states"], out[f"{st}_{s}_moved"] = g, x, m
    for st in ("dWorldQuickStep", "dWorldStep"):
        for s in seeds:
            r = BP.island_program(BP.bind_islands(lib), s, 12, st)
            for k, v in zip(("seeds", "enabled", "states", "moved", "kept_force"), r):
                out[f"islands_{st}_{s}_{k}"] = v
    for st in ("dWorldQuickStep", "dWorldStep"):
        for s in seeds:
            k, x = BP.kinematic_program(BP.bind_islands(lib), s, 20, st)
            out[f"kinematic_{st}_{s}_flags"], out[f"kinematic_{st}_{s}_states"] = k, x
    np.savez_compressed(os.path.join(HERE, "body_step_options.npz"), **out)


def make_rng_kat():
    ref = O.ref("d")
    seeds = [0, 1, 12345, 0xdeadbeef, 0xffffffff]
    ns = [1, 2, 3, 4, 5, 16, 17, 100, 256, 257, 1000, 65536, 65537, 1000000]
    vals = []
    for s in seeds:
        ref.ref_rand_set_seed(s)
        vals.append([ref.ref_rand_int(n) for n in ns for _ in range(7)])
    np.savez_compressed(os.path.join(HERE, "rng_kat.npz"), seeds=np.array(seeds, np.uint32),
                        ns=np.array(ns), vals=np.array(vals))


if __name__ == "__main__":
    assert O.ref_available("d"), "build the reference first: make -C oracle ref"
    only = sys.argv[1:]
    if only:
        for name in only:
            if name == "ray_kats":
                make_ray_kats()
            elif name == "cylinder_kats":
                make_cylinder_kats()
                add_single_outputs("cylinder_kats", hf_class=3)
            elif name.startswith("exact_"):
                make_scene(name[len("exact_"):], exact=True)
            elif name == "hf_big_kats":
                make_hf_big_kats()
            elif name == "space_order":
                make_space_order()
            elif name == "body_step_options":
                make_body_step_options()
            elif name == "single_outputs":
                add_single_outputs("collider_kats")
                add_single_outputs("hf_kats")
                add_single_outputs("ray_kats", hf_class=5)
                add_single_outputs("cylinder_kats", hf_class=3)
            else:
                make_scene(name)
            print("wrote", name)
        sys.exit(0)
    for name in SCENES:
        make_scene(name)
        print("wrote", name)
    for name in EXACT_SCENES:
        make_scene(name, exact=True)
        print("wrote exact_" + name)
    make_collider_kats()
    make_hf_kats()
    make_ray_kats()
    make_cylinder_kats()
    make_hf_big_kats()
    add_single_outputs("collider_kats")
    add_single_outputs("hf_kats")
    add_single_outputs("ray_kats", hf_class=5)
    add_single_outputs("cylinder_kats", hf_class=3)
    make_rng_kat()
    make_tower()
    make_space_order()
    make_body_step_options()
    print("wrote collider_kats, rng_kat")
