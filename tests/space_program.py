"""Seeded programs over ODE's space API (include/ode/collision_space.h), run
through ctypes on any library that exports it: libodegpu, or the reference's
dSINGLE build. Each program returns what a near-callback and the space
getters observe, as geom indices: the order of the (g1, g2) pairs dSpaceCollide
and dSpaceCollide2 pass, and each space's member order. Nothing here calls
dCollide, so the programs without world steps run without a GPU."""
import ctypes as C

import numpy as np

F, P, I, UL = C.c_float, C.c_void_p, C.c_int, C.c_ulong
NEAR = C.CFUNCTYPE(None, P, P, P)


def bind(lib):
    for n in ("dWorldCreate", "dBodyCreate", "dCreateSphere", "dCreateBox", "dCreateCapsule", "dCreateCylinder",
              "dCreatePlane", "dCreateRay", "dSimpleSpaceCreate", "dHashSpaceCreate", "dSpaceGetGeom",
              "dGeomGetSpace", "dJointCreateBall", "dJointCreateContact", "dJointGroupCreate"):
        getattr(lib, n).restype = P
    lib.dInitODE2.argtypes = [C.c_uint]
    lib.dBodyCreate.argtypes = [P]
    lib.dBodySetPosition.argtypes = [P, F, F, F]
    lib.dBodySetQuaternion.argtypes = [P, P]
    lib.dCreateSphere.argtypes = [P, F]
    lib.dCreateBox.argtypes = [P, F, F, F]
    lib.dCreateCapsule.argtypes = lib.dCreateCylinder.argtypes = [P, F, F]
    lib.dCreatePlane.argtypes = [P, F, F, F, F]
    lib.dCreateRay.argtypes = [P, F]
    lib.dSimpleSpaceCreate.argtypes = lib.dHashSpaceCreate.argtypes = [P]
    lib.dHashSpaceSetLevels.argtypes = [P, I, I]
    lib.dSpaceAdd.argtypes = lib.dSpaceRemove.argtypes = lib.dSpaceQuery.argtypes = [P, P]
    lib.dSpaceGetGeom.argtypes = [P, I]
    for n in ("dSpaceGetNumGeoms", "dSpaceClean", "dSpaceDestroy", "dSpaceGetClass", "dGeomGetSpace",
              "dGeomIsSpace", "dGeomEnable", "dGeomDisable", "dGeomDestroy", "dSpaceGetCleanup"):
        getattr(lib, n).argtypes = [P]
    lib.dSpaceSetCleanup.argtypes = lib.dSpaceSetSublevel.argtypes = [P, I]
    lib.dSpaceCollide.argtypes = [P, P, NEAR]
    lib.dSpaceCollide2.argtypes = [P, P, P, NEAR]
    lib.dGeomSetBody.argtypes = [P, P]
    lib.dGeomSetPosition.argtypes = [P, F, F, F]
    lib.dGeomSetQuaternion.argtypes = [P, P]
    lib.dGeomSetOffsetPosition.argtypes = [P, F, F, F]
    lib.dGeomSetCategoryBits.argtypes = lib.dGeomSetCollideBits.argtypes = [P, UL]
    lib.dGeomSphereSetRadius.argtypes = [P, F]
    lib.dGeomBoxSetLengths.argtypes = [P, F, F, F]
    lib.dGeomGetAABB.argtypes = [P, P]
    lib.dGeomGetPosition.restype = C.POINTER(F)
    lib.dGeomGetPosition.argtypes = [P]
    lib.dWorldSetGravity.argtypes = [P, F, F, F]
    lib.dWorldQuickStep.argtypes = lib.dWorldStep.argtypes = [P, F]
    lib.dWorldDestroy.argtypes = [P]
    lib.dJointCreateBall.argtypes = [P, P]
    lib.dJointGroupCreate.argtypes = [I]
    lib.dJointCreateContact.argtypes = [P, P, P]
    lib.dJointAttach.argtypes = [P, P, P]
    lib.dJointSetBallAnchor.argtypes = [P, F, F, F]
    lib.dJointGroupDestroy.argtypes = [P]
    return lib


class _Ids:
    """Pointer -> creation index, so two libraries' records compare."""

    def __init__(self):
        self.ix = {}

    def add(self, p):
        self.ix[p] = len(self.ix)
        return p

    def __call__(self, p):
        return -1 if p is None else self.ix.get(p, -2)


def _quat(a):
    q = np.array(a, dtype=np.float64)
    q /= np.linalg.norm(q)
    return (F * 4)(*q.astype(np.float32))


def _order(lib, ids, sp):
    return [ids(lib.dSpaceGetGeom(sp, i)) for i in range(lib.dSpaceGetNumGeoms(sp))]


def ops_program(lib, seed, kind="hash", n_ops=60):
    """Random edits between collides: geoms of every class in a simple or hash
    space (and a nested simple space), on bodies or free, moved by body and
    geom setters and offsets, resized (to zero too), disabled, re-bitted,
    removed and added back. Returns a flat int64 record."""
    rng = np.random.default_rng(seed)
    ids = _Ids()
    rec = []
    pairs = []
    cb = NEAR(lambda d, a, b: pairs.append((ids(a), ids(b))))
    lib.dInitODE2(0)
    w = lib.dWorldCreate()
    if kind == "sap":
        lib.dSweepAndPruneSpaceCreate.restype = P
        lib.dSweepAndPruneSpaceCreate.argtypes = [P, I]
        axes = [0 | (1 << 2) | (2 << 4), 2 | (1 << 2) | (0 << 4), 1 | (2 << 2) | (0 << 4)][seed % 3]
        top = ids.add(lib.dSweepAndPruneSpaceCreate(None, axes))
    else:
        top = ids.add((lib.dHashSpaceCreate if kind == "hash" else lib.dSimpleSpaceCreate)(None))
    if kind == "hash":
        lib.dHashSpaceSetLevels(top, int(rng.integers(-4, 0)), int(rng.integers(1, 6)))
    sub = ids.add(lib.dSimpleSpaceCreate(top))
    bodies = []
    for _ in range(5):
        b = lib.dBodyCreate(w)
        lib.dBodySetPosition(b, *(rng.uniform(-2, 2, 3)))
        bodies.append(b)
    geoms = []

    def make(space):
        c = int(rng.integers(0, 6))
        if c == 0:
            g = lib.dCreateSphere(space, float(rng.uniform(0.1, 0.8)))
        elif c == 1:
            g = lib.dCreateBox(space, *(rng.uniform(0.1, 1.2, 3)))
        elif c == 2:
            g = lib.dCreateCapsule(space, float(rng.uniform(0.1, 0.5)), float(rng.uniform(0.2, 1.5)))
        elif c == 3:
            g = lib.dCreateCylinder(space, float(rng.uniform(0.1, 0.5)), float(rng.uniform(0.2, 1.5)))
        elif c == 4:
            g = lib.dCreateRay(space, float(rng.uniform(0.5, 3.0)))
        else:
            g = lib.dCreatePlane(space, 0.0, 0.0, 1.0, float(rng.uniform(-3, 0)))
        ids.add(g)
        if c != 5:
            if rng.random() < 0.5:
                lib.dGeomSetBody(g, bodies[int(rng.integers(0, len(bodies)))])
                if rng.random() < 0.3:
                    lib.dGeomSetOffsetPosition(g, *(rng.uniform(-0.5, 0.5, 3)))
            else:
                lib.dGeomSetPosition(g, *(rng.uniform(-3, 3, 3)))
                lib.dGeomSetQuaternion(g, _quat(rng.normal(size=4)))
        geoms.append((g, c))

    for _ in range(14):
        make(top if rng.random() < 0.75 else sub)
    removed = []
    for _ in range(n_ops):
        op = int(rng.integers(0, 12))
        g, c = geoms[int(rng.integers(0, len(geoms)))]
        if op == 0:
            lib.dBodySetPosition(bodies[int(rng.integers(0, len(bodies)))], *(rng.uniform(-3, 3, 3)))
        elif op == 1:
            lib.dBodySetQuaternion(bodies[int(rng.integers(0, len(bodies)))], _quat(rng.normal(size=4)))
        elif op == 2 and c != 5:
            lib.dGeomSetPosition(g, *(rng.uniform(-3, 3, 3)))
        elif op == 3:
            (lib.dGeomDisable if rng.random() < 0.5 else lib.dGeomEnable)(g)
        elif op == 4:
            lib.dGeomSetCategoryBits(g, int(rng.integers(0, 8)))
            lib.dGeomSetCollideBits(g, int(rng.integers(0, 8)))
        elif op == 5 and c == 0:
            lib.dGeomSphereSetRadius(g, float(rng.choice([0.0, 0.3, 0.9])))
        elif op == 5 and c == 1:
            lib.dGeomBoxSetLengths(g, float(rng.choice([0.0, 0.5])), 0.6, 0.7)
        elif op == 6:
            sp = lib.dGeomGetSpace(g)
            if sp is not None:
                lib.dSpaceRemove(sp, g)
                removed.append(g)
        elif op == 7 and removed:
            lib.dSpaceAdd(top if rng.random() < 0.7 else sub, removed.pop(0))
        elif op == 8:
            make(top if rng.random() < 0.75 else sub)
        elif op == 9:
            pairs.clear()
            lib.dSpaceCollide(top, None, cb)
            rec += [len(pairs)] + [x for pr in pairs for x in pr]
        elif op == 10:
            pairs.clear()
            lib.dSpaceCollide2(top, g, None, cb)
            lib.dSpaceCollide2(g, sub, None, cb)
            lib.dSpaceCollide2(sub, top, None, cb)
            rec += [len(pairs)] + [x for pr in pairs for x in pr]
        elif op == 11 and c != 5:
            # ODE 0.12 keeps GEOM_POSR_BAD when dGeomSetBody moves an offset
            # geom to another body, and its next pose read then follows the
            # freed offset (collision_kernel.cpp:507-528, :454-465); reading
            # the pose first keeps the reference clear of that
            lib.dGeomGetPosition(g)
            lib.dGeomSetBody(g, bodies[int(rng.integers(0, len(bodies)))] if rng.random() < 0.7 else None)
        rec += _order(lib, ids, top) + [-9] + _order(lib, ids, sub) + [-9]
    pairs.clear()
    lib.dSpaceCollide(top, None, cb)
    lib.dSpaceCollide(sub, None, cb)
    rec += [len(pairs)] + [x for pr in pairs for x in pr]
    rec += [lib.dSpaceGetNumGeoms(top), lib.dSpaceGetNumGeoms(sub), lib.dSpaceGetClass(top),
            lib.dSpaceGetClass(sub), lib.dGeomIsSpace(sub), ids(lib.dGeomGetSpace(sub)),
            lib.dSpaceQuery(top, sub), lib.dSpaceQuery(sub, sub)]
    box = (F * 6)()
    lib.dGeomGetAABB(sub, box)
    aabb = list(box)
    for g in removed:
        lib.dGeomDestroy(g)
    lib.dSpaceDestroy(top)   # cleanup on: takes sub and every geom with it
    lib.dWorldDestroy(w)
    return np.array(rec, dtype=np.int64), np.array(aabb, dtype=np.float32)


def step_program(lib, seed, n_steps=6, stepper="dWorldQuickStep"):
    """Bodies at rest without gravity, with geoms in a simple space, joined by
    ball joints and depth-0 contact joints attached in shuffled order: a step
    moves nothing, but notifies every body's geoms in island order, which
    reorders the space. Returns per step the space's order and the near
    callback's pairs. The callback calls no collider."""
    rng = np.random.default_rng(seed)
    ids = _Ids()
    rec = []
    pairs = []
    cb = NEAR(lambda d, a, b: pairs.append((ids(a), ids(b))))
    lib.dInitODE2(0)
    w = lib.dWorldCreate()
    lib.dWorldSetGravity(w, 0.0, 0.0, 0.0)
    sp = ids.add(lib.dSimpleSpaceCreate(None))
    grp = lib.dJointGroupCreate(0)
    nb = 12
    bodies = []
    for k in range(nb):
        b = lib.dBodyCreate(w)
        # a 4 x 3 grid, 1 m apart: spheres of radius 0.6 overlap their
        # neighbours' boxes by 0.2 m, far from any rounding
        lib.dBodySetPosition(b, float(k % 4), float(k // 4), 0.0)
        bodies.append(b)
    order = rng.permutation(nb)
    for k in order:
        g = ids.add(lib.dCreateSphere(sp, 0.6))
        lib.dGeomSetBody(g, bodies[int(k)])
        if rng.random() < 0.3:
            g2 = ids.add(lib.dCreateBox(sp, 0.3, 0.3, 0.3))
            lib.dGeomSetBody(g2, bodies[int(k)])
    ids.add(lib.dCreatePlane(sp, 0.0, 0.0, 1.0, -5.0))
    free = ids.add(lib.dCreateSphere(sp, 0.6))
    lib.dGeomSetPosition(free, 1.5, 0.5, 0.0)
    links = [(int(a), int(b)) for a, b in rng.integers(0, nb, size=(7, 2)) if a != b]
    for a, b in links[:4]:
        j = lib.dJointCreateBall(w, None)
        lib.dJointAttach(j, bodies[a], bodies[b])
        lib.dJointSetBallAnchor(j, 0.5 * (a % 4 + b % 4), 0.5 * (a // 4 + b // 4), 0.0)
    contact = (C.c_byte * 256)()   # dContact, zeroed: mode 0, mu 0, depth 0
    for a, b in links[4:]:
        j = lib.dJointCreateContact(w, grp, contact)
        lib.dJointAttach(j, bodies[a], bodies[b] if rng.random() < 0.8 else None)
    rec += _order(lib, ids, sp) + [-9]
    for _ in range(n_steps):
        pairs.clear()
        lib.dSpaceCollide(sp, None, cb)
        rec += [len(pairs)] + [x for pr in pairs for x in pr]
        ok = getattr(lib, stepper)(w, 0.01)
        rec += [int(ok)] + _order(lib, ids, sp) + [-9]
    lib.dJointGroupDestroy(grp)
    lib.dSpaceDestroy(sp)
    lib.dWorldDestroy(w)
    return np.array(rec, dtype=np.int64)


def quad_program(lib, seed, n_ops=60):
    """Random edits between collides in a quadtree space (center 0, extents 4,
    depth 3) holding geoms of every class, a nested simple space, geoms on
    bodies and free ones, moves (re-seated in their blocks when the space is
    cleaned), disabling, bits, removal and re-adding. ODE 0.12 does not
    enumerate a quadtree's geoms, so only the near-callback's pairs and the
    counts are recorded."""
    rng = np.random.default_rng(seed)
    ids = _Ids()
    rec = []
    pairs = []
    cb = NEAR(lambda d, a, b: pairs.append((ids(a), ids(b))))
    lib.dInitODE2(0)
    lib.dQuadTreeSpaceCreate.restype = P
    lib.dQuadTreeSpaceCreate.argtypes = [P, P, P, I]
    w = lib.dWorldCreate()
    center, extents = (F * 4)(0.0, 0.0, 0.0, 0.0), (F * 4)(4.0, 4.0, 4.0, 0.0)
    top = ids.add(lib.dQuadTreeSpaceCreate(None, center, extents, 3))
    sub = ids.add(lib.dSimpleSpaceCreate(top))
    bodies = []
    for _ in range(4):
        b = lib.dBodyCreate(w)
        lib.dBodySetPosition(b, *(rng.uniform(-3, 3, 3)))
        bodies.append(b)
    geoms = []

    def make(space):
        c = int(rng.integers(0, 6))
        if c == 0:
            g = lib.dCreateSphere(space, float(rng.uniform(0.1, 0.6)))
        elif c == 1:
            g = lib.dCreateBox(space, *(rng.uniform(0.1, 1.0, 3)))
        elif c == 2:
            g = lib.dCreateCapsule(space, float(rng.uniform(0.1, 0.4)), float(rng.uniform(0.2, 1.2)))
        elif c == 3:
            g = lib.dCreateCylinder(space, float(rng.uniform(0.1, 0.4)), float(rng.uniform(0.2, 1.2)))
        elif c == 4:
            g = lib.dCreateRay(space, float(rng.uniform(0.5, 2.5)))
        else:
            g = lib.dCreatePlane(space, 0.0, 0.0, 1.0, float(rng.uniform(-3, 0)))
        ids.add(g)
        if c != 5:
            if rng.random() < 0.4:
                lib.dGeomSetBody(g, bodies[int(rng.integers(0, len(bodies)))])
            else:
                lib.dGeomSetPosition(g, *(rng.uniform(-5, 5, 3)))
                lib.dGeomSetQuaternion(g, _quat(rng.normal(size=4)))
        geoms.append((g, c))

    for _ in range(16):
        make(top if rng.random() < 0.8 else sub)
    removed = []
    for _ in range(n_ops):
        op = int(rng.integers(0, 11))
        g, c = geoms[int(rng.integers(0, len(geoms)))]
        if op == 0:
            lib.dBodySetPosition(bodies[int(rng.integers(0, len(bodies)))], *(rng.uniform(-5, 5, 3)))
        elif op == 1 and c != 5:
            lib.dGeomSetPosition(g, *(rng.uniform(-5, 5, 3)))
        elif op == 2:
            (lib.dGeomDisable if rng.random() < 0.5 else lib.dGeomEnable)(g)
        elif op == 3:
            lib.dGeomSetCategoryBits(g, int(rng.integers(0, 8)))
            lib.dGeomSetCollideBits(g, int(rng.integers(0, 8)))
        elif op == 4:
            sp = lib.dGeomGetSpace(g)
            if sp is not None:
                lib.dSpaceRemove(sp, g)
                removed.append(g)
        elif op == 5 and removed:
            lib.dSpaceAdd(top if rng.random() < 0.7 else sub, removed.pop(0))
        elif op == 6:
            make(top if rng.random() < 0.8 else sub)
        elif op in (7, 8):
            pairs.clear()
            lib.dSpaceCollide(top, None, cb)
            rec += [len(pairs)] + [x for pr in pairs for x in pr]
        elif op == 9:
            pairs.clear()
            lib.dSpaceCollide2(top, g, None, cb)
            lib.dSpaceCollide2(g, top, None, cb)
            lib.dSpaceCollide2(sub, top, None, cb)
            rec += [len(pairs)] + [x for pr in pairs for x in pr]
        elif op == 10 and c != 5:
            lib.dGeomGetPosition(g)   # see ops_program: keeps the reference clear of its offset crash
            lib.dGeomSetBody(g, bodies[int(rng.integers(0, len(bodies)))] if rng.random() < 0.7 else None)
        rec += [lib.dSpaceGetNumGeoms(top), lib.dSpaceGetNumGeoms(sub)]
    pairs.clear()
    lib.dSpaceCollide(top, None, cb)
    rec += [len(pairs)] + [x for pr in pairs for x in pr]
    # (dSpaceGetGeom is left out: ODE 0.12 aborts in it for a quadtree)
    rec += [lib.dSpaceGetClass(top), lib.dSpaceQuery(top, sub)]
    box = (F * 6)()
    lib.dGeomGetAABB(top, box)
    rec += [float(x) for x in box]
    for g in removed:
        lib.dGeomDestroy(g)
    lib.dWorldDestroy(w)
    return np.array(rec, dtype=np.float64)


def sap_tie_program(lib, seed, n_rounds=12):
    """A sweep-and-prune space where many boxes share their lower bound on the
    sweep axis, negative ones included, collided again and again while a few
    move: the order of equal keys out of the radix sort, which depends on the
    previous sorts, sets the pair order."""
    rng = np.random.default_rng(seed)
    ids = _Ids()
    pairs = []
    cb = NEAR(lambda d, a, b: pairs.append((ids(a), ids(b))))
    lib.dInitODE2(0)
    lib.dSweepAndPruneSpaceCreate.restype = P
    lib.dSweepAndPruneSpaceCreate.argtypes = [P, I]
    sp = ids.add(lib.dSweepAndPruneSpaceCreate(None, 0 | (1 << 2) | (2 << 4)))
    xs = [-2.5, -1.0, -0.25, 0.0, 0.5, 1.75]
    geoms = []
    for _ in range(30):
        g = ids.add(lib.dCreateBox(sp, 1.0, float(rng.uniform(0.2, 1.0)), float(rng.uniform(0.2, 1.0))))
        lib.dGeomSetPosition(g, float(rng.choice(xs)), float(rng.uniform(-1, 1)), float(rng.uniform(-1, 1)))
        geoms.append(g)
    rec = []
    for _ in range(n_rounds):
        for g in rng.choice(len(geoms), size=3, replace=False):
            lib.dGeomSetPosition(geoms[int(g)], float(rng.choice(xs)), float(rng.uniform(-1, 1)),
                                 float(rng.uniform(-1, 1)))
        pairs.clear()
        lib.dSpaceCollide(sp, None, cb)
        rec += [len(pairs)] + [x for pr in pairs for x in pr] + _order(lib, ids, sp)
        pairs.clear()
        lib.dSpaceCollide(sp, None, cb)   # again with nothing moved: the previous order is kept
        rec += [len(pairs)] + [x for pr in pairs for x in pr]
    lib.dSpaceDestroy(sp)
    return np.array(rec, dtype=np.int64)
