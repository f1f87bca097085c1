"""A seeded program over ODE's body-update options (damping, the angular speed
cap, finite rotation with and without an axis, moved callbacks), run through
ctypes on libodegpu or on the reference's dSINGLE build. Bodies spin and fall
without contacts, some joined by a ball joint, so the trajectories are smooth
and the two libraries agree to FP32 rounding. Returns the getters' answers
and the body states after each step."""
import ctypes as C

import numpy as np

F, P, I = C.c_float, C.c_void_p, C.c_int
MOVED = C.CFUNCTYPE(None, P)


def bind(lib):
    for n in ("dWorldCreate", "dBodyCreate", "dJointCreateBall", "dBodyGetFirstGeom", "dBodyGetNextGeom",
              "dCreateSphere"):
        getattr(lib, n).restype = P
    lib.dInitODE2.argtypes = [C.c_uint]
    lib.dBodyCreate.argtypes = [P]
    for n in ("dBodySetPosition", "dBodySetLinearVel", "dBodySetAngularVel", "dBodySetFiniteRotationAxis",
              "dWorldSetGravity"):
        getattr(lib, n).argtypes = [P, F, F, F]
    for n in ("dWorldSetLinearDamping", "dWorldSetAngularDamping", "dWorldSetLinearDampingThreshold",
              "dWorldSetAngularDampingThreshold", "dWorldSetMaxAngularSpeed", "dBodySetLinearDamping",
              "dBodySetAngularDamping", "dBodySetLinearDampingThreshold", "dBodySetAngularDampingThreshold",
              "dBodySetMaxAngularSpeed"):
        getattr(lib, n).argtypes = [P, F]
    lib.dWorldSetDamping.argtypes = lib.dBodySetDamping.argtypes = [P, F, F]
    for n in ("dWorldGetLinearDamping", "dWorldGetAngularDamping", "dWorldGetLinearDampingThreshold",
              "dWorldGetAngularDampingThreshold", "dWorldGetMaxAngularSpeed", "dBodyGetLinearDamping",
              "dBodyGetAngularDamping", "dBodyGetLinearDampingThreshold", "dBodyGetAngularDampingThreshold",
              "dBodyGetMaxAngularSpeed"):
        getattr(lib, n).restype = F
        getattr(lib, n).argtypes = [P]
    lib.dBodySetFiniteRotationMode.argtypes = [P, I]
    lib.dBodyGetFiniteRotationMode.argtypes = [P]
    lib.dBodyGetFiniteRotationAxis.argtypes = [P, P]
    lib.dBodySetDampingDefaults.argtypes = [P]
    lib.dBodySetMovedCallback.argtypes = [P, MOVED]
    lib.dBodyGetFirstGeom.argtypes = [P]
    lib.dBodyGetNextGeom.argtypes = [P]
    lib.dCreateSphere.argtypes = [P, F]
    lib.dGeomSetBody.argtypes = [P, P]
    lib.dBodySetMass.argtypes = [P, P]
    lib.dMassSetBox.argtypes = [P, F, F, F, F]
    for n in ("dBodyGetPosition", "dBodyGetQuaternion", "dBodyGetLinearVel", "dBodyGetAngularVel"):
        getattr(lib, n).restype = C.POINTER(F)
        getattr(lib, n).argtypes = [P]
    lib.dJointCreateBall.argtypes = [P, P]
    lib.dJointAttach.argtypes = [P, P, P]
    lib.dJointSetBallAnchor.argtypes = [P, F, F, F]
    lib.dWorldQuickStep.argtypes = lib.dWorldStep.argtypes = [P, F]
    lib.dWorldDestroy.argtypes = [P]
    return lib


class Mass(C.Structure):
    _fields_ = [("mass", F), ("c", F * 4), ("I", F * 12)]


def state(lib, b):
    out = []
    for n, k in (("dBodyGetPosition", 3), ("dBodyGetQuaternion", 4), ("dBodyGetLinearVel", 3),
                 ("dBodyGetAngularVel", 3)):
        p = getattr(lib, n)(b)
        out += [p[i] for i in range(k)]
    return out


def program(lib, seed, n_steps=30, stepper="dWorldQuickStep"):
    """Returns (getters, states [n_steps][nb][13], moved-callback order)."""
    rng = np.random.default_rng(seed)
    lib.dInitODE2(0)
    w = lib.dWorldCreate()
    lib.dWorldSetGravity(w, 0.0, 0.0, -9.81)
    getters = []
    # world defaults, then the world's damping (bodies created afterwards take it)
    getters += [lib.dWorldGetLinearDamping(w), lib.dWorldGetAngularDampingThreshold(w),
                lib.dWorldGetMaxAngularSpeed(w)]
    lib.dWorldSetDamping(w, 0.01, 0.02)
    lib.dWorldSetLinearDampingThreshold(w, 0.5)
    lib.dWorldSetAngularDampingThreshold(w, 0.25)
    lib.dWorldSetMaxAngularSpeed(w, 12.0)
    bodies = []
    for k in range(8):
        b = lib.dBodyCreate(w)
        m = Mass()
        lib.dMassSetBox(C.byref(m), 1.0, *(float(x) for x in rng.uniform(0.2, 1.0, 3)))
        lib.dBodySetMass(b, C.byref(m))
        lib.dBodySetPosition(b, float(2 * k), 0.0, 5.0)
        lib.dBodySetLinearVel(b, *(float(x) for x in rng.normal(0, 2, 3)))
        lib.dBodySetAngularVel(b, *(float(x) for x in rng.normal(0, 8, 3)))
        bodies.append(b)
    b = bodies
    # per-body options over the world's
    lib.dBodySetDamping(b[1], 0.0, 0.0)                 # damping off
    lib.dBodySetLinearDamping(b[2], 0.05)
    lib.dBodySetAngularDampingThreshold(b[2], 100.0)    # above its speed: no angular damping
    lib.dBodySetMaxAngularSpeed(b[3], float("inf"))     # cap off
    lib.dBodySetMaxAngularSpeed(b[4], 3.0)
    for bb in b[5:]:                                    # fast spin, uncapped: finite rotation shows
        lib.dBodySetMaxAngularSpeed(bb, float("inf"))
        lib.dBodySetAngularVel(bb, *(float(x) for x in rng.normal(0, 25, 3)))
    lib.dBodySetFiniteRotationMode(b[5], 1)             # finite about w
    lib.dBodySetFiniteRotationAxis(b[6], 0.0, 0.0, 2.0) # axis first (normalised), then the mode
    lib.dBodySetFiniteRotationMode(b[6], 1)
    lib.dBodySetFiniteRotationMode(b[7], 1)
    lib.dBodySetFiniteRotationAxis(b[7], *(float(x) for x in rng.normal(size=3)))
    lib.dBodySetLinearDamping(b[0], 0.03)
    lib.dBodySetDampingDefaults(b[0])                   # back to the world's
    ax = (F * 4)()
    for bb in b:
        lib.dBodyGetFiniteRotationAxis(bb, ax)
        getters += [lib.dBodyGetLinearDamping(bb), lib.dBodyGetAngularDamping(bb),
                    lib.dBodyGetLinearDampingThreshold(bb), lib.dBodyGetAngularDampingThreshold(bb),
                    lib.dBodyGetMaxAngularSpeed(bb), lib.dBodyGetFiniteRotationMode(bb)] + list(ax)[:3]
    # two bodies joined by a ball joint form one island
    j = lib.dJointCreateBall(w, None)
    lib.dJointAttach(j, b[3], b[4])
    lib.dJointSetBallAnchor(j, 7.0, 0.0, 5.0)
    # body geom lists and moved callbacks
    g1, g2 = lib.dCreateSphere(None, 0.1), lib.dCreateSphere(None, 0.2)
    lib.dGeomSetBody(g1, b[2])
    lib.dGeomSetBody(g2, b[2])
    getters += [int(lib.dBodyGetFirstGeom(b[2]) == g2), int(lib.dBodyGetNextGeom(g2) == g1),
                int(lib.dBodyGetNextGeom(g1) is None), int(lib.dBodyGetFirstGeom(b[0]) is None)]
    ix = {bb: k for k, bb in enumerate(b)}
    moved = []
    cb = MOVED(lambda p: moved.append(ix.get(p, -1)))
    for bb in b:
        lib.dBodySetMovedCallback(bb, cb)
    states = []
    for _ in range(n_steps):
        getattr(lib, stepper)(w, 0.01)
        states.append([state(lib, bb) for bb in b])
    lib.dWorldDestroy(w)
    return (np.array(getters, dtype=np.float64), np.array(states, dtype=np.float64),
            np.array(moved, dtype=np.int64))


class Surface(C.Structure):
    _fields_ = [("mode", I), ("mu", F), ("mu2", F), ("bounce", F), ("bounce_vel", F), ("soft_erp", F),
                ("soft_cfm", F), ("motion1", F), ("motion2", F), ("motionN", F), ("slip1", F), ("slip2", F)]


class ContactGeom(C.Structure):
    _fields_ = [("pos", F * 4), ("normal", F * 4), ("depth", F), ("g1", P), ("g2", P), ("side1", I),
                ("side2", I)]


class Contact(C.Structure):
    _fields_ = [("surface", Surface), ("geom", ContactGeom), ("fdir1", F * 4)]


def bind_islands(lib):
    bind(lib)
    for n in ("dJointCreateNull", "dJointGroupCreate", "dJointCreateContact"):
        getattr(lib, n).restype = P
    lib.dJointCreateNull.argtypes = [P, P]
    lib.dJointGroupCreate.argtypes = [I]
    lib.dJointCreateContact.argtypes = [P, P, P]
    lib.dJointGroupEmpty.argtypes = lib.dJointGroupDestroy.argtypes = [P]
    lib.dBodyEnable.argtypes = lib.dBodyDisable.argtypes = lib.dBodyIsEnabled.argtypes = [P]
    lib.dRandSetSeed.argtypes = [C.c_ulong]
    lib.dRandGetSeed.restype = C.c_ulong
    lib.dBodySetForce.argtypes = [P, F, F, F]
    lib.dBodyGetForce.restype = C.POINTER(F)
    lib.dBodyGetForce.argtypes = [P]
    return lib


def island_program(lib, seed, n_steps=12, stepper="dWorldQuickStep"):
    """Boxes resting on ground contacts (depth 0.01, friction), linked by ball
    and null joints, some disabled: a null joint merges two islands, a
    disabled body joined to an enabled one is woken, disabled bodies joined
    only to each other or to the ground stay put with their forces kept.
    Returns per step the RNG seed (its draws follow every island's row count),
    the enabled flags, the states and the moved-callback order."""
    rng = np.random.default_rng(seed)
    lib.dInitODE2(0)
    lib.dRandSetSeed(1234 + seed)
    w = lib.dWorldCreate()
    lib.dWorldSetGravity(w, 0.0, 0.0, -9.81)
    b = []
    for k in range(9):
        bb = lib.dBodyCreate(w)
        m = Mass()
        lib.dMassSetBox(C.byref(m), 1.0, 0.5, 0.5, 0.5)
        lib.dBodySetMass(bb, C.byref(m))
        lib.dBodySetPosition(bb, float(k), 0.0, 0.25 + 0.01 * float(rng.random()))
        lib.dBodySetLinearVel(bb, *(float(x) for x in rng.normal(0, 0.2, 3)))
        b.append(bb)
    order = [int(x) for x in rng.permutation(9)]
    links = [("ball", 0, 1), ("null", 2, 3), ("null", 4, 6), ("ball", 7, 8), ("null", 3, 0)]
    for kind, i, k in links:
        j = (lib.dJointCreateBall if kind == "ball" else lib.dJointCreateNull)(w, None)
        lib.dJointAttach(j, b[i], b[k])
        if kind == "ball":
            lib.dJointSetBallAnchor(j, 0.5 * (i + k), 0.0, 0.25)
    lib.dBodyDisable(b[6])          # joined to b4 by a null joint: woken
    lib.dBodyDisable(b[7])          # joined only to b8 ...
    lib.dBodyDisable(b[8])          # ... both disabled: they stay
    lib.dBodyDisable(b[5])          # a ground contact only: stays
    lib.dBodySetForce(b[5], 1.0, 2.0, 3.0)
    grp = lib.dJointGroupCreate(0)
    ix = {bb: k for k, bb in enumerate(b)}
    moved = []
    cb = MOVED(lambda p: moved.append(ix.get(p, -1)))
    for bb in b:
        lib.dBodySetMovedCallback(bb, cb)
    seeds, flags, states = [], [], []
    for _ in range(n_steps):
        lib.dJointGroupEmpty(grp)
        for k in order:           # ground contacts, created in a shuffled order
            c = Contact()
            c.surface.mode = 0
            c.surface.mu = 0.5
            p = lib.dBodyGetPosition(b[k])
            c.geom.pos[0], c.geom.pos[1], c.geom.pos[2] = p[0], p[1], 0.0
            c.geom.normal[2] = 1.0
            c.geom.depth = 0.01
            j = lib.dJointCreateContact(w, grp, C.byref(c))
            lib.dJointAttach(j, b[k], None)
        getattr(lib, stepper)(w, 0.01)
        seeds.append(lib.dRandGetSeed())
        flags.append([lib.dBodyIsEnabled(bb) for bb in b])
        states.append([state(lib, bb) for bb in b])
    f5 = lib.dBodyGetForce(b[5])
    kept = [f5[0], f5[1], f5[2]]
    lib.dJointGroupDestroy(grp)
    lib.dWorldDestroy(w)
    return (np.array(seeds, dtype=np.int64), np.array(flags, dtype=np.int64), np.array(states, dtype=np.float64),
            np.array(moved, dtype=np.int64), np.array(kept, dtype=np.float64))


def kinematic_program(lib, seed, n_steps=20, stepper="dWorldQuickStep"):
    """A kinematic box (ode.cpp:834-852: zero inverse mass and inertia) moving
    and spinning at set velocities, a dynamic box hanging on it by a ball
    joint under gravity, and a second dynamic box on a ground contact. The
    kinematic body keeps its velocities and moves by them; the others follow.
    Returns the IsKinematic answers and the states after each step."""
    rng = np.random.default_rng(seed)
    lib.dInitODE2(0)
    for n in ("dBodySetKinematic", "dBodySetDynamic", "dBodyIsKinematic"):
        getattr(lib, n).argtypes = [P]
    w = lib.dWorldCreate()
    lib.dWorldSetGravity(w, 0.0, 0.0, -9.81)
    b = []
    for k in range(3):
        bb = lib.dBodyCreate(w)
        m = Mass()
        lib.dMassSetBox(C.byref(m), 1.0, *(float(x) for x in rng.uniform(0.3, 0.8, 3)))
        lib.dBodySetMass(bb, C.byref(m))
        lib.dBodySetPosition(bb, float(k), 0.0, 1.0 + 0.5 * k)
        b.append(bb)
    got = [lib.dBodyIsKinematic(b[0])]
    lib.dBodySetKinematic(b[0])
    lib.dBodySetLinearVel(b[0], 1.0, 0.2, 0.0)
    lib.dBodySetAngularVel(b[0], 0.0, 0.0, 0.5)
    lib.dBodySetKinematic(b[2])
    lib.dBodySetDynamic(b[2])                  # back to its mass
    got += [lib.dBodyIsKinematic(b[0]), lib.dBodyIsKinematic(b[2])]
    j = lib.dJointCreateBall(w, None)
    lib.dJointAttach(j, b[0], b[1])
    lib.dJointSetBallAnchor(j, 0.5, 0.0, 1.25)
    grp = lib.dJointGroupCreate(0)
    states = []
    for _ in range(n_steps):
        lib.dJointGroupEmpty(grp)
        c = Contact()
        c.surface.mu = 0.5
        p = lib.dBodyGetPosition(b[2])
        c.geom.pos[0], c.geom.pos[1], c.geom.pos[2] = p[0], p[1], p[2] - 0.2
        c.geom.normal[2] = 1.0
        c.geom.depth = 0.02
        jc = lib.dJointCreateContact(w, grp, C.byref(c))
        lib.dJointAttach(jc, b[2], b[0])       # a contact with the kinematic body too
        getattr(lib, stepper)(w, 0.01)
        states.append([state(lib, bb) for bb in b])
    lib.dJointGroupDestroy(grp)
    lib.dWorldDestroy(w)
    return np.array(got, dtype=np.int64), np.array(states, dtype=np.float64)
