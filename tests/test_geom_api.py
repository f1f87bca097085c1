"""ODE's geom placement API on the host, against the reference's dSINGLE build:
offsets from the body (ode/src/collision_kernel.cpp:1017-1250), the geom
pose setters and getters with and without offsets (:507-703), bounding boxes
of every class on this path (sphere.cpp:59-67, box.cpp:60-77,
capsule.cpp:60-74, cylinder.cpp:59-76, plane.cpp:80-107, ray.cpp:56-89,
heightfield.cpp:475-600), category / collide bits and the enabled flag
(:735-782), geom-frame points (:784-874), the class setters and point depths,
and dBodyDestroy's detach (ode.cpp:301-310). None of these calls reaches the
GPU, so the same call sequence runs on both libraries here."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F, P, I, UL = C.c_float, C.c_void_p, C.c_int, C.c_ulong
V4, M12 = F * 4, F * 12
dSphereClass, dBoxClass, dCapsuleClass, dCylinderClass, dPlaneClass, dRayClass = 0, 1, 2, 3, 4, 5


def _libs():
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    for lib in (ours, ref):
        for n in ("dWorldCreate", "dBodyCreate", "dCreateSphere", "dCreateBox", "dCreateCapsule", "dCreateCylinder",
                  "dCreatePlane", "dCreateRay", "dGeomGetBody", "dGeomGetSpace", "dCreateHeightfield",
                  "dGeomHeightfieldDataCreate"):
            getattr(lib, n).restype = P
        lib.dBodyCreate.argtypes = [P]
        lib.dBodySetPosition.argtypes = [P, F, F, F]
        lib.dBodySetRotation.argtypes = [P, P]
        lib.dBodyDestroy.argtypes = [P]
        lib.dBodyGetPosition.restype = lib.dBodyGetRotation.restype = C.POINTER(F)
        lib.dBodyGetPosition.argtypes = lib.dBodyGetRotation.argtypes = [P]
        lib.dRFromAxisAndAngle.argtypes = [P, F, F, F, F]
        lib.dQFromAxisAndAngle.argtypes = [P, F, F, F, F]
        lib.dCreateSphere.argtypes = [P, F]
        lib.dCreateBox.argtypes = [P, F, F, F]
        lib.dCreateCapsule.argtypes = lib.dCreateCylinder.argtypes = [P, F, F]
        lib.dCreatePlane.argtypes = [P, F, F, F, F]
        lib.dCreateRay.argtypes = [P, F]
        for n in ("dGeomSetBody",):
            getattr(lib, n).argtypes = [P, P]
        for n in ("dGeomSetPosition", "dGeomSetOffsetPosition", "dGeomSetOffsetWorldPosition"):
            getattr(lib, n).argtypes = [P, F, F, F]
        for n in ("dGeomSetRotation", "dGeomSetQuaternion", "dGeomSetOffsetRotation", "dGeomSetOffsetQuaternion",
                  "dGeomSetOffsetWorldRotation", "dGeomSetOffsetWorldQuaternion", "dGeomCopyPosition",
                  "dGeomCopyRotation", "dGeomGetQuaternion", "dGeomGetAABB", "dGeomCopyOffsetPosition",
                  "dGeomCopyOffsetRotation", "dGeomGetOffsetQuaternion"):
            getattr(lib, n).argtypes = [P, P]
        for n in ("dGeomGetPosition", "dGeomGetRotation", "dGeomGetOffsetPosition", "dGeomGetOffsetRotation"):
            getattr(lib, n).restype = C.POINTER(F)
            getattr(lib, n).argtypes = [P]
        for n in ("dGeomClearOffset", "dGeomIsOffset", "dGeomIsSpace", "dGeomGetSpace", "dGeomEnable",
                  "dGeomDisable", "dGeomIsEnabled", "dGeomDestroy", "dGeomGetCategoryBits", "dGeomGetCollideBits",
                  "dGeomGetBody", "dGeomGetClass"):
            getattr(lib, n).argtypes = [P]
        lib.dGeomGetCategoryBits.restype = lib.dGeomGetCollideBits.restype = UL
        lib.dGeomSetCategoryBits.argtypes = lib.dGeomSetCollideBits.argtypes = [P, UL]
        for n in ("dGeomGetRelPointPos", "dGeomGetPosRelPoint", "dGeomVectorToWorld", "dGeomVectorFromWorld"):
            getattr(lib, n).argtypes = [P, F, F, F, P]
        for n in ("dGeomSpherePointDepth", "dGeomBoxPointDepth", "dGeomPlanePointDepth", "dGeomCapsulePointDepth"):
            getattr(lib, n).restype = F
            getattr(lib, n).argtypes = [P, F, F, F]
        lib.dGeomSphereSetRadius.argtypes = [P, F]
        lib.dGeomBoxSetLengths.argtypes = [P, F, F, F]
        lib.dGeomPlaneSetParams.argtypes = [P, F, F, F, F]
        lib.dGeomCapsuleSetParams.argtypes = [P, F, F]
        lib.dGeomPlaneGetParams.argtypes = lib.dGeomBoxGetLengths.argtypes = [P, P]
        lib.dGeomSphereGetRadius.restype = F
        lib.dGeomSphereGetRadius.argtypes = [P]
        lib.dGeomCapsuleGetParams.argtypes = [P, P, P]
        lib.dGeomHeightfieldDataBuildSingle.argtypes = [P, P, I, F, F, I, I, F, F, F, I]
        lib.dGeomHeightfieldDataSetBounds.argtypes = [P, F, F]
        lib.dGeomHeightfieldDataDestroy.argtypes = [P]
        lib.dCreateHeightfield.argtypes = [P, P, I]
        lib.dWorldDestroy.argtypes = [P]
    return ours, ref


def _rot(lib, a):
    R = M12()
    lib.dRFromAxisAndAngle(R, *a)
    return R


def _quat(lib, a):
    q = V4()
    lib.dQFromAxisAndAngle(q, *a)
    return q


def _v3(p):
    return [p[k] for k in range(3)]


def _m9(p):
    return [p[r * 4 + c] for r in range(3) for c in range(3)]


def _out4(lib, fn, g):
    r = V4()
    fn(g, r)
    return list(r)


def _pose(lib, g):
    return _v3(lib.dGeomGetPosition(g)) + _m9(lib.dGeomGetRotation(g))


def _aabb(lib, g):
    a = (F * 6)()
    lib.dGeomGetAABB(g, a)
    return list(a)


def _points(lib, g, pts):
    out = []
    for name in ("dGeomGetRelPointPos", "dGeomGetPosRelPoint", "dGeomVectorToWorld", "dGeomVectorFromWorld"):
        for p in pts:
            r = V4()
            getattr(lib, name)(g, *p, r)
            out += list(r)[:3]
    return out


def _offset_sequence(lib, a):
    """Offsets, the offset-aware setters and getters, then detach."""
    out = []
    w = lib.dWorldCreate()
    b = lib.dBodyCreate(w)
    lib.dBodySetPosition(b, *a[0:3])
    lib.dBodySetRotation(b, _rot(lib, a[3:7]))
    g = lib.dCreateBox(None, abs(a[7]) + 0.2, abs(a[8]) + 0.2, abs(a[9]) + 0.2)
    lib.dGeomSetBody(g, b)
    out += [lib.dGeomIsOffset(g)] + _pose(lib, g) + _out4(lib, lib.dGeomGetQuaternion, g)
    lib.dGeomSetOffsetPosition(g, *a[10:13])
    lib.dGeomSetOffsetRotation(g, _rot(lib, a[13:17]))
    out += [lib.dGeomIsOffset(g)] + _pose(lib, g) + _out4(lib, lib.dGeomGetQuaternion, g)
    out += _out4(lib, lib.dGeomCopyOffsetPosition, g)[:3] + _v3(lib.dGeomGetOffsetPosition(g))
    out += _m9(lib.dGeomGetOffsetRotation(g)) + _out4(lib, lib.dGeomGetOffsetQuaternion, g)
    out += _aabb(lib, g) + _points(lib, g, [a[17:20], a[20:23]])
    out += [lib.dGeomBoxPointDepth(g, *p) for p in (a[0:3], a[17:20], a[20:23])]
    pos = V4()
    R = M12()
    lib.dGeomCopyPosition(g, pos)
    lib.dGeomCopyRotation(g, R)
    out += list(pos)[:3] + _m9(R)
    lib.dGeomSetOffsetQuaternion(g, _quat(lib, a[23:27]))
    out += _pose(lib, g)
    lib.dGeomSetOffsetWorldPosition(g, *a[27:30])
    out += _pose(lib, g) + _v3(lib.dGeomGetOffsetPosition(g))
    lib.dGeomSetOffsetWorldRotation(g, _rot(lib, a[30:34]))
    out += _pose(lib, g) + _m9(lib.dGeomGetOffsetRotation(g))
    lib.dGeomSetOffsetWorldQuaternion(g, _quat(lib, a[34:38]))
    out += _pose(lib, g) + _m9(lib.dGeomGetOffsetRotation(g))
    # the pose setters move the body so that body + offset lands on the pose
    lib.dGeomSetPosition(g, *a[38:41])
    out += _pose(lib, g) + _v3(lib.dBodyGetPosition(b)) + _m9(lib.dBodyGetRotation(b))
    lib.dGeomSetRotation(g, _rot(lib, a[41:45]))
    out += _pose(lib, g) + _v3(lib.dBodyGetPosition(b)) + _m9(lib.dBodyGetRotation(b))
    lib.dGeomSetQuaternion(g, _quat(lib, a[45:49]))
    out += _pose(lib, g) + _v3(lib.dBodyGetPosition(b)) + _m9(lib.dBodyGetRotation(b))
    # moving the body moves the offset geom
    lib.dBodySetPosition(b, *a[49:52])
    out += _pose(lib, g) + _aabb(lib, g)
    # detach keeps the final pose; a second geom keeps the body's
    g2 = lib.dCreateSphere(None, 0.3)
    lib.dGeomSetBody(g2, b)
    lib.dGeomSetBody(g, None)
    out += [lib.dGeomIsOffset(g), int(lib.dGeomGetBody(g) is None)] + _pose(lib, g)
    lib.dBodySetPosition(b, 0.0, 0.0, 0.0)
    out += _pose(lib, g)
    # clearing an offset returns the geom to its body's pose
    lib.dGeomSetBody(g, b)
    lib.dGeomSetOffsetPosition(g, 0.5, -0.25, 1.0)
    lib.dGeomClearOffset(g)
    out += [lib.dGeomIsOffset(g)] + _pose(lib, g) + _out4(lib, lib.dGeomGetOffsetQuaternion, g)
    out += _v3(lib.dGeomGetOffsetPosition(g)) + _m9(lib.dGeomGetOffsetRotation(g))
    # dBodyDestroy detaches the body's geoms in place
    lib.dBodySetPosition(b, *a[52:55])
    lib.dGeomSetOffsetPosition(g, *a[55:58])
    before = _pose(lib, g)
    lib.dBodyDestroy(b)
    out += before + [int(lib.dGeomGetBody(g) is None), int(lib.dGeomGetBody(g2) is None)]
    out += _pose(lib, g) + _pose(lib, g2)
    lib.dGeomDestroy(g)
    lib.dGeomDestroy(g2)
    lib.dWorldDestroy(w)
    return np.array(out, dtype=np.float32)


def _shape_sequence(lib, a):
    """Free geoms of every class: AABBs, point depths, setters, bits."""
    out = []
    pts = [a[0:3], a[3:6], [0.0, 0.0, 0.0]]
    geoms = [lib.dCreateSphere(None, abs(a[6]) + 0.1), lib.dCreateBox(None, abs(a[7]) + 0.1, abs(a[8]) + 0.1, 0.7),
             lib.dCreateCapsule(None, abs(a[9]) + 0.1, abs(a[10]) + 0.2),
             lib.dCreateCylinder(None, abs(a[11]) + 0.1, abs(a[12]) + 0.2), lib.dCreateRay(None, abs(a[13]) + 0.5)]
    for i, g in enumerate(geoms):
        lib.dGeomSetPosition(g, *a[14 + 3 * i:17 + 3 * i])
        lib.dGeomSetQuaternion(g, _quat(lib, a[29 + 4 * i:33 + 4 * i]))
        out += [lib.dGeomGetClass(g), lib.dGeomIsSpace(g), int(lib.dGeomGetSpace(g) is None)]
        out += _pose(lib, g) + _out4(lib, lib.dGeomGetQuaternion, g) + _aabb(lib, g) + _points(lib, g, pts[:2])
    sph, box, cap, cyl, ray = geoms
    out += [lib.dGeomSpherePointDepth(sph, *p) for p in pts]
    out += [lib.dGeomBoxPointDepth(box, *p) for p in pts]
    out += [lib.dGeomCapsulePointDepth(cap, *p) for p in pts]
    # setters
    lib.dGeomSphereSetRadius(sph, 0.75)
    lib.dGeomBoxSetLengths(box, 0.5, 1.5, 2.5)
    lib.dGeomCapsuleSetParams(cap, 0.25, 1.75)
    r, l = F(), F()
    lib.dGeomCapsuleGetParams(cap, C.byref(r), C.byref(l))
    out += [lib.dGeomSphereGetRadius(sph), r.value, l.value] + _out4(lib, lib.dGeomBoxGetLengths, box)[:3]
    out += _aabb(lib, sph) + _aabb(lib, box) + _aabb(lib, cap)
    out += [lib.dGeomSpherePointDepth(sph, *pts[0]), lib.dGeomBoxPointDepth(box, *pts[0]),
            lib.dGeomCapsulePointDepth(cap, *pts[0])]
    # planes: normalised parameters, half-space boxes along an axis
    pl = lib.dCreatePlane(None, a[44], a[45], a[46], a[47])
    out += _out4(lib, lib.dGeomPlaneGetParams, pl) + _aabb(lib, pl)
    out += [lib.dGeomPlanePointDepth(pl, *p) for p in pts] + _points(lib, pl, pts[:1])
    for prm in ((0.0, 0.0, -2.0, 0.5), (0.0, 3.0, 0.0, -1.0), (4.0, 0.0, 0.0, 2.0), (0.0, 0.0, 0.0, 1.0),
                (a[48], a[49], 0.0, a[50])):
        lib.dGeomPlaneSetParams(pl, *prm)
        out += _out4(lib, lib.dGeomPlaneGetParams, pl) + _aabb(lib, pl)
        out += [lib.dGeomPlanePointDepth(pl, *pts[0])]
    # bits and the enabled flag
    g = geoms[0]
    out += [float(lib.dGeomGetCategoryBits(g) == C.c_ulong(-1).value),
            float(lib.dGeomGetCollideBits(g) == C.c_ulong(-1).value), lib.dGeomIsEnabled(g)]
    lib.dGeomSetCategoryBits(g, 0x5)
    lib.dGeomSetCollideBits(g, 0xA0)
    lib.dGeomDisable(g)
    out += [lib.dGeomGetCategoryBits(g), lib.dGeomGetCollideBits(g), lib.dGeomIsEnabled(g)]
    lib.dGeomEnable(g)
    out += [lib.dGeomIsEnabled(g)]
    for g in geoms + [pl]:
        lib.dGeomDestroy(g)
    return np.array(out, dtype=np.float32)


def _heightfield_sequence(lib, a, heights, wrap):
    out = []
    d = lib.dGeomHeightfieldDataCreate()
    h = np.ascontiguousarray(heights, dtype=np.float32)
    nz, nx = h.shape
    lib.dGeomHeightfieldDataBuildSingle(d, h.ctypes.data, 0, 6.0, 4.0, nx, nz, 1.5, -0.25, 0.5, wrap)
    fixed = lib.dCreateHeightfield(None, d, 0)
    placed = lib.dCreateHeightfield(None, d, 1)
    lib.dGeomSetPosition(placed, *a[0:3])
    lib.dGeomSetRotation(placed, _rot(lib, a[3:7]))
    out += _aabb(lib, fixed) + _aabb(lib, placed) + _points(lib, fixed, [a[7:10]])
    # new bounds reach boxes computed afterwards
    lib.dGeomHeightfieldDataSetBounds(d, -2.0, 3.0)
    for bp in (0, 1):
        g = lib.dCreateHeightfield(None, d, bp)
        if bp:
            lib.dGeomSetPosition(g, *a[0:3])
            lib.dGeomSetRotation(g, _rot(lib, a[3:7]))
        out += _aabb(lib, g)
        lib.dGeomDestroy(g)
    lib.dGeomDestroy(fixed)
    lib.dGeomDestroy(placed)
    lib.dGeomHeightfieldDataDestroy(d)
    return np.array(out, dtype=np.float32)


def _close(x, y, rtol):
    """Equal where both are infinite; within rtol * (1 + |y|) elsewhere."""
    assert x.shape == y.shape
    inf = np.isinf(y)
    assert np.array_equal(np.isinf(x), inf) and np.array_equal(x[inf], y[inf]), (x[inf], y[inf])
    err = np.abs(x[~inf] - y[~inf]) / (1.0 + np.abs(y[~inf]))
    assert err.max(initial=0.0) <= rtol, (err.max(), int(np.argmax(err)))


def test_geom_offsets_match_reference_fp32():
    ours, ref = _libs()
    rng = np.random.default_rng(41)
    for _ in range(60):
        a = [float(x) for x in rng.normal(size=58)]
        x, y = _offset_sequence(ours, a), _offset_sequence(ref, a)
        # within FP32 rounding: dBodySetRotation keeps a body's orientation
        # through a quaternion formed in FP64 here and in FP32 in the
        # reference (a few ulps of R), which every later pose inherits
        _close(x, y, 2e-5)


def test_geom_shapes_bits_and_bounds_match_reference_fp32():
    ours, ref = _libs()
    rng = np.random.default_rng(43)
    for _ in range(60):
        a = [float(x) for x in rng.normal(size=51)]
        x, y = _shape_sequence(ours, a), _shape_sequence(ref, a)
        _close(x, y, 2e-6)


@pytest.mark.parametrize("wrap", [0, 1])
def test_heightfield_bounds_match_reference_fp32(wrap):
    ours, ref = _libs()
    rng = np.random.default_rng(47 + wrap)
    for _ in range(20):
        a = [float(x) for x in rng.normal(size=10)]
        heights = rng.normal(size=(5, 7)) * 2.0
        x, y = _heightfield_sequence(ours, a, heights, wrap), _heightfield_sequence(ref, a, heights, wrap)
        _close(x, y, 2e-6)


def test_heightfield_callback_bounds_and_data_handles_match_reference():
    """dGeomHeightfieldDataBuildCallback (heightfield.cpp:676-697): infinite
    vertical bounds until dGeomHeightfieldDataSetBounds, and ODE 0.12's
    dGeomHeightfieldSetHeightfieldData, which stores the handle as the geom's
    user data (:869-880); the callback is asked for every sample here."""
    ours, ref = _libs()
    HCB = C.CFUNCTYPE(F, P, I, I)
    calls = []

    def height(_, x, z):
        calls.append((x, z))
        return F(0.25 * x - 0.5 * z + 0.125 * x * z).value

    cb = HCB(height)
    outs = []
    for lib in (ours, ref):
        lib.dGeomHeightfieldDataBuildCallback.argtypes = [P, P, HCB, F, F, I, I, F, F, F, I]
        lib.dGeomHeightfieldSetHeightfieldData.argtypes = [P, P]
        lib.dGeomHeightfieldGetHeightfieldData.restype = P
        lib.dGeomHeightfieldGetHeightfieldData.argtypes = [P]
        lib.dGeomGetData.restype = P
        lib.dGeomGetData.argtypes = [P]
        out = []
        for wrap in (0, 1):
            d = lib.dGeomHeightfieldDataCreate()
            lib.dGeomHeightfieldDataBuildCallback(d, None, cb, 6.0, 4.0, 7, 5, 1.5, -0.25, 0.5, wrap)
            g = lib.dCreateHeightfield(None, d, 0)
            out += _aabb(lib, g)
            lib.dGeomHeightfieldDataSetBounds(d, -1.0, 2.0)
            g2 = lib.dCreateHeightfield(None, d, 0)
            out += _aabb(lib, g2)
            d2 = lib.dGeomHeightfieldDataCreate()
            lib.dGeomHeightfieldSetHeightfieldData(g2, d2)
            out += [float(lib.dGeomHeightfieldGetHeightfieldData(g2) == d), float(lib.dGeomGetData(g2) == d2)]
            for h in (g, g2):
                lib.dGeomDestroy(h)
            lib.dGeomHeightfieldDataDestroy(d)
            lib.dGeomHeightfieldDataDestroy(d2)
        outs.append(np.array(out, dtype=np.float32))
    assert np.array_equal(outs[0], outs[1]), outs
    assert (6, 4) in calls   # every sample was read here


def test_configuration_and_working_memory_calls():
    """dCheckConfiguration's whole-token match (ode.cpp:2241-2275) agrees with
    the reference on tokens both builds share, and the working-memory calls
    accept what the reference accepts (objects.h:157-289)."""
    ours, ref = _libs()
    tokens = [b"ODE", b"ODE_single_precision", b"ODE_single", b"single_precision", b"ODE_double_precision",
              b"", b"a b", b"ODE_EXT_trimesh", b"ODE_EXT_opcode"]
    for lib in (ours, ref):
        lib.dCheckConfiguration.argtypes = [C.c_char_p]
        lib.dGetConfiguration.restype = C.c_char_p
    for t in tokens:
        assert ours.dCheckConfiguration(t) == ref.dCheckConfiguration(t), t
    assert b"ODE_single_precision" in ours.dGetConfiguration()

    class Reserve(C.Structure):
        _fields_ = [("struct_size", C.c_uint), ("reserve_factor", F), ("reserve_minimum", C.c_uint)]

    for lib in (ours, ref):
        lib.dWorldSetStepMemoryReservationPolicy.argtypes = [P, P]
        lib.dWorldUseSharedWorkingMemory.argtypes = [P, P]
        lib.dWorldCleanupWorkingMemory.argtypes = [P]
        lib.dAllocateODEDataForThread.argtypes = [C.c_uint]
        lib.dWorldCreate.restype = P
        lib.dWorldDestroy.argtypes = [P]
    got = []
    for lib in (ours, ref):
        lib.dInitODE2(0)
        w = lib.dWorldCreate()
        good, bad = Reserve(C.sizeof(Reserve), 1.5, 4096), Reserve(C.sizeof(Reserve), 0.5, 4096)
        got.append([lib.dWorldSetStepMemoryReservationPolicy(w, C.byref(good)),
                    lib.dWorldSetStepMemoryReservationPolicy(w, None), lib.dAllocateODEDataForThread(0xffffffff)])
        lib.dWorldCleanupWorkingMemory(w)
        lib.dWorldDestroy(w)
    assert got[0] == got[1] == [1, 1, 1], got
    w = ours.dWorldCreate()
    assert ours.dWorldSetStepMemoryReservationPolicy(w, C.byref(bad)) == 0
    ours.dWorldDestroy(w)


def test_collider_override_matches_reference():
    """dSetColliderOverride (collision_kernel.cpp:275-336): the caller's
    collider runs in place of the built-in one, as given for (i, j) and with
    the geoms swapped and normals, geoms and sides flipped back for (j, i), so
    an override of a class with itself takes the swapped form; a null
    override leaves the pair without contacts. dCloseODE then dInitODE2 give
    the built-in colliders back."""
    ours, ref = _libs()

    class CG(C.Structure):
        _fields_ = [("pos", F * 4), ("normal", F * 4), ("depth", F), ("g1", P), ("g2", P), ("side1", I),
                    ("side2", I)]

    CB = C.CFUNCTYPE(I, P, P, I, P, I)

    def fake(o1, o2, flags, contact, skip):
        n = min(2, flags & 0xffff)
        for i in range(n):
            c = CG.from_address(contact + i * skip)
            c.pos[0], c.pos[1], c.pos[2] = 1.0 + i, 2.0, 3.0
            c.normal[0], c.normal[1], c.normal[2] = 0.6, 0.0, 0.8
            c.depth = 0.25 * (i + 1)
            c.g1, c.g2 = o1, o2
            c.side1, c.side2 = 7, 9 + i
        return n

    cb = CB(fake)
    outs = []
    for lib in (ours, ref):
        lib.dInitODE2.argtypes = [C.c_uint]
        lib.dInitODE2(0)
        lib.dSetColliderOverride.argtypes = [I, I, P]
        lib.dCollide.argtypes = [P, P, I, P, I]
        lib.dSetColliderOverride(dSphereClass, dBoxClass, C.cast(cb, P))
        lib.dSetColliderOverride(dSphereClass, dSphereClass, C.cast(cb, P))
        lib.dSetColliderOverride(dBoxClass, dBoxClass, None)
        s1, s2 = lib.dCreateSphere(None, 0.5), lib.dCreateSphere(None, 0.5)
        b1, b2 = lib.dCreateBox(None, 1.0, 1.0, 1.0), lib.dCreateBox(None, 1.0, 1.0, 1.0)
        ids = {s1: 0, s2: 1, b1: 2, b2: 3, None: -1}
        out = []
        for o1, o2, nmax in ((s1, b1, 4), (b1, s1, 4), (s1, s2, 1), (b1, b2, 4)):
            buf = (CG * 4)()
            n = lib.dCollide(o1, o2, nmax, buf, C.sizeof(CG))
            out += [n]
            for i in range(n):
                c = buf[i]
                out += list(c.pos)[:3] + list(c.normal)[:3] + [c.depth, ids[c.g1], ids[c.g2], c.side1, c.side2]
        for g in (s1, s2, b1, b2):
            lib.dGeomDestroy(g)
        lib.dCloseODE()
        lib.dInitODE2(0)
        outs.append(np.array(out, dtype=np.float32))
    assert np.array_equal(outs[0], outs[1]), (outs[0], outs[1])
    assert outs[0][0] == 2 and outs[0][-1] == 0


def test_user_geom_classes_match_reference():
    """dCreateGeomClass / dCreateGeom / dGeomGetClassData (collision_kernel.cpp:
    900-1012): the class's collider getter resolved on a pair's first
    dCollide, from the other user class when the first has none, the caller's
    box and box test used by a space's pair search, the destructor on
    dGeomDestroy, all as in the reference's dSINGLE build."""
    ours, ref = _libs()

    class CG(C.Structure):
        _fields_ = [("pos", F * 4), ("normal", F * 4), ("depth", F), ("g1", P), ("g2", P), ("side1", I),
                    ("side2", I)]

    FN = C.CFUNCTYPE(I, P, P, I, P, I)
    GET = C.CFUNCTYPE(P, I)
    AABB = C.CFUNCTYPE(None, P, C.POINTER(F))
    TEST = C.CFUNCTYPE(I, P, P, C.POINTER(F))
    DTOR = C.CFUNCTYPE(None, P)

    class GeomClass(C.Structure):
        _fields_ = [("bytes", I), ("collider", GET), ("aabb", AABB), ("aabb_test", TEST), ("dtor", DTOR)]

    outs = []
    for lib in (ours, ref):
        lib.dInitODE2.argtypes = [C.c_uint]
        lib.dInitODE2(0)
        for n in ("dCreateGeomClass",):
            getattr(lib, n).argtypes = [P]
        lib.dCreateGeom.restype = lib.dGeomGetClassData.restype = P
        lib.dCreateGeom.argtypes = [I]
        lib.dGeomGetClassData.argtypes = [P]
        lib.dCollide.argtypes = [P, P, I, P, I]
        lib.dSimpleSpaceCreate.restype = P
        lib.dSimpleSpaceCreate.argtypes = [P]
        lib.dSpaceAdd.argtypes = [P, P]
        NEAR = C.CFUNCTYPE(None, P, P, P)
        lib.dSpaceCollide.argtypes = [P, P, NEAR]
        lib.dSpaceDestroy.argtypes = [P]
        ids, log = {}, []

        def mk_fn(tag):
            def fn(o1, o2, flags, contact, skip):
                log.append((tag, ids[o1], ids[o2]))
                c = CG.from_address(contact)
                c.pos[0], c.pos[1], c.pos[2] = float(tag), 0.5, 0.25
                c.normal[0], c.normal[1], c.normal[2] = 0.0, 0.6, 0.8
                c.depth = 0.125
                c.g1, c.g2, c.side1, c.side2 = o1, o2, 3, 4
                return 1
            return fn

        fn_sphere, fn_self = FN(mk_fn(1)), FN(mk_fn(2))
        keep = [fn_sphere, fn_self]

        def getter(num):
            log.append(("get", num))
            if num == dSphereClass:
                return C.cast(fn_sphere, P).value
            if num >= 14:
                return C.cast(fn_self, P).value
            return None

        def aabb(g, out):
            p = lib.dGeomGetPosition(g)
            r = C.cast(lib.dGeomGetClassData(g), C.POINTER(F))[0]
            for k in range(3):
                out[2 * k], out[2 * k + 1] = p[k] - r, p[k] + r

        def test(g1, g2, box):
            return 0 if lib.dGeomGetClass(g2) == dBoxClass else 1

        def dtor(g):
            log.append(("dtor", ids[g]))

        gc = GeomClass(8, GET(getter), AABB(aabb), TEST(test), DTOR(dtor))
        keep += [gc]
        cls = lib.dCreateGeomClass(C.byref(gc))
        sp = lib.dSimpleSpaceCreate(None)
        u1, u2 = lib.dCreateGeom(cls), lib.dCreateGeom(cls)
        s = lib.dCreateSphere(sp, 0.5)
        b = lib.dCreateBox(sp, 1.0, 1.0, 1.0)
        for k, g in enumerate((u1, u2, s, b)):
            ids[g] = k
        for g, pos, r in ((u1, (0.0, 0.0, 0.0), 0.6), (u2, (0.8, 0.0, 0.0), 0.5)):
            C.cast(lib.dGeomGetClassData(g), C.POINTER(F))[0] = r
            lib.dGeomSetPosition(g, *pos)
            lib.dSpaceAdd(sp, g)
        lib.dGeomSetPosition(s, 0.3, 0.3, 0.0)
        lib.dGeomSetPosition(b, -0.4, 0.0, 0.2)
        out = [cls, lib.dGeomGetClass(u1)]
        for o1, o2 in ((u1, s), (s, u1), (u1, u2), (u2, u1), (u1, b), (b, u2)):
            buf = (CG * 2)()
            n = lib.dCollide(o1, o2, 2, buf, C.sizeof(CG))
            out += [n] + ([] if n == 0 else list(buf[0].pos)[:3] + list(buf[0].normal)[:3] +
                          [ids[buf[0].g1], ids[buf[0].g2], buf[0].side1, buf[0].side2])
        out += _aabb(lib, u1)
        pairs = []
        near = NEAR(lambda d, a, c: pairs.append((ids[a], ids[c])))
        lib.dSpaceCollide(sp, None, near)
        out += [x for pr in pairs for x in pr]
        lib.dGeomDestroy(u1)
        lib.dSpaceDestroy(sp)
        lib.dCloseODE()
        lib.dInitODE2(0)
        outs.append((np.array(out, dtype=np.float32), log))
    assert np.array_equal(outs[0][0], outs[1][0]), (outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1], (outs[0][1], outs[1][1])


def test_geom_transform_matches_reference():
    """dCreateGeomTransform and its calls (collision_transform.cpp:38-209): the
    wrapped geom's box at the carried pose, collisions with the wrapped geom
    at that pose and with the transform's body (both argument orders, info
    mode naming the transform), space pairs, cleanup on destroy. The wrapped
    geom is of a user class, so its collider is the test's own host code and
    records the pose it sees; against the reference's dSINGLE build."""
    ours, ref = _libs()

    class CG(C.Structure):
        _fields_ = [("pos", F * 4), ("normal", F * 4), ("depth", F), ("g1", P), ("g2", P), ("side1", I),
                    ("side2", I)]

    FN = C.CFUNCTYPE(I, P, P, I, P, I)
    GET = C.CFUNCTYPE(P, I)
    AABB = C.CFUNCTYPE(None, P, C.POINTER(F))
    DTOR = C.CFUNCTYPE(None, P)

    class GeomClass(C.Structure):
        _fields_ = [("bytes", I), ("collider", GET), ("aabb", AABB), ("aabb_test", P), ("dtor", DTOR)]

    outs = []
    for lib in (ours, ref):
        lib.dInitODE2.argtypes = [C.c_uint]
        lib.dInitODE2(0)
        lib.dCreateGeomClass.argtypes = [P]
        lib.dCreateGeom.restype = lib.dGeomGetClassData.restype = lib.dCreateGeomTransform.restype = P
        lib.dGeomTransformGetGeom.restype = P
        lib.dCreateGeom.argtypes = [I]
        lib.dGeomGetClassData.argtypes = lib.dGeomTransformGetGeom.argtypes = [P]
        lib.dCreateGeomTransform.argtypes = [P]
        lib.dGeomTransformSetGeom.argtypes = [P, P]
        for n in ("dGeomTransformSetCleanup", "dGeomTransformSetInfo"):
            getattr(lib, n).argtypes = [P, I]
        lib.dGeomTransformGetCleanup.argtypes = lib.dGeomTransformGetInfo.argtypes = [P]
        lib.dCollide.argtypes = [P, P, I, P, I]
        lib.dSimpleSpaceCreate.restype = P
        lib.dSimpleSpaceCreate.argtypes = [P]
        NEAR = C.CFUNCTYPE(None, P, P, P)
        lib.dSpaceCollide.argtypes = [P, P, NEAR]
        lib.dSpaceDestroy.argtypes = [P]
        ids, log = {}, []

        def coll(o1, o2, flags, contact, skip):
            p = lib.dGeomGetPosition(o1)
            R = lib.dGeomGetRotation(o1)
            log.append(("coll", ids.get(o1, -1), ids.get(o2, -1), p[0], p[1], p[2], R[0], R[1], R[5]))
            c = CG.from_address(contact)
            c.pos[0], c.pos[1], c.pos[2] = p[0], p[1], p[2]
            c.normal[2] = 1.0
            c.depth = 0.1
            c.g1, c.g2 = o1, o2
            return 1

        fn = FN(coll)

        def getter(num):
            return C.cast(fn, P).value if num == dSphereClass else None

        def aabb(g, out):
            p = lib.dGeomGetPosition(g)
            for k in range(3):
                out[2 * k], out[2 * k + 1] = p[k] - 0.4, p[k] + 0.4

        def dtor(g):
            log.append(("dtor", ids.get(g, -1)))

        gc = GeomClass(4, GET(getter), AABB(aabb), None, DTOR(dtor))
        cls = lib.dCreateGeomClass(C.byref(gc))
        w = lib.dWorldCreate()
        body = lib.dBodyCreate(w)
        lib.dBodySetPosition(body, 0.5, -0.25, 1.0)
        lib.dBodySetRotation(body, _rot(lib, [0.2, 0.9, -0.3, 0.7]))
        sp = lib.dSimpleSpaceCreate(None)
        tr = lib.dCreateGeomTransform(sp)
        u = lib.dCreateGeom(cls)
        s = lib.dCreateSphere(sp, 0.5)
        s2 = lib.dCreateSphere(None, 0.3)
        for k, g in enumerate((tr, u, s, s2)):
            ids[g] = k
        out = [lib.dGeomTransformGetCleanup(tr), lib.dGeomTransformGetInfo(tr),
               int(lib.dGeomTransformGetGeom(tr) is None)] + _aabb(lib, tr)
        lib.dGeomTransformSetGeom(tr, u)
        lib.dGeomTransformSetCleanup(tr, 1)
        lib.dGeomSetPosition(u, 0.25, 0.0, -0.5)
        lib.dGeomSetRotation(u, _rot(lib, [1.0, 0.0, 0.5, 0.3]))
        lib.dGeomSetPosition(tr, 1.0, 2.0, 3.0)
        lib.dGeomSetRotation(tr, _rot(lib, [0.0, 1.0, 1.0, 0.8]))
        lib.dGeomSetPosition(s, 1.2, 2.1, 2.6)
        out += _aabb(lib, tr) + _pose(lib, tr)
        for info in (0, 1):
            lib.dGeomTransformSetInfo(tr, info)
            for o1, o2 in ((tr, s), (s, tr)):
                buf = (CG * 2)()
                n = lib.dCollide(o1, o2, 2, buf, C.sizeof(CG))
                out += [n] + list(buf[0].pos)[:3] + list(buf[0].normal)[:3] + [ids[buf[0].g1], ids[buf[0].g2]]
        pairs = []
        near = NEAR(lambda d, a, b: pairs.append((ids[a], ids[b])))
        lib.dSpaceCollide(sp, None, near)
        out += [x for pr in pairs for x in pr]
        # on a body: the wrapped geom takes the body for the same-body rule
        lib.dGeomSetBody(tr, body)
        lib.dGeomSetBody(s2, body)
        buf = (CG * 2)()
        out += [lib.dCollide(tr, s2, 2, buf, C.sizeof(CG))] + _aabb(lib, tr)
        lib.dGeomSetBody(s2, None)
        lib.dGeomSetPosition(s2, 1.0, -0.2, 0.9)
        out += [lib.dCollide(tr, s2, 2, buf, C.sizeof(CG))] + list(buf[0].pos)[:3]
        lib.dGeomDestroy(tr)            # cleanup on: the user geom goes too
        lib.dSpaceDestroy(sp)
        lib.dGeomDestroy(s2)
        lib.dWorldDestroy(w)
        lib.dCloseODE()
        lib.dInitODE2(0)
        outs.append((np.array(out, dtype=np.float64), log))
    _close(outs[0][0].astype(np.float32), outs[1][0].astype(np.float32), 2e-6)
    la, lb = outs[0][1], outs[1][1]
    assert [x[:3] for x in la] == [x[:3] for x in lb], (la, lb)
    _close(np.array([x[3:] for x in la if x[0] == "coll"], dtype=np.float32),
           np.array([x[3:] for x in lb if x[0] == "coll"], dtype=np.float32), 2e-6)
