"""C ABI checks that need no GPU: libodegpu loads and exports every function
declared in include/*.h, the ODE-API demo compiles and links against it, and
the library refuses to run without a CUDA device (no CPU fallback)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"typedef\s+\w+\s*\**\s*d\w+\s*\([^;]*;", "", txt)   # function types (dNearCallback)
    names = re.findall(r"\b(d[A-Z]\w+|odegpu[A-Z]\w+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", os.path.dirname(LIB), "libodegpu.so"], check=True)
    return C.CDLL(LIB)


@pytest.mark.parametrize("header", ["odegpu.h", "ode_gpu.h"])
def test_exports_every_declared_symbol(lib, header):
    names = declared(header)
    assert len(names) > 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_demo_links_against_libodegpu():
    import c_api_util as U
    with tempfile.TemporaryDirectory() as d:
        U.build_gpu_demo(os.path.join(d, "demo"))
        U.build_gpu_demo(os.path.join(d, "player"), src=U.PLAYER)


def test_scene_player_is_the_reference_harness_sequence():
    """tests/c_api/scene_player.c, built against the reference ODE 0.12
    (dSINGLE) where it was built in this checkout, reproduces the reference
    harness bit for bit on the joint-type scene and the cylinder pile: the program the GPU test
    links against libodegpu is a faithful ODE program."""
    import c_api_util as U
    import numpy as np
    import oracle_lib as O
    from odegpu import scene as S
    if not (U.ref_demo_available() and O.ref_available("s")):
        pytest.skip("reference not built in this checkout")
    with tempfile.TemporaryDirectory() as d:
        exe = U.build_ref_demo(os.path.join(d, "player"), src=U.PLAYER)
        for sc in (S.mechanisms(n_worlds=2, steps=60), S.cylinder_pile(n_worlds=1)):
            for w in range(sc.n_worlds):
                inp = os.path.join(d, f"in{w}.txt")
                U.player_input(sc, w, 60, inp)
                st = U.run_demo(exe, inp).astype(np.float32).astype(np.float64)
                ref = O.run_world(O.ref("s").ref_run_world, sc, w, 60)["state"][-1]
                assert np.array_equal(st, ref), float(np.abs(st - ref).max())
        # and with dWorldStep
        sc = S.mechanisms(n_worlds=2, steps=60)
        with O.exact_stepper(O.ref("s")):
            for w in range(sc.n_worlds):
                inp = os.path.join(d, f"in{w}.txt")
                U.player_input(sc, w, 40, inp)
                st = U.run_demo(exe, inp, "exact").astype(np.float32).astype(np.float64)
                ref = O.run_world(O.ref("s").ref_run_world, sc, w, 40)["state"][-1]
                assert np.array_equal(st, ref), float(np.abs(st - ref).max())


def test_no_device_fails_loudly():
    """Without a CUDA device, creating a batch returns ODEGPU_E_CUDA with a
    message; nothing silently runs on the CPU."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from odegpu import scene as S
    from odegpu._lib import OdeGpuError
    from odegpu.batch import Batch
    with pytest.raises(OdeGpuError, match="CUDA"):
        Batch(S.box_drop(seed=0))


def test_rotation_utilities_match_reference_fp32():
    """dRFromAxisAndAngle, dRFromEulerAngles, dRFrom2Axes, dRFromZAxis,
    dQFromAxisAndAngle, dQMultiply0-3, dRfromQ, dQfromR, dDQfromW,
    dSafeNormalize3/4 and dPlaneSpace of the library (host code, no GPU)
    against the reference's dSINGLE build on seeded inputs: bit-identical
    (the reference's transcendentals are the same libm calls)."""
    import ctypes as C
    import numpy as np
    import c_api_util as U
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    F = C.c_float
    V4 = F * 4
    M12 = F * 12
    rng = np.random.default_rng(4)
    for lib in (ours, ref):
        for name in ("dRFromAxisAndAngle", "dQFromAxisAndAngle"):
            getattr(lib, name).argtypes = [C.c_void_p, F, F, F, F]
        lib.dRFromEulerAngles.argtypes = [C.c_void_p, F, F, F]
        lib.dRFrom2Axes.argtypes = [C.c_void_p, F, F, F, F, F, F]
        lib.dRFromZAxis.argtypes = [C.c_void_p, F, F, F]
    for _ in range(200):
        a = [float(x) for x in rng.normal(size=7)]
        outs = []
        for lib in (ours, ref):
            R1, R2, R3, R4 = M12(), M12(), M12(), M12()
            q1, q2 = V4(), V4()
            lib.dRFromAxisAndAngle(R1, *a[:4])
            lib.dRFromEulerAngles(R2, *a[:3])
            lib.dRFrom2Axes(R3, *a[:6])
            lib.dRFromZAxis(R4, *a[:3])
            lib.dQFromAxisAndAngle(q1, *a[3:7])
            lib.dQfromR(q2, R1)
            qm = []
            for k in range(4):
                r = V4()
                getattr(lib, f"dQMultiply{k}")(r, q1, q2)
                qm += list(r)
            R5, dq = M12(), V4()
            lib.dRfromQ(R5, q1)
            w = V4(*a[:3], 0.0)
            lib.dDQfromW(dq, w, q1)
            n3, n4 = V4(*a[:3], 0.0), V4(*a[:4])
            r3 = lib.dSafeNormalize3(n3)
            r4 = lib.dSafeNormalize4(n4)
            p, q = V4(), V4()
            lib.dPlaneSpace(n3, p, q)
            outs.append(np.array(list(R1) + list(R2) + list(R3) + list(R4) + list(q1) + list(q2) + qm + list(R5) +
                                 list(dq) + list(n3)[:3] + list(n4) + [r3, r4] + list(p)[:3] + list(q)[:3],
                                 dtype=np.float32))
        assert np.array_equal(outs[0], outs[1]), np.abs(outs[0] - outs[1]).max()


def test_mass_algebra_and_body_helpers_match_reference_fp32():
    """dMassTranslate / dMassRotate / dMassAdd (ode/src/mass.cpp:454-541) and
    the body helpers dBodyAddRel*/At*Pos, dBodyGetRelPointPos / PosRelPoint /
    RelPointVel / PointVel, dBodyVectorTo/FromWorld, dBodyGetNumJoints /
    GetJoint and dAreConnected (ode/src/ode.cpp:537-830, 1518-1526) of the
    library (host code, no GPU) against the reference's dSINGLE build on
    seeded inputs."""
    import ctypes as C
    import numpy as np
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    F, P = C.c_float, C.c_void_p
    V4 = F * 4
    M12 = F * 12

    class Mass(C.Structure):
        _fields_ = [("mass", F), ("c", F * 4), ("I", F * 12)]

    for lib in (ours, ref):
        lib.dRFromAxisAndAngle.argtypes = [P, F, F, F, F]
        lib.dMassSetBox.argtypes = [P, F, F, F, F]
        lib.dMassSetSphereTotal.argtypes = [P, F, F]
        lib.dMassTranslate.argtypes = [P, F, F, F]
        lib.dMassRotate.argtypes = [P, P]
        lib.dMassAdd.argtypes = [P, P]
        lib.dWorldCreate.restype = P
        lib.dBodyCreate.restype = P
        lib.dBodyCreate.argtypes = [P]
        lib.dBodySetPosition.argtypes = [P, F, F, F]
        lib.dBodySetRotation.argtypes = [P, P]
        lib.dBodySetLinearVel.argtypes = [P, F, F, F]
        lib.dBodySetAngularVel.argtypes = [P, F, F, F]
        for name in ("dBodyAddRelForce", "dBodyAddRelTorque", "dBodySetForce", "dBodySetTorque"):
            getattr(lib, name).argtypes = [P, F, F, F]
        for name in ("dBodyAddForceAtPos", "dBodyAddForceAtRelPos", "dBodyAddRelForceAtPos",
                     "dBodyAddRelForceAtRelPos"):
            getattr(lib, name).argtypes = [P] + [F] * 6
        for name in ("dBodyGetRelPointPos", "dBodyGetPosRelPoint", "dBodyGetRelPointVel", "dBodyGetPointVel",
                     "dBodyVectorToWorld", "dBodyVectorFromWorld"):
            getattr(lib, name).argtypes = [P, F, F, F, P]
        lib.dBodyGetForce.restype = C.POINTER(F)
        lib.dBodyGetTorque.restype = C.POINTER(F)
        lib.dBodyGetForce.argtypes = lib.dBodyGetTorque.argtypes = [P]
        lib.dJointCreateBall.restype = lib.dJointCreateHinge.restype = P
        lib.dJointCreateBall.argtypes = lib.dJointCreateHinge.argtypes = [P, P]
        lib.dJointAttach.argtypes = [P, P, P]
        lib.dBodyGetJoint.restype = P
        lib.dBodyGetJoint.argtypes = [P, C.c_int]
        lib.dBodyGetNumJoints.argtypes = [P]
        lib.dAreConnected.argtypes = [P, P]
        lib.dWorldDestroy.argtypes = [P]
    rng = np.random.default_rng(9)
    for _ in range(100):
        a = [float(x) for x in rng.normal(size=24)]
        outs = []
        for lib in (ours, ref):
            R = M12()
            lib.dRFromAxisAndAngle(R, *a[:4])
            m1, m2 = Mass(), Mass()
            lib.dMassSetBox(C.byref(m1), 500.0, abs(a[4]) + 0.1, abs(a[5]) + 0.1, abs(a[6]) + 0.1)
            lib.dMassTranslate(C.byref(m1), *a[7:10])
            lib.dMassRotate(C.byref(m1), R)
            lib.dMassSetSphereTotal(C.byref(m2), abs(a[10]) + 0.5, abs(a[11]) + 0.05)
            lib.dMassTranslate(C.byref(m2), *a[12:15])
            lib.dMassAdd(C.byref(m1), C.byref(m2))
            out = [m1.mass] + list(m1.c)[:3] + list(m1.I)
            w = lib.dWorldCreate()
            b = lib.dBodyCreate(w)
            lib.dBodySetPosition(b, *a[15:18])
            lib.dBodySetRotation(b, R)
            lib.dBodySetLinearVel(b, *a[18:21])
            lib.dBodySetAngularVel(b, *a[21:24])
            lib.dBodySetForce(b, 1.0, -2.0, 0.5)
            lib.dBodySetTorque(b, 0.0, 0.25, -1.0)
            lib.dBodyAddRelForce(b, *a[:3])
            lib.dBodyAddRelTorque(b, *a[3:6])
            lib.dBodyAddForceAtPos(b, *a[6:12])
            lib.dBodyAddForceAtRelPos(b, *a[9:15])
            lib.dBodyAddRelForceAtPos(b, *a[12:18])
            lib.dBodyAddRelForceAtRelPos(b, *a[15:21])
            fp, tp = lib.dBodyGetForce(b), lib.dBodyGetTorque(b)
            out += [fp[k] for k in range(3)] + [tp[k] for k in range(3)]
            for name in ("dBodyGetRelPointPos", "dBodyGetPosRelPoint", "dBodyGetRelPointVel", "dBodyGetPointVel",
                         "dBodyVectorToWorld", "dBodyVectorFromWorld"):
                r = V4()
                getattr(lib, name)(b, *a[18:21], r)
                out += list(r)[:3]
            b2, b3 = lib.dBodyCreate(w), lib.dBodyCreate(w)
            j1, j2, j3 = lib.dJointCreateBall(w, None), lib.dJointCreateHinge(w, None), lib.dJointCreateBall(w, None)
            lib.dJointAttach(j1, b, b2)
            lib.dJointAttach(j2, b2, b)
            lib.dJointAttach(j3, b3, None)
            js = [j1, j2, j3]
            order = [js.index(lib.dBodyGetJoint(b, k)) for k in range(lib.dBodyGetNumJoints(b))]
            out += [float(x) for x in order] + [float(lib.dBodyGetNumJoints(b3)),
                                                float(lib.dAreConnected(b, b2)), float(lib.dAreConnected(b2, b3)),
                                                float(lib.dAreConnected(b3, None)), float(lib.dAreConnected(b, None))]
            lib.dWorldDestroy(w)
            outs.append(np.array(out, dtype=np.float32))
        # the mass algebra and the integer answers bit-identical; the body
        # helpers within FP32 rounding, since dBodySetRotation keeps its
        # orientation through a quaternion formed in FP64 here and in FP32
        # in the reference (a few ulps of R)
        assert np.array_equal(outs[0][:16], outs[1][:16]), np.abs(outs[0][:16] - outs[1][:16]).max()
        assert np.array_equal(outs[0][40:], outs[1][40:]), (outs[0][40:], outs[1][40:])
        scale = 1.0 + np.abs(outs[1][16:40])
        assert (np.abs(outs[0][16:40] - outs[1][16:40]) <= 4e-6 * scale).all(), \
            np.abs(outs[0][16:40] - outs[1][16:40]).max()


def test_connecting_joints_and_small_accessors_match_reference_fp32():
    """dConnectingJoint[List], dJointGetNumBodies, dWorldImpulseToForce,
    dRandReal, dJointGetBallAnchor2 and dJointGetBall/Hinge/Hinge2Param
    (ode/src/ode.cpp:1399-1515, 1783-1791; misc.cpp:57-60; joints/ball.cpp,
    hinge.cpp, hinge2.cpp) against the reference's dSINGLE build."""
    import ctypes as C
    import numpy as np
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    F, P = C.c_float, C.c_void_p
    outs = []
    for lib in (ours, ref):
        lib.dWorldCreate.restype = lib.dBodyCreate.restype = P
        lib.dBodyCreate.argtypes = [P]
        lib.dBodySetPosition.argtypes = [P, F, F, F]
        for n in ("dJointCreateBall", "dJointCreateHinge", "dJointCreateHinge2"):
            getattr(lib, n).restype = P
            getattr(lib, n).argtypes = [P, P]
        lib.dJointAttach.argtypes = [P, P, P]
        lib.dJointSetBallAnchor.argtypes = [P, F, F, F]
        lib.dJointGetBallAnchor2.argtypes = [P, P]
        lib.dConnectingJoint.restype = P
        lib.dConnectingJoint.argtypes = [P, P]
        lib.dConnectingJointList.argtypes = [P, P, P]
        lib.dJointGetNumBodies.argtypes = [P]
        lib.dWorldImpulseToForce.argtypes = [P, F, F, F, F, P]
        lib.dRandReal.restype = F
        lib.dRandSetSeed.argtypes = [C.c_ulong]
        for n in ("dJointSetBallParam", "dJointSetHingeParam", "dJointSetHinge2Param"):
            getattr(lib, n).argtypes = [P, C.c_int, F]
        for n in ("dJointGetBallParam", "dJointGetHingeParam", "dJointGetHinge2Param"):
            getattr(lib, n).restype = F
            getattr(lib, n).argtypes = [P, C.c_int]
        w = lib.dWorldCreate()
        b1, b2, b3 = lib.dBodyCreate(w), lib.dBodyCreate(w), lib.dBodyCreate(w)
        lib.dBodySetPosition(b1, 0.1, 0.2, 0.3)
        lib.dBodySetPosition(b2, 1.1, -0.4, 0.7)
        lib.dBodySetPosition(b3, 0.0, 2.0, 0.0)
        jb, jh, jh2, jd = (lib.dJointCreateBall(w, None), lib.dJointCreateHinge(w, None),
                           lib.dJointCreateHinge2(w, None), lib.dJointCreateBall(w, None))
        js = [jb, jh, jh2, jd, None]
        lib.dJointAttach(jb, b2, b1)
        lib.dJointSetBallAnchor(jb, 0.5, 0.0, 0.5)
        lib.dBodySetPosition(b2, 1.3, -0.4, 0.9)
        lib.dJointAttach(jh, b1, b2)
        lib.dJointAttach(jh2, b3, b2)
        lib.dJointAttach(jd, b3, None)
        out = []
        a2 = (F * 4)()
        lib.dJointGetBallAnchor2(jb, a2)
        out += list(a2)[:3]
        lst = (P * 8)()
        n = lib.dConnectingJointList(b1, b2, lst)
        out += [n] + [js.index(lst[k]) for k in range(n)]
        out += [js.index(lib.dConnectingJoint(b1, b2)), js.index(lib.dConnectingJoint(None, b3)),
                js.index(lib.dConnectingJoint(b2, b3)), js.index(lib.dConnectingJoint(b1, b3))]
        out += [lib.dJointGetNumBodies(j) for j in (jb, jh2, jd)]
        f = (F * 4)()
        lib.dWorldImpulseToForce(w, 0.01, 1.5, -2.0, 0.3, f)
        out += list(f)[:3]
        lib.dRandSetSeed(12345)
        out += [lib.dRandReal() for _ in range(4)]
        lib.dJointSetBallParam(jb, 3, 0.5)      # dParamVel: not a ball parameter
        lib.dJointSetBallParam(jb, 6, 1e-4)     # dParamCFM
        lib.dJointSetHingeParam(jh, 0, -0.7)    # dParamLoStop
        lib.dJointSetHingeParam(jh, 2, 1.25)    # dParamVel
        lib.dJointSetHinge2Param(jh2, 0x102, 3.0)   # dParamVel2
        lib.dJointSetHinge2Param(jh2, 9, 0.4)       # dParamSuspensionERP
        out += [lib.dJointGetBallParam(jb, p) for p in (3, 6, 11)]
        out += [lib.dJointGetHingeParam(jh, p) for p in (0, 1, 2, 3, 4, 5, 6, 7, 8)]
        out += [lib.dJointGetHinge2Param(jh2, p) for p in (0, 2, 9, 10, 0x100, 0x102, 0x103)]
        lib.dWorldDestroy(w)
        outs.append(np.array(out, dtype=np.float32))
    assert np.array_equal(outs[0], outs[1]), (outs[0], outs[1])


def test_mass_check_matches_reference():
    """dMassCheck (ode/src/mass.cpp:44-83, dIsPositiveDefinite of
    matrix.cpp:124-160) against the reference's dSINGLE build on valid masses,
    masses moved far off their centre, and random (mostly indefinite) ones."""
    import ctypes as C
    import numpy as np
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    F = C.c_float

    class Mass(C.Structure):
        _fields_ = [("mass", F), ("c", F * 4), ("I", F * 12)]

    for lib in (ours, ref):
        lib.dMassCheck.argtypes = [C.c_void_p]
    rng = np.random.default_rng(17)
    got, want = [], []
    for k in range(600):
        m = Mass()
        m.mass = float(rng.uniform(-0.5, 3.0))
        if k % 3 == 0:    # a box's inertia, possibly with its centre moved away
            d = rng.uniform(0.1, 2.0, 3)
            I = m.mass / 12 * np.diag([d[1] ** 2 + d[2] ** 2, d[0] ** 2 + d[2] ** 2, d[0] ** 2 + d[1] ** 2])
            c = rng.normal(size=3) * (0.05 if k % 2 else 2.0)
        else:
            a = rng.normal(size=(3, 3))
            I = a @ a.T if k % 3 == 1 else (a + a.T) / 2
            c = rng.normal(size=3) * 0.3
        for i in range(3):
            m.c[i] = float(c[i])
            for j in range(3):
                m.I[i * 4 + j] = float(I[i, j])
        got.append(ours.dMassCheck(C.byref(m)))
        want.append(ref.dMassCheck(C.byref(m)))
    assert got == want
    assert 100 < sum(want) < 500
    # NaN in the mass, the centre or the inertia
    for field in ("mass", "c", "I"):
        m = Mass()
        m.mass = 1.0
        for i in range(3):
            m.I[i * 4 + i] = 0.1
        if field == "mass":
            m.mass = float("nan")
        elif field == "c":
            m.c[1] = float("nan")
        else:
            m.I[0] = float("nan")
        assert ours.dMassCheck(C.byref(m)) == ref.dMassCheck(C.byref(m)), field


def test_matrix_helpers_kinematic_bodies_and_orthogonalize_match_reference():
    """dMakeRandomVector / Matrix, dClearUpperTriangle, dMaxDifference[LowerTriangle]
    (ode/src/misc.cpp:139-195), dOrthogonalizeR (odemath.cpp:187-211),
    dInfiniteAABB and dBodySetKinematic / SetDynamic / IsKinematic
    (ode.cpp:834-852) against the reference's dSINGLE build, bit for bit."""
    import ctypes as C
    import numpy as np
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    F, P = C.c_float, C.c_void_p
    outs = []
    for path in (os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"),
                 os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")):
        lib = C.CDLL(path)
        lib.dRandSetSeed.argtypes = [C.c_ulong]
        lib.dMakeRandomVector.argtypes = [P, C.c_int, F]
        lib.dMakeRandomMatrix.argtypes = [P, C.c_int, C.c_int, F]
        lib.dClearUpperTriangle.argtypes = [P, C.c_int]
        lib.dMaxDifference.restype = lib.dMaxDifferenceLowerTriangle.restype = F
        lib.dMaxDifference.argtypes = [P, P, C.c_int, C.c_int]
        lib.dMaxDifferenceLowerTriangle.argtypes = [P, P, C.c_int]
        lib.dOrthogonalizeR.argtypes = [P]
        lib.dInfiniteAABB.argtypes = [P, P]
        lib.dWorldCreate.restype = lib.dBodyCreate.restype = P
        lib.dBodyCreate.argtypes = [P]
        for n in ("dBodySetKinematic", "dBodySetDynamic", "dBodyIsKinematic", "dBodySetMass", "dBodyGetMass"):
            getattr(lib, n).argtypes = [P] if n not in ("dBodySetMass", "dBodyGetMass") else [P, P]
        lib.dMassSetBox.argtypes = [P, F, F, F, F]
        lib.dWorldDestroy.argtypes = [P]
        lib.dRandSetSeed(77)
        out = []
        v = (F * 7)()
        lib.dMakeRandomVector(v, 7, 2.5)
        out += list(v)
        a, b = (F * 24)(), (F * 24)()   # 3 x 5, rows padded to 8
        lib.dMakeRandomMatrix(a, 3, 5, 1.5)
        lib.dMakeRandomMatrix(b, 3, 5, 1.5)
        out += [lib.dMaxDifference(a, b, 3, 5)]
        sq, sq2 = (F * 40)(), (F * 40)()   # 5 x 5, rows padded to 8
        lib.dMakeRandomMatrix(sq, 5, 5, 1.0)
        lib.dMakeRandomMatrix(sq2, 5, 5, 1.0)
        out += [lib.dMaxDifferenceLowerTriangle(sq, sq2, 5)]
        lib.dClearUpperTriangle(sq, 5)
        out += list(sq)
        rng = np.random.default_rng(5)
        for _ in range(20):
            m = (F * 12)(*rng.normal(size=12).astype(np.float32))
            lib.dOrthogonalizeR(m)
            out += list(m)
        box = (F * 6)()
        lib.dInfiniteAABB(None, box)
        out += list(box)
        w = lib.dWorldCreate()
        bd = lib.dBodyCreate(w)

        class Mass(C.Structure):
            _fields_ = [("mass", F), ("c", F * 4), ("I", F * 12)]

        m = Mass()
        lib.dMassSetBox(C.byref(m), 2.0, 0.3, 0.4, 0.5)
        lib.dBodySetMass(bd, C.byref(m))
        out += [lib.dBodyIsKinematic(bd)]
        lib.dBodySetKinematic(bd)
        out += [lib.dBodyIsKinematic(bd)]
        lib.dBodySetDynamic(bd)
        out += [lib.dBodyIsKinematic(bd)]
        lib.dWorldDestroy(w)
        outs.append(np.array(out, dtype=np.float32))
    assert np.array_equal(outs[0], outs[1]), \
        np.flatnonzero(outs[0] != outs[1])


def test_closest_segment_points_and_box_touches_box_match_reference():
    """dClosestLineSegmentPoints (ode/src/collision_util.cpp:109-209, the
    colliders' own host-and-device routine) and dBoxTouchesBox (:388-449) on
    seeded segments and box pairs near contact, against the reference's
    dSINGLE build: points bit for bit, the boolean exactly."""
    import ctypes as C
    import numpy as np
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    F, P = C.c_float, C.c_void_p
    V4, M12 = F * 4, F * 12
    libs = [C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")),
            C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))]
    for lib in libs:
        lib.dClosestLineSegmentPoints.argtypes = [P] * 6
        lib.dBoxTouchesBox.argtypes = [P] * 6
        lib.dRFromAxisAndAngle.argtypes = [P, F, F, F, F]
    rng = np.random.default_rng(13)
    touches = 0
    for k in range(3000):
        pts = rng.normal(size=(4, 3)).astype(np.float32)
        if k % 10 == 0:
            pts[1] = pts[0]                 # a degenerate segment
        if k % 10 == 1:
            pts[3] = pts[2] + (pts[1] - pts[0])   # parallel segments
        ax = [float(x) for x in rng.normal(size=8)]
        s1, s2 = rng.uniform(0.2, 1.5, 3), rng.uniform(0.2, 1.5, 3)
        p2 = rng.normal(size=3) * 1.2
        res = []
        for lib in libs:
            v = [V4(*pts[i], 0.0) for i in range(4)]
            c1, c2 = V4(), V4()
            lib.dClosestLineSegmentPoints(v[0], v[1], v[2], v[3], c1, c2)
            R1, R2 = M12(), M12()
            lib.dRFromAxisAndAngle(R1, *ax[:4])
            lib.dRFromAxisAndAngle(R2, *ax[4:])
            t = lib.dBoxTouchesBox(V4(0.1, -0.2, 0.3, 0), R1, V4(*s1, 0), V4(*p2, 0), R2, V4(*s2, 0))
            res.append((list(c1)[:3] + list(c2)[:3], t))
        assert res[0][0] == res[1][0], (k, res)
        assert res[0][1] == res[1][1], (k, res)
        touches += res[0][1]
    assert 300 < touches < 2700, touches


def test_print_matrix_writes_what_the_reference_writes(tmp_path):
    """dPrintMatrix (ode/src/misc.cpp:128-136): padded rows, the caller's
    format, one line per row, byte for byte as the reference's."""
    import ctypes as C
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    libc = C.CDLL(None)
    libc.fopen.restype = C.c_void_p
    libc.fopen.argtypes = [C.c_char_p, C.c_char_p]
    libc.fclose.argtypes = [C.c_void_p]
    A = (C.c_float * 16)(*[0.5 * k - 2.25 for k in range(16)])   # 2 rows padded to 8
    texts = []
    for name, path in (("ours", os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")),
                       ("ref", os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))):
        lib = C.CDLL(path)
        lib.dPrintMatrix.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_void_p]
        out = str(tmp_path / f"{name}.txt")
        f = libc.fopen(out.encode(), b"w")
        lib.dPrintMatrix(A, 3, 3, b"%10.4f ", f)
        lib.dPrintMatrix(A, 2, 5, b"%g,", f)
        libc.fclose(f)
        texts.append(open(out).read())
    assert texts[0] == texts[1] and texts[0].count("\n") == 5, texts


def test_space_demo_builds_both_ways_and_pairs_agree():
    """tests/c_api/space_stack_demo.c, an ODE program in the shape of ODE's
    demos (hash space, near-callback with dCollide and contact joints,
    auto-disable, damping), compiles unchanged against include/ode_gpu.h and
    against the reference. Its first dSpaceCollide comes before any step and
    needs no GPU, so both builds must print the same pairs for it; the
    reference build runs to the end."""
    import c_api_util as U
    if not U.ref_demo_available():
        pytest.skip("reference not built in this checkout")
    src = os.path.join(ROOT, "tests", "c_api", "space_stack_demo.c")
    with tempfile.TemporaryDirectory() as d:
        ours = U.build_gpu_demo(os.path.join(d, "ours"), src=src)
        ref = U.build_ref_demo(os.path.join(d, "ref"), src=src)
        r = subprocess.run([ref, "24", "30", "7"], capture_output=True, text=True, check=True)
        o = subprocess.run([ours, "24", "30", "7"], capture_output=True, text=True)
    ref_lines, our_lines = r.stdout.splitlines(), o.stdout.splitlines()
    assert ref_lines[0].startswith("pairs") and int(ref_lines[0].split()[1]) >= 8, ref_lines[0]
    assert our_lines[0] == ref_lines[0]
    assert len(ref_lines) == 2 * 30 + 24


def test_box_box_matches_reference_fp32():
    """dBoxBox (ode/src/box.cpp:331-713), the colliders' own host-and-device
    box-box routine, on seeded box pairs near contact against the
    reference's dSINGLE build: contact count, return code (set only on the
    paths that make contacts), normal, deepest penetration, and each
    contact's position and depth, bit for bit."""
    import ctypes as C
    import numpy as np
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    F, P, I = C.c_float, C.c_void_p, C.c_int
    V4, M12 = F * 4, F * 12

    class CG(C.Structure):
        _fields_ = [("pos", F * 4), ("normal", F * 4), ("depth", F), ("g1", P), ("g2", P), ("side1", I),
                    ("side2", I)]

    libs = [C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")),
            C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))]
    for lib in libs:
        lib.dBoxBox.argtypes = [P] * 7 + [P, P, I, P, I]
        lib.dRFromAxisAndAngle.argtypes = [P, F, F, F, F]
    rng = np.random.default_rng(17)
    worst, made, mism = 0.0, 0, 0
    for k in range(2000):
        ax = [float(x) for x in rng.normal(size=8)]
        s1, s2 = rng.uniform(0.3, 1.5, 3), rng.uniform(0.3, 1.5, 3)
        p2 = rng.normal(size=3) * 0.9
        res = []
        for lib in libs:
            R1, R2 = M12(), M12()
            lib.dRFromAxisAndAngle(R1, *ax[:4])
            lib.dRFromAxisAndAngle(R2, *ax[4:])
            normal, depth, code = V4(), F(-777.0), I(-777)
            buf = (CG * 8)()
            n = lib.dBoxBox(V4(0.1, 0.0, -0.2, 0), R1, V4(*s1, 0), V4(*p2, 0), R2, V4(*s2, 0), normal,
                            C.byref(depth), C.byref(code), 8, buf, C.sizeof(CG))
            res.append((n, code.value, list(normal)[:3], depth.value,
                        [list(buf[i].pos)[:3] + [buf[i].depth] for i in range(n)]))
        a, b = res
        if a[0] != b[0] or a[1] != b[1]:
            mism += 1   # only where the reference's deepest point is within rounding of touching
            assert max([c[3] for c in b[4]] + [0.0]) < 1e-4 and abs(b[3]) < 1e-3, (k, a, b)
            continue
        made += a[0] > 0
        if a[0] > 0:
            worst = max(worst, float(np.abs(np.array(a[2]) - b[2]).max()), abs(a[3] - b[3]),
                        float(np.abs(np.array(a[4]) - np.array(b[4])).max()))
    # measured: bit for bit on every pair (the host runs the same FP32 code
    # as the reference's dSINGLE build, in the same order)
    assert made > 300 and mism == 0, (made, mism)
    assert worst == 0.0, worst
