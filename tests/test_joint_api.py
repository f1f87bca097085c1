"""Joint calls of ODE's API that run on the host, against the reference's
dSINGLE build on seeded poses: the hinge2 and universal angle rates
(ode/src/joints/hinge2.cpp:357-390, universal.cpp:682-726), the universal
axis offsets (universal.cpp:418-556), dJointSetHingeAnchorDelta /
AxisOffset (hinge.cpp:163-230), dJointSetSliderAxisDelta (slider.cpp:243-262)
and dJointSetBallAnchor2 (ball.cpp:79-88), read back through the getters.
The setters' arithmetic is FP64 here and FP32 there."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F, P, I = C.c_float, C.c_void_p, C.c_int


def _bind(lib):
    for n in ("dWorldCreate", "dBodyCreate", "dJointCreateHinge2", "dJointCreateUniversal", "dJointCreateHinge",
              "dJointCreateSlider", "dJointCreateBall"):
        getattr(lib, n).restype = P
    lib.dBodyCreate.argtypes = [P]
    for n in ("dJointCreateHinge2", "dJointCreateUniversal", "dJointCreateHinge", "dJointCreateSlider",
              "dJointCreateBall"):
        getattr(lib, n).argtypes = [P, P]
    for n in ("dBodySetPosition", "dBodySetLinearVel", "dBodySetAngularVel"):
        getattr(lib, n).argtypes = [P, F, F, F]
    lib.dBodySetQuaternion.argtypes = [P, P]
    lib.dJointAttach.argtypes = [P, P, P]
    for n in ("dJointSetHinge2Anchor", "dJointSetHinge2Axis1", "dJointSetHinge2Axis2", "dJointSetUniversalAnchor",
              "dJointSetHingeAnchor", "dJointSetHingeAxis", "dJointSetBallAnchor", "dJointSetBallAnchor2",
              "dJointSetSliderAxis"):
        getattr(lib, n).argtypes = [P, F, F, F]
    lib.dJointSetUniversalAxis1Offset.argtypes = lib.dJointSetUniversalAxis2Offset.argtypes = [P, F, F, F, F, F]
    lib.dJointSetHingeAnchorDelta.argtypes = lib.dJointSetSliderAxisDelta.argtypes = [P, F, F, F, F, F, F]
    lib.dJointSetHingeAxisOffset.argtypes = [P, F, F, F, F]
    for n in ("dJointGetHinge2Angle1Rate", "dJointGetHinge2Angle2Rate", "dJointGetUniversalAngle1Rate",
              "dJointGetUniversalAngle2Rate", "dJointGetUniversalAngle1", "dJointGetUniversalAngle2",
              "dJointGetHingeAngle", "dJointGetHingeAngleRate", "dJointGetSliderPosition", "dJointGetHinge2Angle1"):
        getattr(lib, n).restype = F
        getattr(lib, n).argtypes = [P]
    for n in ("dJointGetHingeAnchor", "dJointGetHingeAnchor2", "dJointGetBallAnchor2", "dJointGetUniversalAxis1",
              "dJointGetUniversalAxis2", "dJointGetHingeAxis"):
        getattr(lib, n).argtypes = [P, P]
    lib.dWorldDestroy.argtypes = [P]
    return lib


def _q(rng):
    q = rng.normal(size=4)
    return (F * 4)(*(q / np.linalg.norm(q)).astype(np.float32))


def _program(lib, seed):
    rng = np.random.default_rng(seed)
    f = lambda n: [float(x) for x in rng.normal(size=n)]
    w = lib.dWorldCreate()
    bs = []
    for _ in range(4):
        b = lib.dBodyCreate(w)
        lib.dBodySetPosition(b, *f(3))
        lib.dBodySetQuaternion(b, _q(rng))
        lib.dBodySetLinearVel(b, *f(3))
        lib.dBodySetAngularVel(b, *f(3))
        bs.append(b)
    out = []
    v = (F * 4)()
    # hinge2 rates
    h2 = lib.dJointCreateHinge2(w, None)
    lib.dJointAttach(h2, bs[0], bs[1])
    lib.dJointSetHinge2Anchor(h2, *f(3))
    lib.dJointSetHinge2Axis1(h2, 0.0, 0.0, 1.0)
    lib.dJointSetHinge2Axis2(h2, 0.0, 1.0, 0.2)
    out += [lib.dJointGetHinge2Angle1Rate(h2), lib.dJointGetHinge2Angle2Rate(h2)]
    # universal offsets and rates, straight and reversed
    for b1, b2 in ((bs[0], bs[2]), (None, bs[3]), (bs[1], None)):
        u = lib.dJointCreateUniversal(w, None)
        lib.dJointAttach(u, b1, b2)
        lib.dJointSetUniversalAnchor(u, *f(3))
        a = f(3)
        offs = [0.5 * x for x in f(2)]
        # reversed onto one body, Axis1Offset builds a rotation from the axis
        # and itself: ODE 0.12's dRFrom2Axes returns on the zero vector and
        # leaves its matrix uninitialised (universal.cpp:449-453), so that
        # case has no defined answer there and is left out
        if b1 is not None:
            lib.dJointSetUniversalAxis1Offset(u, *a, *offs)
        out += [lib.dJointGetUniversalAngle1(u), lib.dJointGetUniversalAngle2(u),
                lib.dJointGetUniversalAngle1Rate(u), lib.dJointGetUniversalAngle2Rate(u)]
        lib.dJointGetUniversalAxis1(u, v)
        out += list(v)[:3]
        b = np.cross(a, f(3))
        lib.dJointSetUniversalAxis2Offset(u, *[float(x) for x in b], *[0.5 * x for x in f(2)])
        out += [lib.dJointGetUniversalAngle1(u), lib.dJointGetUniversalAngle2(u)]
        lib.dJointGetUniversalAxis2(u, v)
        out += list(v)[:3]
    # hinge anchor delta and axis offset, to a body and to the environment
    for b1, b2 in ((bs[1], bs[2]), (bs[3], None), (None, bs[0])):
        h = lib.dJointCreateHinge(w, None)
        lib.dJointAttach(h, b1, b2)
        lib.dJointSetHingeAnchorDelta(h, *f(6))
        lib.dJointGetHingeAnchor(h, v)
        out += list(v)[:3]
        lib.dJointGetHingeAnchor2(h, v)
        out += list(v)[:3]
        lib.dJointSetHingeAxisOffset(h, *f(3), 0.7 * f(1)[0])
        out += [lib.dJointGetHingeAngle(h), lib.dJointGetHingeAngleRate(h)]
    # slider axis delta, to the environment and to a body
    for b1, b2 in ((bs[2], None), (bs[0], bs[3])):
        s = lib.dJointCreateSlider(w, None)
        lib.dJointAttach(s, b1, b2)
        lib.dJointSetSliderAxisDelta(s, *f(6))
        out += [lib.dJointGetSliderPosition(s)]
    # ball anchor 2, as given
    bj = lib.dJointCreateBall(w, None)
    lib.dJointAttach(bj, bs[0], bs[1])
    lib.dJointSetBallAnchor(bj, *f(3))
    lib.dJointSetBallAnchor2(bj, *f(3))
    lib.dJointGetBallAnchor2(bj, v)
    out += list(v)[:3]
    lib.dWorldDestroy(w)
    return np.array(out, dtype=np.float64)


def test_joint_rates_offsets_and_deltas_match_reference_fp32():
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = _bind(C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")))
    ref = _bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))
    for seed in range(60):
        a, b = _program(ours, seed), _program(ref, seed)
        err = np.abs(a - b) / (1.0 + np.abs(b))
        # FP64 setters here against FP32 ones there (measured 2.2e-6), plus angles through
        # atan2 near +-pi where an FP32 rounding can flip the branch
        flips = np.abs(np.abs(a - b) - 2 * np.pi) < 1e-3
        assert ((err <= 2e-5) | flips).all(), (seed, int(np.argmax(err)), a[np.argmax(err)], b[np.argmax(err)])
