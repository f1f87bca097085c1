"""The body-update options of ODE's API (damping, the angular speed cap,
finite rotation, moved callbacks, body geom lists: ode/src/ode.cpp:767-806,
:1000-1133, :1930-2011) on the host: every getter's answer after a seeded
sequence of world and body settings equals the reference's dSINGLE build's,
bit for bit. The steps that apply them run on the GPU
(tests/test_gpu_ode_api.py, against tests/golden/body_step_options.npz)."""
import ctypes as C
import os

import numpy as np
import pytest

import body_step_program as BP

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_body_option_getters_match_reference():
    import oracle_lib as O
    g = np.load(os.path.join(ROOT, "tests", "golden", "body_step_options.npz"))
    ours = BP.bind(C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        got, _, _ = BP.program(ours, int(s), 1)   # the step itself fails without a device
        assert np.array_equal(got, g[f"dWorldQuickStep_{s}_getters"]), int(s)
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ref = BP.bind(C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so")))
    for s in range(4, 12):
        a, _, _ = BP.program(ours, s, 1)
        b, _, _ = BP.program(ref, s, 1)
        assert np.array_equal(a, b), s


def _autodisable_program(lib, n_steps=16):
    """Auto-disable (ode/src/util.cpp:98-230) on free bodies of spherical mass
    without gravity, so velocities stay as set and the decisions depend on
    the settings alone: idle from the start, below and above either
    threshold, no joint (never frozen in mid-air), a two-sample average of
    alternating velocities, an idle time, the flag turned off, and a body
    enabled again after it was disabled. Each body but the mid-air one hangs
    on a null joint. Returns the getters and, per step, the enabled flags and
    the velocities."""
    F, P = C.c_float, C.c_void_p
    for n in ("dWorldCreate", "dBodyCreate", "dJointCreateNull"):
        getattr(lib, n).restype = P
    lib.dBodyCreate.argtypes = [P]
    lib.dJointCreateNull.argtypes = [P, P]
    lib.dJointAttach.argtypes = [P, P, P]
    lib.dBodySetLinearVel.argtypes = lib.dBodySetAngularVel.argtypes = [P, F, F, F]
    lib.dBodyGetLinearVel.restype = lib.dBodyGetAngularVel.restype = C.POINTER(F)
    lib.dBodyGetLinearVel.argtypes = lib.dBodyGetAngularVel.argtypes = [P]
    lib.dWorldSetGravity.argtypes = [P, F, F, F]
    lib.dWorldSetAutoDisableFlag.argtypes = [P, C.c_int]
    lib.dWorldGetAutoDisableFlag.argtypes = [P]
    for n in ("dWorldGetAutoDisableLinearThreshold", "dWorldGetAutoDisableAngularThreshold",
              "dWorldGetAutoDisableTime", "dBodyGetAutoDisableTime", "dBodyGetAutoDisableLinearThreshold"):
        getattr(lib, n).restype = F
        getattr(lib, n).argtypes = [P]
    lib.dWorldSetAutoDisableLinearThreshold.argtypes = [P, F]
    lib.dBodySetAutoDisableSteps.argtypes = [P, C.c_int]
    lib.dBodySetAutoDisableTime.argtypes = lib.dBodySetAutoDisableAngularThreshold.argtypes = [P, F]
    lib.dBodySetAutoDisableAverageSamplesCount.argtypes = [P, C.c_uint]
    lib.dBodySetAutoDisableFlag.argtypes = [P, C.c_int]
    for n in ("dBodyGetAutoDisableFlag", "dBodyGetAutoDisableSteps", "dBodyGetAutoDisableAverageSamplesCount",
              "dWorldGetAutoDisableSteps", "dWorldGetAutoDisableAverageSamplesCount", "dBodyIsEnabled"):
        getattr(lib, n).argtypes = [P]
    lib.dBodyEnable.argtypes = [P]
    lib.dMassSetSphere.argtypes = [P, F, F]
    lib.dBodySetMass.argtypes = [P, P]
    lib.dWorldQuickStep.argtypes = [P, F]
    lib.dWorldDestroy.argtypes = [P]
    lib.dInitODE2(0)
    w = lib.dWorldCreate()
    lib.dWorldSetGravity(w, 0.0, 0.0, 0.0)
    got = [lib.dWorldGetAutoDisableFlag(w), lib.dWorldGetAutoDisableLinearThreshold(w),
           lib.dWorldGetAutoDisableSteps(w), lib.dWorldGetAutoDisableAverageSamplesCount(w)]
    lib.dWorldSetAutoDisableFlag(w, 1)
    lib.dWorldSetAutoDisableLinearThreshold(w, 0.02)
    got += [lib.dWorldGetAutoDisableFlag(w), lib.dWorldGetAutoDisableLinearThreshold(w),
            lib.dWorldGetAutoDisableAngularThreshold(w), lib.dWorldGetAutoDisableTime(w)]
    b = []
    for k in range(9):
        bb = lib.dBodyCreate(w)
        m = BP.Mass()
        lib.dMassSetSphere(C.byref(m), 1.0, 0.3)
        lib.dBodySetMass(bb, C.byref(m))
        if k != 4:
            j = lib.dJointCreateNull(w, None)
            lib.dJointAttach(j, bb, None)
        b.append(bb)
    lib.dBodySetLinearVel(b[1], 0.01, 0.0, 0.005)      # below 0.02
    lib.dBodySetLinearVel(b[2], 0.05, 0.0, 0.0)        # above
    lib.dBodySetAngularVel(b[3], 0.0, 0.02, 0.0)       # above the angular 0.01
    lib.dBodySetAutoDisableAverageSamplesCount(b[5], 2)
    lib.dBodySetAutoDisableSteps(b[6], 1)
    lib.dBodySetAutoDisableTime(b[6], 0.05)
    lib.dBodySetAutoDisableFlag(b[7], 0)
    lib.dBodySetAutoDisableSteps(b[8], 3)
    for bb in b:
        got += [lib.dBodyGetAutoDisableFlag(bb), lib.dBodyGetAutoDisableSteps(bb), lib.dBodyGetAutoDisableTime(bb),
                lib.dBodyGetAutoDisableAverageSamplesCount(bb), lib.dBodyGetAutoDisableLinearThreshold(bb)]
    flags, vel = [], []
    for step in range(n_steps):
        lib.dBodySetLinearVel(b[5], 0.05 if step % 2 else -0.05, 0.0, 0.0)   # averages to 0
        if step == 6:
            lib.dBodyEnable(b[8])
        lib.dWorldQuickStep(w, 0.01)
        flags.append([lib.dBodyIsEnabled(bb) for bb in b])
        v = []
        for bb in b:
            lv, av = lib.dBodyGetLinearVel(bb), lib.dBodyGetAngularVel(bb)
            v += [lv[0], lv[1], lv[2], av[0], av[1], av[2]]
        vel.append(v)
    lib.dWorldDestroy(w)
    return np.array(got, dtype=np.float64), np.array(flags), np.array(vel, dtype=np.float64)


def test_auto_disable_matches_reference():
    """The auto-disable check runs on the host before the GPU step (a step
    without a device fails after it), so with velocities that no step changes
    the decisions compare with the reference's dSINGLE build over 16 steps:
    getters, enabled flags and zeroed velocities exactly."""
    import oracle_lib as O
    if not O.ref_available("s"):
        pytest.skip("reference not built in this checkout")
    ours = C.CDLL(os.path.join(ROOT, "ode-0.12_gb300", "libodegpu.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libode_ref_s.so"))
    a, b = _autodisable_program(ours), _autodisable_program(ref)
    assert np.array_equal(a[0], b[0]), (a[0], b[0])
    assert np.array_equal(a[1], b[1]), (a[1], b[1])
    assert np.array_equal(a[2], b[2])
    assert a[1][-1].tolist() != [1] * 9 and a[1][0].tolist() == [1] * 9   # some bodies went to sleep
