"""The ODE-compatible C API (include/ode_gpu.h) on the GPU: plain ODE
programs (tests/c_api/box_drop_demo.c, tests/c_api/scene_player.c) linked
against libodegpu, and dCollide on the reference's collider known-answer
poses."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest

from odegpu import scene as S
import c_api_util as U
import oracle_lib as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_demo_program_matches_batch_path_and_oracle():
    """100 steps of the 20-box drop through dCollide + dJointCreateContact +
    dWorldQuickStep + dJointGroupEmpty. Same kernels as the batched path, so
    the states agree to FP32 rounding (1e-5); against the FP64 oracle the
    chaotic drop stays within 5 mm over 100 steps."""
    from odegpu.batch import Batch
    sc = S.box_drop(seed=0)
    steps = 100
    with tempfile.TemporaryDirectory() as d:
        exe = U.build_gpu_demo(os.path.join(d, "demo"))
        inp = os.path.join(d, "in.txt")
        U.scene_input(sc, steps, inp)
        st = U.run_demo(exe, inp)
    B = Batch(sc)
    B.step(steps)
    bt = B.state()
    assert np.abs(st[:, :3] - bt[:, :3]).max() < 1e-5
    assert np.abs(st[:, 7:] - bt[:, 7:]).max() < 1e-3
    ref = O.run_world(O.oracle().oracle_run_world, sc, 0, steps)["state"][-1]
    assert np.abs(st[:, :3] - ref[:, :3]).max() < 5e-3


def test_scene_player_joint_types_on_gpu():
    """tests/c_api/scene_player.c (plain ODE calls: dJointCreateSlider /
    Universal / Fixed with their setters and per-step dJointAddSliderForce,
    dJointAddUniversalTorques, dJointSet*Param stops) linked against
    libodegpu, on the joint-type scene. Same kernels as the batched path, so
    after 40 steps the states agree to 1e-4 m / 1e-2 m/s (the API path takes
    FP32 inputs for its FP64 setters and sums controls on the host); against
    the FP64 oracle within 2e-3 m after 20 steps."""
    from odegpu.batch import Batch
    sc = S.mechanisms(n_worlds=3, steps=40)
    steps = 40
    B = Batch(sc)
    B.step(steps)
    bt = B.state()
    B.close()
    with tempfile.TemporaryDirectory() as d:
        exe = U.build_gpu_demo(os.path.join(d, "player"), src=U.PLAYER)
        for w in range(sc.n_worlds):
            b0, b1 = sc.world_bodies(w)
            inp = os.path.join(d, "in.txt")
            U.player_input(sc, w, steps, inp)
            st = U.run_demo(exe, inp)
            assert np.abs(st[:, :3] - bt[b0:b1, :3]).max() < 1e-4, w
            assert np.abs(st[:, 7:] - bt[b0:b1, 7:]).max() < 1e-2, w
            U.player_input(sc, w, 20, inp)
            st = U.run_demo(exe, inp)
            ref = O.run_world(O.oracle().oracle_run_world, sc, w, 20)["state"][-1]
            assert np.abs(st[:, :3] - ref[:, :3]).max() < 2e-3, w


def test_scene_player_dworldstep_on_gpu():
    """scene_player.c stepping with dWorldStep (ode.cpp:1787), linked against
    libodegpu, on the joint-type scene: agrees with the batched dWorldStep
    path after 40 steps and with the FP64 oracle's dWorldStep after 20."""
    from odegpu.batch import Batch
    sc = S.mechanisms(n_worlds=2, steps=40)
    steps = 40
    B = Batch(sc)
    B.set_stepper(True)
    B.step(steps)
    bt = B.state()
    B.close()
    with tempfile.TemporaryDirectory() as d:
        exe = U.build_gpu_demo(os.path.join(d, "player"), src=U.PLAYER)
        for w in range(sc.n_worlds):
            b0, b1 = sc.world_bodies(w)
            inp = os.path.join(d, "in.txt")
            U.player_input(sc, w, steps, inp)
            st = U.run_demo(exe, inp, "exact")
            assert np.abs(st[:, :3] - bt[b0:b1, :3]).max() < 1e-4, w
            U.player_input(sc, w, 20, inp)
            st = U.run_demo(exe, inp, "exact")
            with O.exact_stepper():
                ref = O.run_world(O.oracle().oracle_run_world, sc, w, 20)["state"][-1]
            assert np.abs(st[:, :3] - ref[:, :3]).max() < 2e-3, w


def test_scene_player_cylinders_on_gpu():
    """scene_player.c with dCreateCylinder geoms (the plane world of the
    cylinder pile) linked against libodegpu: agrees with the batched path
    after 60 steps (same kernels; FP32 inputs to the host setters)."""
    from odegpu.batch import Batch
    sc = S.cylinder_pile(n_worlds=1)
    steps = 60
    B = Batch(sc)
    B.step(steps)
    bt = B.state()
    B.close()
    with tempfile.TemporaryDirectory() as d:
        exe = U.build_gpu_demo(os.path.join(d, "player"), src=U.PLAYER)
        inp = os.path.join(d, "in.txt")
        U.player_input(sc, 0, steps, inp)
        st = U.run_demo(exe, inp)
        assert np.abs(st[:, :3] - bt[:, :3]).max() < 1e-4
        assert np.abs(st[:, 7:] - bt[:, 7:]).max() < 1e-2


def _api():
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dCreateSphere.restype = v; L.dCreateSphere.argtypes = [v, f]
    L.dCreateBox.restype = v; L.dCreateBox.argtypes = [v, f, f, f]
    L.dCreatePlane.restype = v; L.dCreatePlane.argtypes = [v, f, f, f, f]
    L.dCreateCapsule.restype = v; L.dCreateCapsule.argtypes = [v, f, f]
    L.dCreateCylinder.restype = v; L.dCreateCylinder.argtypes = [v, f, f]
    L.dGeomSetPosition.argtypes = [v, f, f, f]
    L.dGeomSetRotation.argtypes = [v, C.POINTER(f)]
    L.dGeomDestroy.argtypes = [v]
    L.dCollide.restype = i; L.dCollide.argtypes = [v, v, i, v, i]
    return L


class ContactGeom(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("normal", C.c_float * 4), ("depth", C.c_float),
                ("g1", C.c_void_p), ("g2", C.c_void_p), ("side1", C.c_int), ("side2", C.c_int)]


def test_dcollide_on_reference_kats():
    """dCollide through the ODE API on the GPU for every collider on the path,
    against the reference's FP64 outputs: contact counts equal except where the
    deepest point is within 1e-5 of touching; positions/normals/depths within
    FP32 tolerance (depth only where the reference's normal is undefined)."""
    g = np.load(os.path.join(GOLDEN, "collider_kats.npz"))
    L = _api()
    n = len(g["t1"])
    count_mism = near = 0
    worst = 0.0
    mk = {0: lambda p: L.dCreateSphere(None, p[0]), 1: lambda p: L.dCreateBox(None, p[0], p[1], p[2]),
          2: lambda p: L.dCreateCapsule(None, p[0], p[1]),
          4: lambda p: L.dCreatePlane(None, p[0], p[1], p[2], p[3])}
    for k in range(n):
        geoms = []
        for t, p, pos, R in ((g["t1"][k], g["p1"][k], g["pos1"][k], g["R1"][k]),
                             (g["t2"][k], g["p2"][k], g["pos2"][k], g["R2"][k])):
            h = mk[int(t)](p)
            if t != 4:
                L.dGeomSetPosition(h, *pos)
                R4 = (C.c_float * 12)(*[R[0], R[1], R[2], 0, R[3], R[4], R[5], 0, R[6], R[7], R[8], 0])
                L.dGeomSetRotation(h, R4)
            geoms.append(h)
        out = (ContactGeom * 16)()
        nc = L.dCollide(geoms[0], geoms[1], int(g["flags"][k]), out, C.sizeof(ContactGeom))
        ref_n = int(g["nc"][k])
        ref = g["out"][k]
        if nc != ref_n:
            deepest = ref[:max(ref_n, 1), 6].max() if ref_n else 0.0
            if ref_n and deepest > 1e-5:
                count_mism += 1
            else:
                near += 1
        else:
            t1, t2 = int(g["t1"][k]), int(g["t2"][k])
            # capsule-box with the capsule's axis inside the box: the closest
            # line and box points coincide, and the reference takes the normal
            # (and the position built on it) from rounding noise of pl - pb
            # (dCollideCapsuleBox, ode/src/capsule.cpp:216-228); only the depth
            # (the radius) is defined there
            rc = g["p1"][k][0] if t1 == 2 else g["p2"][k][0]
            degenerate = {t1, t2} == {1, 2} and nc and abs(ref[0, 6] - rc) < 1e-4
            for c in range(nc):
                got = np.array(list(out[c].pos[:3]) + list(out[c].normal[:3]) + [out[c].depth])
                cols = [6] if degenerate else list(range(7))
                worst = max(worst, np.abs(got[cols] - ref[c, cols]).max())
        for h in geoms:
            L.dGeomDestroy(h)
    assert count_mism <= n // 200, (count_mism, near)
    assert worst < 1e-3, worst


def test_dcollide_with_offset_geoms():
    """A geom placed on its body by an offset (ode/src/collision_kernel.cpp:
    1036-1250) collides from its final pose, body.R * offset + body.pos
    (dxGeom::computePosr, :454-465): dCollide of the offset geom equals dCollide
    of a free geom put at that pose, bit for bit, and the pose follows the body
    through a dWorldQuickStep."""
    L = _api()
    f, v = C.c_float, C.c_void_p
    for n in ("dWorldCreate", "dBodyCreate"):
        getattr(L, n).restype = v
    L.dBodyCreate.argtypes = [v]
    L.dWorldSetGravity.argtypes = [v, f, f, f]
    L.dWorldQuickStep.argtypes = [v, f]
    L.dWorldDestroy.argtypes = [v]
    L.dBodySetPosition.argtypes = [v, f, f, f]
    L.dBodySetRotation.argtypes = [v, C.POINTER(f)]
    L.dBodySetAngularVel.argtypes = [v, f, f, f]
    L.dBodyGetPosition.restype = L.dBodyGetRotation.restype = C.POINTER(f)
    L.dBodyGetPosition.argtypes = L.dBodyGetRotation.argtypes = [v]
    L.dRFromAxisAndAngle.argtypes = [C.POINTER(f), f, f, f, f]
    L.dGeomSetBody.argtypes = [v, v]
    L.dGeomSetOffsetPosition.argtypes = [v, f, f, f]
    L.dGeomSetOffsetRotation.argtypes = [v, C.POINTER(f)]
    L.dGeomGetPosition.restype = L.dGeomGetRotation.restype = C.POINTER(f)
    L.dGeomGetPosition.argtypes = L.dGeomGetRotation.argtypes = [v]
    M12 = f * 12

    def rot(a):
        R = M12()
        L.dRFromAxisAndAngle(R, *a)
        return R

    def contacts(g1, g2):
        out = (ContactGeom * 8)()
        n = L.dCollide(g1, g2, 8, out, C.sizeof(ContactGeom))
        return n, [list(out[c].pos[:3]) + list(out[c].normal[:3]) + [out[c].depth] for c in range(n)]

    rng = np.random.default_rng(53)
    hits = 0
    for _ in range(40):
        a = [float(x) for x in rng.normal(size=16)]
        w = L.dWorldCreate()
        L.dWorldSetGravity(w, 0.0, 0.0, -9.81)
        b = L.dBodyCreate(w)
        L.dBodySetPosition(b, *a[0:3])
        L.dBodySetRotation(b, rot(a[3:7]))
        L.dBodySetAngularVel(b, *a[13:16])
        g = L.dCreateBox(None, 0.6, 0.4, 0.8)
        L.dGeomSetBody(g, b)
        L.dGeomSetOffsetPosition(g, 0.5 * a[7], 0.5 * a[8], 0.5 * a[9])
        L.dGeomSetOffsetRotation(g, rot(a[9:13]))
        gp = L.dGeomGetPosition(g)
        s = L.dCreateSphere(None, 0.35)
        L.dGeomSetPosition(s, gp[0] + 0.3 * a[10], gp[1] + 0.3 * a[11], gp[2] + 0.3 * a[12])
        free = L.dCreateBox(None, 0.6, 0.4, 0.8)
        L.dGeomSetPosition(free, gp[0], gp[1], gp[2])
        gR = L.dGeomGetRotation(g)
        L.dGeomSetRotation(free, M12(*[gR[k] for k in range(12)]))
        n1, c1 = contacts(g, s)
        n2, c2 = contacts(free, s)
        assert n1 == n2 and c1 == c2, (n1, n2)
        n3, c3 = contacts(s, g)
        n4, c4 = contacts(s, free)
        assert n3 == n4 and c3 == c4, (n3, n4)
        hits += n1 > 0
        assert L.dWorldQuickStep(w, 0.01) == 1
        bp, bR = L.dBodyGetPosition(b), L.dBodyGetRotation(b)
        Rb = np.array([[bR[r * 4 + c] for c in range(3)] for r in range(3)], dtype=np.float32)
        want = Rb @ np.float32([0.5 * a[7], 0.5 * a[8], 0.5 * a[9]]) + np.float32([bp[0], bp[1], bp[2]])
        gp = L.dGeomGetPosition(g)
        assert np.allclose([gp[0], gp[1], gp[2]], want, atol=1e-5)
        for h in (g, s, free):
            L.dGeomDestroy(h)
        L.dWorldDestroy(w)
    assert hits >= 10, hits


@pytest.mark.parametrize("stepper", ["dWorldQuickStep", "dWorldStep"])
def test_space_order_after_steps_matches_reference(stepper):
    """A simple space through world steps (tests/space_program.py
    step_program): each step notifies every body's geoms in island order
    (util.cpp:334-336 from quickstep.cpp:1004-1008 / step.cpp:810-812, islands
    by util.cpp:413-470), which moves them to the front of the space. The space
    order and the near-callback's pairs after every step equal the reference's
    dSINGLE build's (tests/golden/space_order.npz), entry for entry."""
    import space_program as SP
    g = np.load(os.path.join(GOLDEN, "space_order.npz"))
    L = SP.bind(C.CDLL(os.path.join(os.path.dirname(GOLDEN), "..", "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        got = SP.step_program(L, int(s), int(g["n_steps"]), stepper)
        want = g[f"{stepper}_{s}"]
        assert np.array_equal(got, want), (int(s), got[:40], want[:40])


@pytest.mark.parametrize("stepper", ["dWorldQuickStep", "dWorldStep"])
def test_body_step_options_match_reference(stepper):
    """Damping, the angular speed cap and finite rotation (with and without an
    axis) in the step's body update on the GPU (dxStepBody,
    ode/src/util.cpp:255-360) against the reference's dSINGLE build over 30
    steps of spinning, falling bodies (tests/body_step_program.py,
    tests/golden/body_step_options.npz): states within 1e-4 (1 + |x|), the
    moved callbacks in the reference's island order, the getters exact. Each
    option changes the states by far more than the tolerance (damping by a
    few percent of the velocities per step, the cap from 8 to 3 rad/s, finite
    against infinitesimal rotation by about 1e-3 per step at 25 rad/s)."""
    import body_step_program as BP
    g = np.load(os.path.join(GOLDEN, "body_step_options.npz"))
    L = BP.bind(C.CDLL(os.path.join(os.path.dirname(GOLDEN), "..", "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        got_g, got_x, got_m = BP.program(L, int(s), int(g["n_steps"]), stepper)
        want_x = g[f"{stepper}_{s}_states"]
        assert np.array_equal(got_g, g[f"{stepper}_{s}_getters"])
        assert np.array_equal(got_m, g[f"{stepper}_{s}_moved"])
        err = np.abs(got_x - want_x) / (1.0 + np.abs(want_x))
        assert err.max() <= 1e-4, (int(s), float(err.max()), np.unravel_index(np.argmax(err), err.shape))


@pytest.mark.parametrize("stepper", ["dWorldQuickStep", "dWorldStep"])
def test_disabled_bodies_and_null_joints_match_reference(stepper):
    """Islands with null joints (ode/src/joints/null.cpp: no rows, one island)
    and disabled bodies (util.cpp:413-470: reached ones are woken, the rest are
    not stepped and keep their forces) against the reference's dSINGLE build
    over 12 steps of boxes on ground contacts (tests/body_step_program.py
    island_program): the RNG seed after every step exactly (SOR's shuffle
    draws follow each island's row count, so a wrongly merged or split island
    changes it), the enabled flags, the moved-callback order and the kept
    forces exactly, states within 1e-4 (1 + |x|)."""
    import body_step_program as BP
    g = np.load(os.path.join(GOLDEN, "body_step_options.npz"))
    L = BP.bind_islands(C.CDLL(os.path.join(os.path.dirname(GOLDEN), "..", "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        seeds, flags, states, moved, kept = BP.island_program(L, int(s), 12, stepper)
        pre = f"islands_{stepper}_{s}_"
        assert np.array_equal(seeds, g[pre + "seeds"]), (int(s), seeds, g[pre + "seeds"])
        assert np.array_equal(flags, g[pre + "enabled"])
        assert np.array_equal(moved, g[pre + "moved"])
        assert np.array_equal(kept, g[pre + "kept_force"])
        want = g[pre + "states"]
        err = np.abs(states - want) / (1.0 + np.abs(want))
        assert err.max() <= 1e-4, (int(s), float(err.max()))


@pytest.mark.parametrize("stepper", ["dWorldQuickStep", "dWorldStep"])
def test_kinematic_bodies_match_reference(stepper):
    """A kinematic body (zero inverse mass and inertia, ode.cpp:834-852) in a
    ball joint and a contact, stepped on the GPU, against the reference's
    dSINGLE build over 20 steps (tests/body_step_program.py
    kinematic_program): the kinematic body moves by its set velocities
    untouched by gravity or constraints, the others follow; states within
    1e-4 (1 + |x|), IsKinematic answers exactly."""
    import body_step_program as BP
    g = np.load(os.path.join(GOLDEN, "body_step_options.npz"))
    L = BP.bind_islands(C.CDLL(os.path.join(os.path.dirname(GOLDEN), "..", "ode-0.12_gb300", "libodegpu.so")))
    for s in g["seeds"]:
        flags, states = BP.kinematic_program(L, int(s), 20, stepper)
        assert np.array_equal(flags, g[f"kinematic_{stepper}_{s}_flags"])
        want = g[f"kinematic_{stepper}_{s}_states"]
        err = np.abs(states - want) / (1.0 + np.abs(want))
        assert err.max() <= 1e-4, (int(s), float(err.max()), np.unravel_index(np.argmax(err), err.shape))


class JointFeedback(C.Structure):
    _fields_ = [("f1", C.c_float * 4), ("t1", C.c_float * 4), ("f2", C.c_float * 4), ("t2", C.c_float * 4)]


class Mass(C.Structure):
    _fields_ = [("mass", C.c_float), ("c", C.c_float * 4), ("I", C.c_float * 12)]


@pytest.mark.parametrize("stepper", ["dWorldQuickStep", "dWorldStep"])
def test_joint_feedback_through_ode_api(stepper):
    """dJointSetFeedback on a three-link ball chain hanging at rest from the
    environment: after a step the top joint's f1 carries the chain's weight,
    the middle joint two links' weight (force on body 1 = J1^T lambda), and f2
    of the lower joints is the reaction on the link below; with either
    stepper."""
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dWorldCreate.restype = v
    L.dWorldSetGravity.argtypes = [v, f, f, f]
    L.dWorldSetCFM.argtypes = [v, f]
    L.dBodyCreate.restype = v; L.dBodyCreate.argtypes = [v]
    L.dBodySetPosition.argtypes = [v, f, f, f]
    L.dMassSetSphereTotal.argtypes = [C.POINTER(Mass), f, f]
    L.dBodySetMass.argtypes = [v, C.POINTER(Mass)]
    L.dJointCreateBall.restype = v; L.dJointCreateBall.argtypes = [v, v]
    L.dJointAttach.argtypes = [v, v, v]
    L.dJointSetBallAnchor.argtypes = [v, f, f, f]
    L.dJointSetFeedback.argtypes = [v, C.POINTER(JointFeedback)]
    step = getattr(L, stepper)
    step.restype = i; step.argtypes = [v, f]
    L.dWorldDestroy.argtypes = [v]
    w = L.dWorldCreate()
    L.dWorldSetGravity(w, 0.0, 0.0, -9.81)
    L.dWorldSetCFM(w, 1e-5)
    m = 2.0
    bodies, joints, fbs = [], [], []
    for k in range(3):
        b = L.dBodyCreate(w)
        L.dBodySetPosition(b, 0.0, 0.0, -0.5 - k)
        M = Mass()
        L.dMassSetSphereTotal(C.byref(M), m, 0.1)
        L.dBodySetMass(b, C.byref(M))
        bodies.append(b)
    for k in range(3):
        j = L.dJointCreateBall(w, None)
        L.dJointAttach(j, bodies[k], bodies[k - 1] if k > 0 else None)
        L.dJointSetBallAnchor(j, 0.0, 0.0, -float(k))
        fb = JointFeedback()
        L.dJointSetFeedback(j, C.byref(fb))
        joints.append(j)
        fbs.append(fb)
    for _ in range(5):
        assert step(w, 0.01) == 1
    weight = m * 9.81
    # joint k holds link k (body 1) to link k-1 / the environment (body 2)
    for k in range(3):
        f1 = np.array(fbs[k].f1[:3])
        assert abs(f1[2] - (3 - k) * weight) < 0.05 * weight, (k, f1)
        assert np.abs(f1[:2]).max() < 0.05 * weight
        if k > 0:
            f2 = np.array(fbs[k].f2[:3])
            assert np.abs(f2 + f1).max() < 1e-3 * weight, (k, f1, f2)
        else:
            assert np.array(fbs[k].f2[:3]).tolist() == [0.0, 0.0, 0.0]
    L.dWorldDestroy(w)


@pytest.mark.parametrize("fixture", ["hf_kats", "hf_big_kats"])
@pytest.mark.parametrize("build", ["double", "callback"])
def test_dcollide_heightfield_through_ode_api(fixture, build):
    """dGeomHeightfieldDataBuildDouble (or BuildCallback over the same
    samples) + dCreateHeightfield (placeable) +
    dCollide on the reference's golden heightfield calls, in both argument
    orders (the reversed call negates the normals): counts exact, records
    within 1e-4 (of the coordinates' scale, ~12 m, for hf_big_kats, whose
    geoms cover more than the lane's 10 x 10 samples)."""
    g = np.load(os.path.join(GOLDEN, f"{fixture}.npz"))
    scale = 1.0 if fixture == "hf_kats" else 12.0
    L = _api()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dGeomHeightfieldDataCreate.restype = v
    L.dGeomHeightfieldDataBuildDouble.argtypes = [v, C.POINTER(C.c_double), i, f, f, i, i, f, f, f, i]
    L.dCreateHeightfield.restype = v
    L.dCreateHeightfield.argtypes = [v, v, i]
    L.dGeomHeightfieldDataDestroy.argtypes = [v]
    h = np.ascontiguousarray(g["heights"], dtype=np.float64)
    sp = float(g["spacing"])
    nz, nx = h.shape
    hd = L.dGeomHeightfieldDataCreate()
    # the same samples through dGeomHeightfieldDataBuildCallback (sampled at build)
    HCB = C.CFUNCTYPE(f, v, i, i)
    cb = HCB(lambda _, x, z: float(h[z, x]))
    if build == "double":
        L.dGeomHeightfieldDataBuildDouble(hd, h.ctypes.data_as(C.POINTER(C.c_double)), 1, sp * (nx - 1),
                                          sp * (nz - 1), nx, nz, 1.0, 0.0, 1.0, 0)
    else:
        L.dGeomHeightfieldDataBuildCallback.argtypes = [v, v, HCB, f, f, i, i, f, f, f, i]
        L.dGeomHeightfieldDataBuildCallback(hd, None, cb, sp * (nx - 1), sp * (nz - 1), nx, nz, 1.0, 0.0, 1.0, 0)
    hg = L.dCreateHeightfield(None, hd, 1)
    L.dGeomSetPosition(hg, *[float(x) for x in g["hf_pos"]])
    Rh = g["hf_R"]
    L.dGeomSetRotation(hg, (C.c_float * 12)(*[Rh[0], Rh[1], Rh[2], 0, Rh[3], Rh[4], Rh[5], 0, Rh[6], Rh[7],
                                               Rh[8], 0]))
    mk = {0: lambda p: L.dCreateSphere(None, p[0]), 1: lambda p: L.dCreateBox(None, p[0], p[1], p[2]),
          2: lambda p: L.dCreateCapsule(None, p[0], p[1]), 3: lambda p: L.dCreateCylinder(None, p[0], p[1])}
    n = len(g["t2"])
    count_mism, worst = [], 0.0
    for k in range(n):
        t, p, pos, R = int(g["t2"][k]), g["p2"][k], g["pos2"][k], g["R2"][k]
        gh = mk[t](p)
        L.dGeomSetPosition(gh, *pos)
        L.dGeomSetRotation(gh, (C.c_float * 12)(*[R[0], R[1], R[2], 0, R[3], R[4], R[5], 0, R[6], R[7], R[8], 0]))
        ref_n, ref = int(g["nc"][k]), g["out"][k]
        for order, sgn in (((hg, gh), 1.0), ((gh, hg), -1.0)):
            out = (ContactGeom * 16)()
            nc = L.dCollide(order[0], order[1], int(g["flags"][k]), out, C.sizeof(ContactGeom))
            if nc != ref_n:
                count_mism.append((k, nc, ref_n))
                continue
            for c in range(nc):
                got = np.array(list(out[c].pos[:3]) + [sgn * x for x in out[c].normal[:3]] + [out[c].depth])
                worst = max(worst, np.abs(got - ref[c, :7]).max() / scale)
        L.dGeomDestroy(gh)
    L.dGeomDestroy(hg)
    L.dGeomHeightfieldDataDestroy(hd)
    assert not count_mism, count_mism[:10]
    assert worst < 1e-4, worst


def test_hinge_motor_velocity_after_one_dworldstep():
    """The reference's test_Hinge_dParamVel (tests/joints/hinge.cpp:898-922):
    two unit bodies at the origin on a hinge along x, motor FMax = inf,
    Vel = 100; after one dWorldStep(0.001) the relative angular velocity is
    (100, 0, 0) within the reference's dSINGLE tolerance (1e-2 x 100)."""
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dWorldCreate.restype = v
    L.dBodyCreate.restype = v; L.dBodyCreate.argtypes = [v]
    L.dBodySetPosition.argtypes = [v, f, f, f]
    L.dJointCreateHinge.restype = v; L.dJointCreateHinge.argtypes = [v, v]
    L.dJointAttach.argtypes = [v, v, v]
    L.dJointSetHingeAnchor.argtypes = [v, f, f, f]
    L.dJointSetHingeParam.argtypes = [v, i, f]
    L.dWorldStep.restype = i; L.dWorldStep.argtypes = [v, f]
    L.dBodyGetAngularVel.restype = C.POINTER(f); L.dBodyGetAngularVel.argtypes = [v]
    L.dWorldDestroy.argtypes = [v]
    dParamVel, dParamFMax = 2, 3     # include/ode/common.h: dParamLoStop = 0, dParamHiStop, dParamVel, dParamFMax
    w = L.dWorldCreate()
    b1, b2 = L.dBodyCreate(w), L.dBodyCreate(w)
    L.dBodySetPosition(b1, 0, 0, 0)
    L.dBodySetPosition(b2, 0, 0, 0)
    j = L.dJointCreateHinge(w, None)
    L.dJointAttach(j, b1, b2)
    L.dJointSetHingeAnchor(j, 0, 0, 0)
    L.dJointSetHingeParam(j, dParamFMax, float("inf"))
    L.dJointSetHingeParam(j, dParamVel, 100.0)
    assert L.dWorldStep(w, 0.001) == 1
    v1, v2 = L.dBodyGetAngularVel(b1), L.dBodyGetAngularVel(b2)
    rvel = np.array([v1[k] - v2[k] for k in range(3)])
    assert np.abs(rvel - np.array([100.0, 0.0, 0.0])).max() < 1.0, rvel
    L.dWorldDestroy(w)


def test_heightfield_ray_outside_bounds():
    """The reference's test_collision_heightfield_ray_fail
    (tests/collision.cpp:103-131): a 4 x 4 byte heightfield with bounds, a
    ray of length 20 outside the field pointing along -y; dCollide must not
    fail and, as the reference built here returns, finds no contact."""
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dGeomHeightfieldDataCreate.restype = v
    L.dGeomHeightfieldDataBuildByte.argtypes = [v, C.c_char_p, i, f, f, i, i, f, f, f, i]
    L.dGeomHeightfieldDataSetBounds.argtypes = [v, f, f]
    L.dCreateHeightfield.restype = v; L.dCreateHeightfield.argtypes = [v, v, i]
    L.dCreateRay.restype = v; L.dCreateRay.argtypes = [v, f]
    L.dGeomRaySet.argtypes = [v, f, f, f, f, f, f]
    L.dCollide.restype = i; L.dCollide.argtypes = [v, v, i, v, i]
    L.dGeomDestroy.argtypes = [v]
    L.dGeomHeightfieldDataDestroy.argtypes = [v]
    hd = L.dGeomHeightfieldDataCreate()
    L.dGeomHeightfieldDataBuildByte(hd, b"1234567890123456", 0, 4, 4, 4, 4, 1, 0, 0, 0)
    L.dGeomHeightfieldDataSetBounds(hd, float(ord("0")), float(ord("9")))
    h = L.dCreateHeightfield(None, hd, 1)
    r = L.dCreateRay(None, 20)
    L.dGeomRaySet(r, 5, 10, 1, 0, -1, 0)
    out = (ContactGeom * 10)()
    assert L.dCollide(r, h, 10, out, C.sizeof(ContactGeom)) == 0
    assert L.dCollide(h, r, 10, out, C.sizeof(ContactGeom)) == 0
    L.dGeomDestroy(r)
    L.dGeomDestroy(h)
    L.dGeomHeightfieldDataDestroy(hd)


@pytest.mark.parametrize("kind,tol", [("Ball", 1e-4), ("Hinge", 1e-6), ("Hinge2", 1e-4)])
def test_reference_joint_fixtures_with_dworldstep(kind, tol):
    """The reference's set/get consistency fixtures that step the world
    (tests/joints/ball.cpp:41-151, hinge.cpp:786-895, hinge2.cpp:46-160): two
    identical body pairs at (-1,-2,-3) and (11,22,33), rotated 27 degrees
    about fixed axes, joined by a joint; the second joint's anchor (and axes)
    are read back and set again; after four dWorldStep(0.5) both pairs agree
    within the reference's tolerance."""
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    V4 = f * 4
    L.dWorldCreate.restype = v
    L.dWorldSetGravity.argtypes = [v, f, f, f]
    L.dBodyCreate.restype = v; L.dBodyCreate.argtypes = [v]
    L.dBodySetPosition.argtypes = [v, f, f, f]
    L.dBodySetRotation.argtypes = [v, C.POINTER(f)]
    L.dRFromAxisAndAngle.argtypes = [C.POINTER(f), f, f, f, f]
    L.dNormalize3.argtypes = [C.POINTER(f)]
    create = getattr(L, f"dJointCreate{kind}")
    create.restype = v; create.argtypes = [v, v]
    L.dJointAttach.argtypes = [v, v, v]
    L.dWorldStep.restype = i; L.dWorldStep.argtypes = [v, f]
    L.dBodyGetQuaternion.restype = C.POINTER(f); L.dBodyGetQuaternion.argtypes = [v]
    L.dBodyGetPosition.restype = C.POINTER(f); L.dBodyGetPosition.argtypes = [v]
    L.dWorldDestroy.argtypes = [v]
    w = L.dWorldCreate()
    L.dWorldSetGravity(w, 0, 0, 0)
    bodies, joints = [], []
    for _ in range(2):
        pair = []
        for pos, ax in (((-1, -2, -3), (0.53, -0.71, 0.43)), ((11, 22, 33), (1.2, 0.87, -0.33))):
            b = L.dBodyCreate(w)
            L.dBodySetPosition(b, *pos)
            a = V4(*ax, 0.0)
            L.dNormalize3(a)
            R = (f * 12)()
            L.dRFromAxisAndAngle(R, a[0], a[1], a[2], 0.47123)
            L.dBodySetRotation(b, R)
            pair.append(b)
        j = create(w, None)
        L.dJointAttach(j, pair[0], pair[1])
        bodies.append(pair)
        joints.append(j)

    def roundtrip(get, set_):
        g = getattr(L, get); g.argtypes = [v, C.POINTER(f)]
        s = getattr(L, set_); s.argtypes = [v, f, f, f]
        out = V4()
        g(joints[1], out)
        s(joints[1], out[0], out[1], out[2])

    if kind == "Hinge":
        roundtrip("dJointGetHingeAxis", "dJointSetHingeAxis")
    roundtrip(f"dJointGet{kind}Anchor", f"dJointSet{kind}Anchor")
    if kind == "Hinge2":
        roundtrip("dJointGetHinge2Axis1", "dJointSetHinge2Axis1")
        roundtrip("dJointGetHinge2Axis2", "dJointSetHinge2Axis2")
    for _ in range(4):
        assert L.dWorldStep(w, 0.5) == 1
    for b in range(2):
        qa, qb = L.dBodyGetQuaternion(bodies[0][b]), L.dBodyGetQuaternion(bodies[1][b])
        pa, pb = L.dBodyGetPosition(bodies[0][b]), L.dBodyGetPosition(bodies[1][b])
        assert max(abs(qa[k] - qb[k]) for k in range(4)) < tol, (kind, b)
        assert max(abs(pa[k] - pb[k]) for k in range(3)) < tol, (kind, b)
    L.dWorldDestroy(w)


@pytest.mark.parametrize("stepper", ["dWorldQuickStep", "dWorldStep"])
def test_disabled_joint_takes_no_part(stepper):
    """dJointDisable / dJointEnable / dJointIsEnabled (ode/src/ode.cpp:1401-1417):
    a disabled joint neither joins islands nor adds rows (util.cpp:435-510),
    so a pendulum chain carrying a disabled extra ball joint steps
    bit-identically to the same chain without it; once re-enabled it acts."""
    from odegpu._lib import lib
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dWorldCreate.restype = v
    L.dWorldSetGravity.argtypes = [v, f, f, f]
    L.dBodyCreate.restype = v; L.dBodyCreate.argtypes = [v]
    L.dBodySetPosition.argtypes = [v, f, f, f]
    L.dBodyGetPosition.restype = C.POINTER(f); L.dBodyGetPosition.argtypes = [v]
    L.dJointCreateHinge.restype = v; L.dJointCreateHinge.argtypes = [v, v]
    L.dJointCreateBall.restype = v; L.dJointCreateBall.argtypes = [v, v]
    L.dJointAttach.argtypes = [v, v, v]
    L.dJointSetHingeAnchor.argtypes = [v, f, f, f]
    L.dJointSetHingeAxis.argtypes = [v, f, f, f]
    L.dJointSetBallAnchor.argtypes = [v, f, f, f]
    L.dJointDisable.argtypes = L.dJointEnable.argtypes = L.dJointIsEnabled.argtypes = [v]
    step = getattr(L, stepper)
    step.restype = i; step.argtypes = [v, f]
    L.dWorldDestroy.argtypes = [v]

    def chain(extra):
        w = L.dWorldCreate()
        L.dWorldSetGravity(w, 0, 0, -9.81)
        bs = [L.dBodyCreate(w) for _ in range(3)]
        for k, b in enumerate(bs):
            L.dBodySetPosition(b, 0.5 * (k + 1), 0.1 * k, 2.0)
        prev = None
        for k, b in enumerate(bs):
            j = L.dJointCreateHinge(w, None)
            L.dJointAttach(j, b, prev)
            L.dJointSetHingeAnchor(j, 0.5 * k + 0.25, 0.05 * k, 2.0)
            L.dJointSetHingeAxis(j, 0, 1, 0.2 * k)
            prev = b
        jx = None
        if extra:
            jx = L.dJointCreateBall(w, None)
            L.dJointAttach(jx, bs[0], bs[2])
            L.dJointSetBallAnchor(jx, 1.0, 0.0, 2.0)
            L.dJointDisable(jx)
            assert L.dJointIsEnabled(jx) == 0
        return w, bs, jx

    def pos(bs):
        return np.array([[L.dBodyGetPosition(b)[k] for k in range(3)] for b in bs])

    L.dRandSetSeed.argtypes = [C.c_ulong]

    def step_both(k):
        # QuickStep's row shuffle draws from ODE's one global RNG: both
        # worlds start each step from the same seed
        L.dRandSetSeed(1000 + k)
        assert step(wa, 0.01) == 1
        L.dRandSetSeed(1000 + k)
        assert step(wb, 0.01) == 1

    wa, ba, jx = chain(True)
    wb, bb, _ = chain(False)
    for k in range(20):
        step_both(k)
    assert np.array_equal(pos(ba), pos(bb))
    L.dJointEnable(jx)
    assert L.dJointIsEnabled(jx) == 1
    for k in range(5):
        step_both(20 + k)
    assert not np.array_equal(pos(ba), pos(bb))
    L.dWorldDestroy(wa)
    L.dWorldDestroy(wb)


def test_worlds_above_64_bodies_step_through_large_pipeline():
    """dWorldQuickStep on a world above the on-chip kernel's 64 bodies steps
    it through the large-world pipeline with the program's own contacts and
    body joint lists (ode.cpp:1807-1824 puts no cap on the world's size).
    An 80-box drop (box_drop_demo.c) and an 80-link hinge chain with per-step
    hinge torques touching the plane (scene_player.c), each against the
    batched path stepping the same single world through the same pipeline:
    contacts come from the same collider in the same pair order, so the
    states agree to FP32 rounding (1e-4 m, 1e-2 m/s). dWorldStep is not
    available for such a world: the call returns 0 and the program stops."""
    import subprocess
    from odegpu.batch import Batch
    drop = S.box_drop(seed=1, n_boxes=80)
    chain = S.hinge_chains(n_worlds=1, links=80, seed=11, steps=40, plane_z=-2.0)
    with tempfile.TemporaryDirectory() as d:
        inp = os.path.join(d, "in.txt")
        for sc, steps, exe, write in (
                (drop, 70, U.build_gpu_demo(os.path.join(d, "demo")), U.scene_input),
                (chain, 40, U.build_gpu_demo(os.path.join(d, "player"), src=U.PLAYER),
                 lambda s, n, p: U.player_input(s, 0, n, p))):
            assert sc.nb_total > 64
            B = Batch(sc)
            B.step(steps)
            bt = B.state()
            nc = int(B.counts()[0][0])
            assert (B.status() == 0).all(), B.status()
            B.close()
            write(sc, steps, inp)
            st = U.run_demo(exe, inp)
            assert nc > 0
            assert np.abs(st[:, :3] - bt[:, :3]).max() < 1e-4
            assert np.abs(st[:, 7:] - bt[:, 7:]).max() < 1e-2
        U.player_input(chain, 0, 2, inp)
        with pytest.raises(subprocess.CalledProcessError):
            U.run_demo(exe, inp, "exact")


def test_joint_feedback_above_64_bodies():
    """dJointSetFeedback on an 80-link ball chain (above the on-chip kernel's
    64 bodies, so dWorldQuickStep steps it through the large-world pipeline),
    swinging from the environment: after each of five steps every joint's
    feedback equals that of the batched path stepping the same world through
    the same pipeline (which test_gpu_large_world.py checks against the
    warp-per-world path), f2 = t2 = 0 for the joint to the environment, and
    the top joint pulls the chain up."""
    from odegpu._lib import lib
    from odegpu.batch import Batch
    L = lib()
    f, v, i = C.c_float, C.c_void_p, C.c_int
    L.dWorldCreate.restype = v
    L.dWorldSetGravity.argtypes = [v, f, f, f]
    L.dWorldSetCFM.argtypes = [v, f]
    L.dBodyCreate.restype = v; L.dBodyCreate.argtypes = [v]
    L.dBodySetPosition.argtypes = [v, f, f, f]
    L.dBodySetLinearVel.argtypes = [v, f, f, f]
    L.dBodyGetPosition.restype = C.POINTER(f); L.dBodyGetPosition.argtypes = [v]
    L.dMassSetSphereTotal.argtypes = [C.POINTER(Mass), f, f]
    L.dBodySetMass.argtypes = [v, C.POINTER(Mass)]
    L.dJointCreateBall.restype = v; L.dJointCreateBall.argtypes = [v, v]
    L.dJointAttach.argtypes = [v, v, v]
    L.dJointSetBallAnchor.argtypes = [v, f, f, f]
    L.dJointSetFeedback.argtypes = [v, C.POINTER(JointFeedback)]
    L.dWorldQuickStep.restype = i; L.dWorldQuickStep.argtypes = [v, f]
    L.dRandSetSeed.argtypes = [C.c_ulong]
    L.dWorldDestroy.argtypes = [v]
    n, m, r = 80, 2.0, 0.1
    vx = [0.3 * np.sin(0.7 * k) for k in range(n)]
    w = L.dWorldCreate()
    L.dWorldSetGravity(w, 0.0, 0.0, -9.81)
    L.dWorldSetCFM(w, 1e-5)
    bodies, fbs = [], []
    for k in range(n):
        b = L.dBodyCreate(w)
        L.dBodySetPosition(b, 0.0, 0.0, -0.5 - k)
        L.dBodySetLinearVel(b, vx[k], 0.0, 0.0)
        M = Mass()
        L.dMassSetSphereTotal(C.byref(M), m, r)
        L.dBodySetMass(b, C.byref(M))
        bodies.append(b)
    for k in range(n):
        j = L.dJointCreateBall(w, None)
        L.dJointAttach(j, bodies[k], bodies[k - 1] if k > 0 else None)
        L.dJointSetBallAnchor(j, 0.0, 0.0, -float(k))
        fb = JointFeedback()
        L.dJointSetFeedback(j, C.byref(fb))
        fbs.append(fb)
    # the same world for the batched path
    sb = S.SceneBuilder()
    S._std_surface(sb)
    ws = sb.new_world(cfm=1e-5, seed=0)
    for k in range(n):
        mm, I = S.sphere_mass_total(m, r)
        sb.add_body(ws, (0.0, 0.0, -0.5 - k), mm, I, lvel=(vx[k], 0.0, 0.0))
    for k in range(n):
        sb.add_joint(ws, S.JOINT_BALL, k, k - 1 if k > 0 else -1, anchor=(0.0, 0.0, -float(k)),
                     param=(0.2, 1e-5))
    B = Batch(sb.build())
    B.set_feedback(True)
    L.dRandSetSeed(0)
    for s in range(5):
        assert L.dWorldQuickStep(w, 0.01) == 1
        B.step(1)
        ref = B.feedback()
        got = np.array([list(fb.f1[:3]) + list(fb.t1[:3]) + list(fb.f2[:3]) + list(fb.t2[:3]) for fb in fbs])
        scale = max(1.0, float(np.abs(ref).max()))
        assert np.abs(got - ref).max() < 1e-4 * scale, (s, float(np.abs(got - ref).max()), scale)
        assert np.all(got[0, 6:] == 0.0)
        pos = np.array([L.dBodyGetPosition(b)[k] for b in bodies for k in range(3)]).reshape(n, 3)
        assert np.abs(pos - B.state()[:, 0:3]).max() < 1e-5
    assert got[0, 2] > 0.0
    assert (B.status() == 0).all()
    B.close()
    L.dWorldDestroy(w)
