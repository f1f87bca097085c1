"""Hand-written adjoint of the batched step against FP64 central differences
of the CPU oracle (no gradients exist in the reference; the oracle restates
its dWorldQuickStep in FP64, so d(loss)/d(input) is taken by re-running it
with the input moved by +-eps, the RNG seeds identical in both runs).

Tolerance: the gradient vector of each case, against the finite-difference
one, within 1e-3 relative (2-norm of the difference over 2-norm of the
reference). The GPU runs in FP32, the reference in FP64. The difference step
is 1e-4 for the hinge chains; the sliding-box contact case is stiff (contact
rhs ~ erp/h^2 times depth), and there a 1e-4 step itself is off by ~5e-3, so
it uses 1e-6 (FP64 rounding is ~1e-10 at that step)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from odegpu import scene as S

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

EPS = 1e-4
TOL = 1e-3


def _oracle_final(sc, w, n, x0=None):
    if x0 is None:
        return O.run_world(O.oracle().oracle_run_world, sc, w, n)["state"][n]
    return O.run_world_from(sc, w, n, x0)


def _fd(sc, w, n, loss, poke, x0, eps=EPS):
    """Central difference of loss(final state of world w) for the input that
    poke(sign * eps) moves (poke(0) puts it back); x0 is the world's initial
    state array the pokes may edit."""
    poke(eps)
    lp = loss(_oracle_final(sc, w, n, x0))
    poke(-eps)
    lm = loss(_oracle_final(sc, w, n, x0))
    poke(0.0)
    return (lp - lm) / (2 * eps)


def _gpu_grads(sc, n, coef, ckpt=10, x_init=None):
    """GPU rollout of n steps with loss sum(coef * final) (coef [nb, 13]);
    returns (grad init state [nb,13], grad joint torques [S,nj,2] or None, batch,
    final state, initial state)."""
    from odegpu.batch import Batch
    from odegpu.adjoint import rollout
    B = Batch(sc)
    if x_init is not None:
        B.set_state(x_init)
    x0_np = B.state()
    x0 = torch.tensor(x0_np, dtype=torch.float32, device="cuda", requires_grad=True)
    jt = None
    if sc.n_ctrl_steps > 0 and getattr(sc, "joint_torque", None) is not None:
        jt = torch.tensor(sc.joint_torque, dtype=torch.float32, device="cuda", requires_grad=True)
    final = rollout(B, n, x0, jt, None, ckpt_every=ckpt)
    c = torch.tensor(coef, dtype=torch.float32, device="cuda")
    (final * c).sum().backward()
    gj = jt.grad.cpu().numpy() if jt is not None else None
    return x0.grad.cpu().numpy(), gj, B, final.detach().cpu().numpy(), x0_np


def _rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)


def _check_case(sc, n, coef, n_vel=12, n_pos=6, n_tq=12, seed=0, q_dirs=2, eps=EPS, x_init=None, tq_col=0,
                tq_joints=None):
    rng = np.random.default_rng(seed)
    g_state, g_jt, B, _, g0 = _gpu_grads(sc, n, coef, x_init=x_init)
    status = B.adjoint_status()
    assert (status == 0).all(), status
    fd, gpu, names = [], [], []
    for w in range(sc.n_worlds):
        b0, b1 = sc.world_bodies(w)
        cw = coef[b0:b1]
        # the oracle starts from the FP32 state the GPU starts from
        x0 = np.asarray(g0[b0:b1], dtype=np.float64).copy()

        def loss(fin, cw=cw):
            return float(np.sum(cw * fin))

        def state_poke(b, k, x0=x0, b0=b0):
            v0 = x0[b - b0, k]

            def poke(e):
                x0[b - b0, k] = v0 + e
            return poke

        for _ in range(n_vel):
            b = int(rng.integers(b0, b1))
            k = 7 + int(rng.integers(0, 6))
            fd.append(_fd(sc, w, n, loss, state_poke(b, k), x0, eps)); gpu.append(g_state[b, k])
            names.append(f"v{b},{k}")
        for _ in range(n_pos):
            b = int(rng.integers(b0, b1))
            k = int(rng.integers(0, 3))
            fd.append(_fd(sc, w, n, loss, state_poke(b, k), x0, eps)); gpu.append(g_state[b, k])
            names.append(f"x{b},{k}")
        for _ in range(q_dirs):
            b = int(rng.integers(b0, b1))
            k = 3 + int(rng.integers(0, 4))
            fd.append(_fd(sc, w, n, loss, state_poke(b, k), x0, eps)); gpu.append(g_state[b, k])
            names.append(f"q{b},{k}")
        if g_jt is not None:
            j0, j1 = sc.world_joints(w)
            for _ in range(n_tq):
                s = int(rng.integers(0, min(n, sc.n_ctrl_steps)))
                j = j0 + int(rng.choice(tq_joints)) if tq_joints is not None else int(rng.integers(j0, j1))
                v0 = sc.joint_torque[s, j, tq_col]

                def poke(e, s=s, j=j, v0=v0):
                    sc.joint_torque[s, j, tq_col] = v0 + e
                fd.append(_fd(sc, w, n, loss, poke, x0, eps)); gpu.append(g_jt[s, j, tq_col])
                names.append(f"t{s},{j}")
    B.close()
    err = _rel(gpu, fd)
    worst = np.argsort(-np.abs(np.array(gpu) - np.array(fd)))[:5]
    detail = [(names[i], gpu[i], fd[i]) for i in worst]
    return err, detail


def _coef(sc, seed, cols=range(13)):
    rng = np.random.default_rng(seed)
    c = np.zeros((sc.body_off[-1], 13))
    for k in cols:
        c[:, k] = rng.standard_normal(sc.body_off[-1])
    c[:, 3:7] = 0.0     # quaternion outputs: checked through the state they drive
    return c


def test_adjoint_one_step_hinge_chain():
    sc = S.hinge_chains(n_worlds=2, steps=4, plane_z=-100.0)
    err, detail = _check_case(sc, 1, _coef(sc, 1), seed=1)
    assert err < TOL, (err, detail)


def test_adjoint_chain_rollout_100_steps():
    """Differentiable-batch workload (8-link hinge chains, per-step torques,
    100 steps, checkpoints every 10) with the plane out of reach, so the
    trajectory does not switch; loss = squared distance of the end link to a
    seeded target; d/d(initial velocities) and d/d(torques)."""
    n = 100
    sc = S.hinge_chains(n_worlds=2, steps=n, plane_z=-100.0)
    rng = np.random.default_rng(7)
    fin = np.concatenate([_oracle_final(sc, w, n) for w in range(sc.n_worlds)])  # targets only
    coef = np.zeros((sc.body_off[-1], 13))
    # loss = sum over worlds |p_end - target|^2 is quadratic; its gradient at
    # the final state is linear in the final state, so check d/d(input) of
    # the linearisation sum(2 (p_end - target) . p_end) (same gradient).
    for w in range(sc.n_worlds):
        b_end = sc.body_off[w + 1] - 1
        target = fin[b_end, 0:3] + rng.uniform(-0.5, 0.5, 3)
        coef[b_end, 0:3] = 2 * (fin[b_end, 0:3] - target)
    err, detail = _check_case(sc, n, coef, n_vel=16, n_pos=0, n_tq=16, seed=2, q_dirs=0)
    assert err < TOL, (err, detail)


def test_adjoint_sliding_box_contacts():
    """A box sliding on a plane: four persistent contacts, friction rows held at
    +-mu * lambda_normal (the clamp passes the derivative to the normal row)."""
    b = S.SceneBuilder()
    s = S._std_surface(b, 0.5)
    w = b.new_world(cfm=1e-5, seed=5)
    b.add_geom(w, S.GEOM_PLANE, -1, (0, 0, 1, 0), s)
    m, I = S.box_mass(1000.0, 0.6, 0.4, 0.3)
    bi = b.add_body(w, (0.0, 0.0, 0.149), m, I, lvel=(1.5, 0.4, 0.0), avel=(0.0, 0.0, 0.3))
    b.add_geom(w, S.GEOM_BOX, bi, (0.6, 0.4, 0.3), s)
    sc = b.build()
    coef = _coef(sc, 3, cols=[0, 1, 7, 8, 12])
    err, detail = _check_case(sc, 10, coef, n_vel=6, n_pos=3, n_tq=0, seed=3, q_dirs=1, eps=1e-6)
    assert err < TOL, (err, detail)


def test_adjoint_checkpoint_interval_invariant():
    sc = S.hinge_chains(n_worlds=3, steps=30, plane_z=-100.0)
    coef = _coef(sc, 4)
    g1, j1, B1, f1, _ = _gpu_grads(sc, 30, coef, ckpt=1)
    B1.close()
    g2, j2, B2, f2, _ = _gpu_grads(sc, 30, coef, ckpt=7)
    B2.close()
    g3, j3, B3, f3, _ = _gpu_grads(sc, 30, coef, ckpt=30)
    B3.close()
    assert np.array_equal(f1, f2) and np.array_equal(f1, f3)
    assert np.array_equal(g1, g2) and np.array_equal(g1, g3)
    assert np.array_equal(j1, j2) and np.array_equal(j1, j3)


def test_adjoint_vehicles_on_heightfield():
    """Vehicle batch from a settled state (oracle step 40): four steps with
    hinge2 suspension, steering held by per-step stops (limit rows whose rhs
    follows the hinge2 angle) and heightfield contacts of wheels and chassis
    (plane-pass and vertex-pass). d/d(initial velocities) and d/d(rear-wheel
    drive torques) of a linear loss on the chassis state; the contact sets do
    not change over the four steps, so central differences (step 1e-6) are
    smooth."""
    from gpu_helpers import oracle_states, stacked_state
    sc = S.vehicles(n_worlds=4, steps=60, hf_samples=64)
    runs = oracle_states(sc, 41)
    x_init = stacked_state(runs, 40)
    coef = np.zeros((sc.body_off[-1], 13))
    rng = np.random.default_rng(8)
    for w in range(sc.n_worlds):
        b0 = sc.body_off[w]
        coef[b0, 0:3] = rng.standard_normal(3)
        coef[b0, 7:10] = rng.standard_normal(3)
    err, detail = _check_case(sc, 4, coef, n_vel=10, n_pos=0, n_tq=6, seed=9, q_dirs=0, eps=1e-6,
                              x_init=x_init, tq_col=1, tq_joints=[2, 3])
    assert err < TOL, (err, detail)


def test_adjoint_hinge_limit_rows():
    """Hinge chains with stops at [0.1, 0.6] rad; a hinge's angle is 0 at the
    pose it is created in, so every joint starts 0.1 rad below its low stop,
    at a limit: the limit row's rhs -fps stop_erp (angle - stop) follows the hinge
    angle (getHingeAngle, ode/src/joints/joint.cpp:381-450), differentiated
    through both bodies' quaternions. Three steps with the plane out of
    reach; every world must be fully modelled."""
    sc = S.hinge_chains(n_worlds=3, steps=6, plane_z=-100.0)
    sc.joint_param[:, 0] = 0.1       # lostop
    sc.joint_param[:, 1] = 0.6       # histop
    # joints starting beyond a stop: their sixth row is a limit row
    for w in range(sc.n_worlds):
        j0, j1 = sc.world_joints(w)
        assert O.tap_step(sc, w, 0)["total_rows"] > 5 * (j1 - j0)
    err, detail = _check_case(sc, 3, _coef(sc, 11), n_vel=12, n_pos=4, n_tq=8, seed=11, q_dirs=2)
    assert err < TOL, (err, detail)


def _quat_mul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return (w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
            w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2)


def _body_body_scene(top_tilt, top_yaw, spheres=True, top_box=True, lower_q=(1.0, 0.0, 0.0, 0.0)):
    """A 0.4 x 0.3 x 0.2 m box turned top_yaw rad about z and tipped
    top_tilt rad about its x axis, resting on one edge 1 mm deep in a
    0.9 x 0.9 x 0.3 m box that sits on the plane z = 0 (the lower box's top
    face against the tipped box's bottom face: two points; the yaw keeps the
    resting edge off the lower box's edge directions, so no edge axis ties
    with the face axis), and, with spheres, a 0.15 m sphere on the lower box
    and a 0.1 m sphere on that sphere (sphere-box and sphere-sphere)."""
    b = S.SceneBuilder()
    s = S._std_surface(b, 0.5)
    w = b.new_world(cfm=1e-5, seed=9)
    b.add_geom(w, S.GEOM_PLANE, -1, (0, 0, 1, 0), s)
    m0, I0 = S.box_mass(500.0, 0.9, 0.9, 0.3)
    b0 = b.add_body(w, (0.0, 0.0, 0.1495), m0, I0, q=lower_q, lvel=(0.05, 0.0, 0.0))
    b.add_geom(w, S.GEOM_BOX, b0, (0.9, 0.9, 0.3), s)
    if top_box:
        m1, I1 = S.box_mass(300.0, 0.4, 0.3, 0.2)
        qz = (np.cos(top_yaw / 2), 0.0, 0.0, np.sin(top_yaw / 2))
        qx = (np.cos(top_tilt / 2), np.sin(top_tilt / 2), 0.0, 0.0)
        h = 0.5 * (0.3 * np.sin(top_tilt) + 0.2 * np.cos(top_tilt))
        b1 = b.add_body(w, (0.1, 0.05, 0.299 + h), m1, I1, q=_quat_mul(qz, qx), lvel=(0.1, -0.05, 0.0),
                        avel=(0.2, 0.0, 0.1))
        b.add_geom(w, S.GEOM_BOX, b1, (0.4, 0.3, 0.2), s)
    if spheres:
        m2, I2 = S.sphere_mass(400.0, 0.15)
        b2 = b.add_body(w, (-0.25, -0.25, 0.449), m2, I2, lvel=(0.0, 0.2, 0.0))
        b.add_geom(w, S.GEOM_SPHERE, b2, (0.15,), s)
        m3, I3 = S.sphere_mass(400.0, 0.1)
        b3 = b.add_body(w, (-0.25, -0.24, 0.6985), m3, I3, avel=(0.5, 0.0, 0.0))
        b.add_geom(w, S.GEOM_SPHERE, b3, (0.1,), s)
    return b.build()


def test_adjoint_sphere_body_contacts():
    """Sphere-box and sphere-sphere contacts between dynamic bodies (a sphere
    on a box on the plane, a sphere on that sphere): three steps against
    FP64 central differences (step 1e-6)."""
    sc = _body_body_scene(0.0, 0.0, top_box=False)
    coef = _coef(sc, 14, cols=[0, 1, 2, 7, 8, 9, 10, 11, 12])
    err, detail = _check_case(sc, 3, coef, n_vel=12, n_pos=6, n_tq=0, seed=14, q_dirs=2, eps=1e-6)
    assert err < TOL, (err, detail)


def test_adjoint_body_body_contacts():
    """Contacts between two dynamic bodies (box-box, sphere-box and
    sphere-sphere): the rows
    are differentiated with respect to the contact point, normal and depth
    and both bodies, the collider's geometry by central differences of the
    FP32 collider. Two steps, FP64 central differences of the oracle (step
    1e-6: stiff contacts), every world fully modelled."""
    # the lower box starts tipped by a few milliradians (no orientation is
    # exactly axis aligned, so no collider decision - which vertex of a box on
    # the plane comes first, which of two parallel faces is the reference -
    # hangs on the sign of an exact zero that a difference step would flip);
    # the check runs steps 1-2, over which the contact sets do not change
    sc = _body_body_scene(0.3, 0.4, lower_q=_quat_mul((np.cos(0.002), np.sin(0.002), 0.0, 0.0),
                                                      (np.cos(0.003), 0.0, np.sin(0.003), 0.0)))
    from gpu_helpers import oracle_states, stacked_state
    runs = oracle_states(sc, 3)
    x_init = stacked_state(runs, 1)
    gb = sc.geom_body
    for k in (1, 2):
        c = runs[0]["contacts"][k][: runs[0]["ncontacts"][k]]
        pairs = [(int(gb[int(x[7])]), int(gb[int(x[8])])) for x in c]
        assert pairs.count((0, 1)) == 2 and (0, 2) in pairs and (2, 3) in pairs, (k, pairs)
    coef = _coef(sc, 12, cols=[0, 1, 2, 7, 8, 9, 10, 11, 12])
    err, detail = _check_case(sc, 2, coef, n_vel=12, n_pos=6, n_tq=0, seed=12, q_dirs=2, eps=1e-6, x_init=x_init)
    assert err < TOL, (err, detail)


def _link_contact_windows(sc, n_steps, max_windows):
    """(world, step) of the hinge-chain workload where two links touch."""
    out = []
    gb = sc.geom_body
    for w in range(sc.n_worlds):
        r = O.run_world(O.oracle().oracle_run_world, sc, w, n_steps, max_rec=64)
        g0 = sc.geom_off[w]
        for k in range(n_steps):
            c = r["contacts"][k][: r["ncontacts"][k]]
            if any(gb[g0 + int(x[7])] >= 0 and gb[g0 + int(x[8])] >= 0 for x in c):
                out.append((w, k, r["state"][k]))
                break
        if len(out) >= max_windows:
            break
    return out


def test_adjoint_hinge_chains_configured_plane_link_contacts():
    """The differentiable-batch workload as configured (plane at z = -2):
    links of a chain touch each other (box-box contacts between two dynamic
    bodies). Windows of two steps starting where such a contact is present,
    from the oracle's state there: d/d(initial velocities) and d/d(torques)
    against FP64 central differences, every world fully modelled."""
    sc = S.hinge_chains(n_worlds=64, steps=100)
    wins = _link_contact_windows(sc, 100, 4)
    assert len(wins) >= 2
    from odegpu.shard import slice_scene
    for w, k, state in wins:
        sub = slice_scene(sc, w, w + 1)
        err, detail = _check_case(sub, 2, _coef(sub, 13 + w), n_vel=10, n_pos=0, n_tq=6, seed=13 + w, q_dirs=0,
                                  eps=1e-6, x_init=state)
        assert err < TOL, (w, k, err, detail)
