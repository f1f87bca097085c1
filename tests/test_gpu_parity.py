"""Parity of the CUDA path against the FP64 oracle (which is itself pinned
bit-for-bit to the reference ODE 0.12 by test_oracle.py).

Integer outputs (contact counts, island and row counts, row order, findex,
lo/hi, RNG state) must be bit-exact. FP32 outputs are compared to the FP64
oracle with the tolerances written in each test."""
import numpy as np
import pytest

from odegpu import scene as S
from gpu_helpers import oracle_states, stacked_state, seeds_before, state_err
import oracle_lib as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_cls():
    from odegpu.batch import Batch
    return Batch


# one-step tolerances (state after one step from an identical FP64->FP32 start)
POS_ATOL = 2e-5     # m
Q_ATOL = 2e-5
VEL_ATOL = 2e-3     # m/s, rad/s: SOR in FP32 vs FP64 after 20 iterations


def _scenes():
    return {
        "box_drop": S.box_drop(seed=0),
        "batched": S.batched_worlds(n_worlds=48, seed=11),
        "hinge": S.hinge_chains(n_worlds=8, steps=40),
        "tower": S.box_tower(n_worlds=6, yaw=0.0, spacing=0.0),
        "capsule": S.capsule_mix(seed=6),
        "capsule_pile": S.capsule_pile(),
        # slider (to the environment, reversed, body-body with motor / limits /
        # servo stops), universal, fixed (body-body and reversed) joints with
        # ball / fixed erp carried along an island
        "mechanisms": S.mechanisms(n_worlds=16, steps=40),
        # cylinders on a plane and on a heightfield (cylinder-sphere / -box /
        # -plane, heightfield-cylinder)
        "cylinder_pile": S.cylinder_pile(n_worlds=4),
        # aligned equal boxes: exact SAT ties between parallel faces, which FP32
        # and FP64 break differently (ODE's own FP32 build drifts mm here)
        "stack": S.box_stack(n_worlds=4, height=5),
    }


@pytest.mark.parametrize("fused", [False, True], ids=["split", "fused"])
@pytest.mark.parametrize("name", ["box_drop", "batched", "hinge", "tower", "capsule", "capsule_pile",
                                  "mechanisms", "cylinder_pile"])
def test_one_step_from_oracle_state(batch_cls, name, fused):
    """Both step launches: the collide, setup and solve kernels, and the fused
    step kernel that runs the three phases of a world on one warp."""
    sc = _scenes()[name]
    n = 40
    runs = oracle_states(sc, n)
    B = batch_cls(sc)
    B.set_step_kernels(fused)
    worst = dict(pos=0, q=0, lvel=0, avel=0)
    nc_mismatch = 0
    for k in (0, 5, 15, 25, 39):
        B.set_state(stacked_state(runs, k))
        B.set_seeds(seeds_before(sc, runs, k))
        B.set_step_index(k)
        B.step(1)
        g = B.state()
        nc, nr, ni = B.counts()
        ref_nc = np.array([r["ncontacts"][k] for r in runs])
        nc_mismatch += int(np.sum(nc != ref_nc))
        e = state_err(g, stacked_state(runs, k + 1))
        for key in worst:
            worst[key] = max(worst[key], e[key])
        if np.array_equal(nc, ref_nc):
            seeds = B.seeds()
            ref_seeds = np.array([r["seeds"][k] for r in runs], np.uint32)
            assert np.array_equal(seeds, ref_seeds), f"RNG state differs at step {k}"
    assert (B.status() == 0).all()
    assert nc_mismatch == 0, f"contact counts differ in {nc_mismatch} world-steps"
    assert worst["pos"] < POS_ATOL and worst["q"] < Q_ATOL, worst
    assert worst["lvel"] < VEL_ATOL and worst["avel"] < VEL_ATOL, worst


def test_degenerate_stack_integer_parity(batch_cls):
    """Aligned equal-box stacks: contact counts and RNG state stay bit-exact;
    velocities agree to the level ODE's FP32 build reaches (1e-2 m/s)."""
    sc = _scenes()["stack"]
    runs = oracle_states(sc, 40)
    B = batch_cls(sc)
    for k in (0, 10, 20, 39):
        B.set_state(stacked_state(runs, k))
        B.set_seeds(seeds_before(sc, runs, k))
        B.set_step_index(k)
        B.step(1)
        nc, _, _ = B.counts()
        assert np.array_equal(nc, [r["ncontacts"][k] for r in runs])
        assert np.array_equal(B.seeds(), np.array([r["seeds"][k] for r in runs], np.uint32))
        e = state_err(B.state(), stacked_state(runs, k + 1))
        assert e["lvel"] < 1e-2 and e["avel"] < 1e-2, e


@pytest.mark.parametrize("name", ["batched", "hinge", "box_drop", "tower", "mechanisms"])
def test_rows_and_lambda_tap(batch_cls, name):
    """Row assembly (getInfo2 + rhs + cfm) and SOR lambda per world vs the oracle
    taps, from the same starting state."""
    sc = _scenes()[name]
    k = 30
    runs = oracle_states(sc, k)
    B = batch_cls(sc)
    B.set_state(stacked_state(runs, k))
    B.set_seeds(seeds_before(sc, runs, k))
    B.set_step_index(k)
    rows, lam, fc, row_off = B.step_tap()
    nc, nr, ni = B.counts()
    checked = 0
    for w in range(sc.n_worlds):
        t = O.tap_step(sc, w, k)
        M = t["total_rows"]
        assert nr[w] == M, f"world {w}: rows {nr[w]} vs {M}"
        assert ni[w] == int(np.sum(t["island_rows"] > 0)), f"world {w}: islands"
        if M == 0:
            continue
        R = rows[row_off[w]:row_off[w] + M]
        Ri = R.view(np.int32)
        # island-local -> world rows: islands are contiguous in both
        starts = np.concatenate([[0], np.cumsum(t["island_rows"])])
        gfx = Ri[:, 28]
        ofx = t["findex"][:M]
        isl_of_row = np.searchsorted(starts, np.arange(M), side="right") - 1
        ofx_world = np.where(ofx >= 0, ofx + starts[isl_of_row], -1)
        assert np.array_equal(gfx, ofx_world), f"world {w}: findex"
        assert np.array_equal(np.isinf(R[:, 26]), np.isinf(t["lo"][:M])), f"world {w}: lo inf"
        fin = np.isfinite(t["lo"][:M])
        np.testing.assert_allclose(R[fin, 26], t["lo"][:M][fin], rtol=1e-6, atol=0)
        fin = np.isfinite(t["hi"][:M])
        np.testing.assert_allclose(R[fin, 27], t["hi"][:M][fin], rtol=1e-6, atol=0)
        # bodies: oracle island-local tags -> world-local through body_of
        bstart = np.concatenate([[0], np.cumsum(t["island_bodies"])])
        jb = t["jb"][:M]
        wb1 = t["body_of"][bstart[isl_of_row] + jb[:, 0]]
        wb2 = np.where(jb[:, 1] >= 0, t["body_of"][bstart[isl_of_row] + np.maximum(jb[:, 1], 0)], -1)
        assert np.array_equal(Ri[:, 29], wb1), f"world {w}: b1"
        assert np.array_equal(Ri[:, 30], wb2), f"world {w}: b2"
        np.testing.assert_allclose(R[:, :12], t["J"][:M], rtol=1e-4, atol=2e-5)
        # rhs of a limit row is fps^2 * stop_erp * (angle - stop): 2000 x the
        # FP32 error of an angle read through rotated axes (Euler angular motor)
        np.testing.assert_allclose(R[:, 24], t["rhs"][:M], rtol=1e-3, atol=5e-3)
        np.testing.assert_allclose(R[:, 25], t["cfm"][:M], rtol=1e-5)
        # SOR output per body: cforce = invM J^T lambda (acceleration units; times
        # h it is the velocity change). 20 FP32 PGS iterations vs FP64.
        nbi = int(t["island_bodies"].sum())
        gfc = fc[sc.body_off[w] + t["body_of"][:nbi]]
        np.testing.assert_allclose(gfc, t["cforce"][:nbi], rtol=2e-3, atol=3e-2)
        # lambda of clearly loaded rows (above 1% of the largest and 0.01 N s):
        # where friction rows couple to their normal rows through the pyramid
        # bounds (piles, the joint-type scene), 20 FP32 iterations leave up to
        # ~1.7e-2 relative against FP64 (measured on GB300); joint chains and
        # single-contact scenes agree to ~1e-4
        lam_o = t["lam"][:M]
        big = np.abs(lam_o) > max(1e-2 * np.abs(lam_o).max(), 1e-2)
        lam_rtol = 2e-2 if name in ("batched", "mechanisms") else 1e-3
        np.testing.assert_allclose(lam[row_off[w]:row_off[w] + M][big], lam_o[big], rtol=lam_rtol)
        checked += 1
    assert checked > 0


def test_tower_trajectory_200_steps(batch_cls):
    """Non-chaotic stacks (golden fixture from the reference), 200 steps.
    Per world, the GPU's max position error against the FP64 reference must be
    <= max(1e-4 * scene scale, 1.5 x the drift of the reference's own FP32
    build on the same scene); the stated target 1e-4 relative holds where FP32
    ODE itself reaches it (on GB300 the GPU's error equals the FP32 build's in
    every world, 3e-8 to 7e-4 of the scale)."""
    import os
    g = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "tower.npz")))
    sc = S.Scene.from_arrays(g)
    B = batch_cls(sc)
    B.step(int(g["n_steps"]))
    st = B.state()
    assert (B.status() == 0).all()
    n_tight = 0
    for w in range(sc.n_worlds):
        b0, b1 = sc.world_bodies(w)
        ref = g[f"w{w}_final_d"][:, :3]
        scale = np.abs(ref).max()
        err_gpu = np.abs(st[b0:b1, :3] - ref).max()
        err_s = np.abs(g[f"w{w}_final_s"][:, :3] - ref).max()
        assert err_gpu <= max(1e-4 * scale, 1.5 * err_s), (w, err_gpu, err_s, scale)
        n_tight += err_gpu <= 1e-4 * scale
    assert n_tight >= sc.n_worlds - 1


def test_launch_modes_agree(batch_cls):
    """One launch of n steps, n graph-captured single-step launches and the
    one-world-per-launch path run identical arithmetic: bit-identical states."""
    sc = S.batched_worlds(n_worlds=24, seed=5)
    outs = []
    for mode in ("step", "graph", "plain"):
        B = batch_cls(sc)
        getattr(B, {"step": "step", "graph": "step_graph", "plain": "step_plain"}[mode])(12)
        B.sync()
        outs.append(B.state())
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], outs[2])


def test_solve_register_variants_agree(batch_cls):
    """The solve kernel's two register budgets (168 per thread, or capped at
    128) compile the same device code: 40 steps of a batch agree in contacts,
    rows, islands and RNG state, and in state to FP32 rounding."""
    sc = S.batched_worlds(n_worlds=64, seed=3)
    outs = []
    for variant in (0, 1):
        B = batch_cls(sc)
        w, c, _ = B.launch_config_ex(2)
        B.set_launch_config_ex(2, w, c, variant)
        assert B.launch_config_ex(2)[2] == variant
        B.step(40)
        outs.append((B.state(), B.seeds(), B.counts(), B.status()))
        B.close()
    (sa, ea, ca, ta), (sb, eb, cb, tb) = outs
    assert (ta == 0).all() and (tb == 0).all()
    for x, y in zip(ca, cb):
        assert np.array_equal(x, y)
    assert np.array_equal(ea, eb)
    assert np.abs(sa - sb).max() < 1e-5, float(np.abs(sa - sb).max())


def test_fused_step_matches_split_step(batch_cls):
    """The fused step kernel runs the split kernels' device code on one warp
    per world; compiled into another kernel, the arithmetic may contract into
    FMAs differently, so contacts, rows, islands and RNG state are identical
    and states agree within the one-step bars against the oracle (20 FP32 SOR
    iterations amplify last-bit differences in stiff contact sets). Checked
    one step at a time from the split path's state, at settled steps of the
    batched workload."""
    sc = S.batched_worlds(n_worlds=96, seed=7)
    A = batch_cls(sc)
    F = batch_cls(sc)
    F.set_step_kernels(True)
    assert F.step_kernels()[0] and not A.step_kernels()[0]
    A.step(60)
    worst = dict(pos=0.0, q=0.0, lvel=0.0, avel=0.0)
    for k in range(60, 80):
        F.set_state(A.state())
        F.set_seeds(A.seeds())
        F.set_step_index(k)
        A.step(1)
        F.step(1)
        for x, y in zip(A.counts(), F.counts()):
            assert np.array_equal(x, y)
        assert np.array_equal(A.seeds(), F.seeds())
        e = state_err(F.state(), A.state())
        for key in worst:
            worst[key] = max(worst[key], e[key])
    assert (A.status() == 0).all() and (F.status() == 0).all()
    assert worst["pos"] < POS_ATOL and worst["q"] < Q_ATOL, worst
    assert worst["lvel"] < VEL_ATOL and worst["avel"] < VEL_ATOL, worst
    # the autotuner keeps a valid choice and leaves the state alone
    st = F.state()
    F.autotune(2)
    assert np.array_equal(F.state(), st)
    fused, wpb, carve = F.step_kernels()
    assert 1 <= wpb <= 4 and -1 <= carve <= 100


@pytest.mark.parametrize("name", ["hinge", "batched", "mechanisms"])
def test_joint_feedback_one_step(batch_cls, name):
    """dJointFeedback of every persistent joint (quickstep.cpp:918-957): one
    GPU step from the oracle's state against the oracle's feedback of that
    step. FP32 against FP64 after 20 SOR iterations: |gpu - oracle| <=
    1e-2 * max|oracle| + 5e-3 * |oracle| + 1e-3 * (weight of the world's
    heaviest body) per component; the last term covers constraint forces that
    the FP32 rounding of the starting state alone produces (anchor errors of
    ~1e-6 m times erp / h^2 times the body mass)."""
    sc = _scenes()[name]
    n = 30
    runs = [O.run_world(O.oracle().oracle_run_world, sc, w, n, feedback=True) for w in range(sc.n_worlds)]
    B = batch_cls(sc)
    B.set_feedback(True)
    checked = 0
    for k in (0, 10, 29):
        B.set_state(stacked_state(runs, k))
        B.set_seeds(seeds_before(sc, runs, k))
        B.set_step_index(k)
        B.step(1)
        g = B.feedback()
        nc, _, _ = B.counts()
        for w in range(sc.n_worlds):
            if nc[w] != runs[w]["ncontacts"][k]:
                continue
            j0, j1 = sc.world_joints(w)
            if j1 == j0:
                continue
            ref = runs[w]["feedback"][k][: j1 - j0]
            got = g[j0:j1]
            b0, b1 = sc.world_bodies(w)
            floor = 1e-3 * 9.81 * float(sc.body_mass[b0:b1].max())
            bar = 1e-2 * np.abs(ref).max() + 5e-3 * np.abs(ref) + floor
            assert (np.abs(got - ref) <= bar).all(), (name, k, w, np.abs(got - ref).max(), np.abs(ref).max())
            checked += 1
    B.close()
    assert checked > 0
