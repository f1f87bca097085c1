"""The large-world pipeline (one world above the on-chip kernel's 64 bodies,
stepped by grid broadphase, per-pair narrowphase, a one-warp island walk and
a cluster-wide exact-order Gauss-Seidel sweep) on the GPU.

The same world stepped by the warp-per-world kernels and by the large-world
pipeline must agree: both reproduce the reference's contact order, island
order, row order, reshuffles and the sequential sweep in FP32 with the same
expressions, so contact / row / island counts and the RNG state are
identical; the states agree to FP32 rounding (the compiler may fuse the same
expression into FMAs differently in the two kernels). Against the FP64
oracle: contact counts and the RNG state exact, one-step state within the
stated tolerances."""
import numpy as np
import pytest

from odegpu import scene as S
from gpu_helpers import oracle_states, stacked_state, seeds_before, state_err

pytestmark = pytest.mark.gpu


def _run(sc, steps, large):
    from odegpu.batch import Batch
    B = Batch(sc, large_world=large)
    B.step(steps)
    st, seeds, counts, status = B.state(), B.seeds(), B.counts(), B.status()
    B.close()
    return st, seeds, counts, status


@pytest.mark.parametrize("name", ["box_drop", "chains", "capsules"])
def test_large_path_matches_warp_path(name):
    """60 steps of a world that fits both paths: counts and RNG seed
    identical, states within 1e-5."""
    sc = {
        "box_drop": lambda: S.box_drop(seed=0),
        # one world of the batched configuration with ball-joint chains (erp carry)
        "chains": lambda: S.batched_worlds(n_worlds=1, seed=5, nmin=40, nmax=60),
        "capsules": lambda: S.capsule_pile(),
    }[name]()
    a = _run(sc, 60, False)
    b = _run(sc, 60, True)
    assert (a[3] == 0).all() and (b[3] == 0).all(), (a[3], b[3])
    for k in range(3):
        assert np.array_equal(a[2][k], b[2][k]), (k, a[2], b[2])
    assert np.array_equal(a[1], b[1])
    assert np.abs(a[0] - b[0]).max() < 1e-5, float(np.abs(a[0] - b[0]).max())


@pytest.mark.parametrize("name", ["chains", "hinges"])
def test_large_path_feedback_matches_warp_path(name):
    """Joint feedback (quickstep.cpp:918-957) from the large-world pipeline
    against the warp-per-world path, which the parity tests check against the
    oracle: ball chains of the batched configuration and a hinge chain with
    per-step torques touching a plane; 30 steps, the feedback of every step
    within 1e-4 of its scale, and persistent joints only (as ODE's
    dJointFeedback of persistent joints)."""
    from odegpu.batch import Batch
    sc = {
        "chains": lambda: S.batched_worlds(n_worlds=1, seed=5, nmin=40, nmax=60),
        "hinges": lambda: S.hinge_chains(n_worlds=1, links=12, seed=3, steps=30, plane_z=-1.0),
    }[name]()
    A = Batch(sc, large_world=False)
    Lw = Batch(sc, large_world=True)
    for B in (A, Lw):
        B.set_feedback(True)
    worst = 0.0
    for _ in range(30):
        A.step(1)
        Lw.step(1)
        fa, fl = A.feedback(), Lw.feedback()
        scale = max(1.0, float(np.abs(fa).max()))
        worst = max(worst, float(np.abs(fa - fl).max()) / scale)
    assert sc.nj_total > 0
    assert (A.status() == 0).all() and (Lw.status() == 0).all()
    assert np.array_equal(A.counts()[0], Lw.counts()[0])
    assert worst < 1e-4, worst
    A.close()
    Lw.close()


POS_ATOL = 2e-5
Q_ATOL = 2e-5
VEL_ATOL = 5e-3
# angular velocity of the smallest spheres (r = 0.1 m): the linear tolerance / r
AVEL_ATOL = 5e-2


def test_large_world_one_step_from_oracle_state():
    """A 600-sphere pile in a walled box (five static planes, one world):
    from the oracle's FP64 state at several steps, one GPU step against the
    oracle's next state. Contact counts and the RNG state exact; positions /
    orientations within 2e-5, linear velocities within 5e-3 m/s (50 FP32
    iterations on a pile whose initial overlaps push the spheres apart at up
    to a few m/s), angular velocities within that over the smallest radius."""
    from odegpu.batch import Batch
    sc = S.sphere_pile(n=600, box=(2.5, 2.5, 4.0))
    n = 30
    runs = oracle_states(sc, n, max_rec=8)
    B = Batch(sc)
    worst = dict(pos=0, q=0, lvel=0, avel=0)
    for k in (0, 1, 10, 29):
        B.set_state(stacked_state(runs, k))
        B.set_seeds(seeds_before(sc, runs, k))
        B.set_step_index(k)
        B.step(1)
        nc, nr, ni = B.counts()
        assert nc[0] == runs[0]["ncontacts"][k], (k, nc[0], runs[0]["ncontacts"][k])
        assert np.array_equal(B.seeds(), np.array([runs[0]["seeds"][k]], np.uint32)), k
        e = state_err(B.state(), stacked_state(runs, k + 1))
        for key in worst:
            worst[key] = max(worst[key], e[key])
    assert (B.status() == 0).all(), B.status()
    B.close()
    assert worst["pos"] < POS_ATOL and worst["q"] < Q_ATOL, worst
    assert worst["lvel"] < VEL_ATOL and worst["avel"] < AVEL_ATOL, worst


def test_large_world_rejects_what_it_does_not_support():
    from odegpu.batch import Batch
    from odegpu._lib import OdeGpuError
    sc = S.sphere_pile(n=100, box=(2.0, 2.0, 2.0))
    B = Batch(sc)
    with pytest.raises(OdeGpuError, match="large world"):
        B.step_tap()
    B.close()
