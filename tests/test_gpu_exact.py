"""dWorldStep (the exact stepper: ode/src/step.cpp with the Dantzig LCP of
ode/src/lcp.cpp) on the GPU against the FP64 oracle, which is itself
bit-identical to the reference's dWorldStep (test_oracle.py).

The GPU solves each island's LCP in FP32 with the reference's pivoting rules;
the pivot sequence is a function of signs and ratios of FP32 quantities, so
states agree with the FP64 oracle to FP32 rounding of a direct solve.
Integer outputs (contact counts, RNG state) are exact."""
import numpy as np
import pytest

from odegpu import scene as S
from gpu_helpers import stacked_state, seeds_before, state_err
import oracle_lib as O

pytestmark = pytest.mark.gpu

POS_ATOL = 2e-5     # m, one step
Q_ATOL = 2e-5
VEL_ATOL = 2e-3     # m/s, rad/s, one step: FP32 LCP solve vs FP64


def _scenes():
    return {
        "box_drop": S.box_drop(seed=0),
        "batched": S.batched_worlds(n_worlds=32, seed=11),
        "hinge": S.hinge_chains(n_worlds=6, steps=40),
        "mechanisms": S.mechanisms(n_worlds=8, steps=40),
        "vehicles": S.vehicles(n_worlds=4, steps=40, hf_samples=64),
        "cylinder_pile": S.cylinder_pile(n_worlds=2),
    }


def _oracle_exact(sc, n):
    with O.exact_stepper():
        return [O.run_world(O.oracle().oracle_run_world, sc, w, n, max_rec=512, feedback=True)
                for w in range(sc.n_worlds)]


@pytest.mark.parametrize("name", ["box_drop", "batched", "hinge", "mechanisms", "vehicles", "cylinder_pile"])
def test_exact_one_step_from_oracle_state(name):
    """From the oracle's FP64 state at several steps, one dWorldStep on the
    GPU against the oracle's next state: contact counts and RNG state exact,
    positions / orientations within 2e-5, velocities within 2e-3."""
    from odegpu.batch import Batch
    sc = _scenes()[name]
    n = 40
    runs = _oracle_exact(sc, n)
    B = Batch(sc)
    B.set_stepper(True)
    worst = dict(pos=0, q=0, lvel=0, avel=0)
    for k in (0, 5, 15, 25, 39):
        B.set_state(stacked_state(runs, k))
        B.set_seeds(seeds_before(sc, runs, k))
        B.set_step_index(k)
        B.step(1)
        nc, _, _ = B.counts()
        assert np.array_equal(nc, np.array([r["ncontacts"][k] for r in runs])), k
        e = state_err(B.state(), stacked_state(runs, k + 1))
        for key in worst:
            worst[key] = max(worst[key], e[key])
    assert (B.status() == 0).all(), B.status()
    B.close()
    assert worst["pos"] < POS_ATOL and worst["q"] < Q_ATOL, worst
    assert worst["lvel"] < VEL_ATOL and worst["avel"] < VEL_ATOL, worst


def test_exact_tower_trajectory():
    """Non-chaotic stacks (boxes of decreasing size): 100 dWorldStep steps on
    the GPU stay within 1e-4 m of the FP64 oracle."""
    from odegpu.batch import Batch
    sc = S.box_tower(n_worlds=4, yaw=0.0, spacing=0.0)
    n = 100
    runs = _oracle_exact(sc, n)
    B = Batch(sc)
    B.set_stepper(True)
    B.step(n)
    e = state_err(B.state(), stacked_state(runs, n))
    assert (B.status() == 0).all(), B.status()
    B.close()
    assert e["pos"] < 1e-4, e


def test_exact_joint_feedback_one_step():
    """dJointFeedback of the persistent joints (step.cpp:729-770) after one
    dWorldStep from the oracle's state against the oracle's: per component
    within 1e-2 max|oracle| + 5e-3 |oracle| + 1e-3 (weight of the world's
    heaviest body), the bar of the QuickStep feedback test."""
    from odegpu.batch import Batch
    sc = _scenes()["mechanisms"]
    runs = _oracle_exact(sc, 10)
    B = Batch(sc)
    B.set_stepper(True)
    B.set_feedback(True)
    k = 9
    B.set_state(stacked_state(runs, k))
    B.set_seeds(seeds_before(sc, runs, k))
    B.set_step_index(k)
    B.step(1)
    g = B.feedback()
    B.close()
    for w in range(sc.n_worlds):
        j0, j1 = sc.world_joints(w)
        ref = runs[w]["feedback"][k][: j1 - j0]
        b0, b1 = sc.world_bodies(w)
        floor = 1e-3 * 9.81 * float(sc.body_mass[b0:b1].max())
        bar = 1e-2 * np.abs(ref).max() + 5e-3 * np.abs(ref) + floor
        assert (np.abs(g[j0:j1] - ref) <= bar).all(), (w, np.abs(g[j0:j1] - ref).max(), np.abs(ref).max())


def test_exact_launch_modes_agree():
    """dWorldStep through one launch per step, a captured CUDA graph and one
    world per launch gives bit-identical states."""
    from odegpu.batch import Batch
    sc = S.batched_worlds(n_worlds=16, seed=5)
    out = []
    for mode in ("step", "graph", "plain"):
        B = Batch(sc)
        B.set_stepper(True)
        getattr(B, {"step": "step", "graph": "step_graph", "plain": "step_plain"}[mode])(12)
        out.append(B.state())
        B.close()
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])


def test_exact_scratch_sized_by_each_step():
    """The 4096-world batched workload under dWorldStep for 200 steps: each
    step sizes a world's dense scratch by the rows its joints and that step's
    contacts can need, so the device memory the batch holds stays a fraction
    of the layout by row capacity (8 bytes x cap^2 per world, cap = min(1024,
    3 x contact capacity + 6 x joints)), which a captured graph still uses."""
    import torch
    from odegpu.batch import Batch
    sc = S.batched_worlds(n_worlds=4096, seed=1)
    nb = np.diff(sc.body_off)
    nj = np.diff(sc.joint_off)
    cap = np.minimum(1024, 3 * (8 * nb + 16) + 6 * nj).astype(np.float64)
    by_capacity = float((8.0 * cap * cap).sum())
    torch.cuda.init()
    free0, _ = torch.cuda.mem_get_info()
    B = Batch(sc)
    B.set_stepper(True)
    B.step(200)
    free1, _ = torch.cuda.mem_get_info()
    nc = B.counts()[0]
    B.close()
    used = free0 - free1
    assert nc.sum() > 4096 * 10
    assert by_capacity > 8e9
    assert used < 0.2 * by_capacity, (used / 1e9, by_capacity / 1e9)


def test_exact_stepper_guards():
    """The adjoint, the parity taps and the autotuner refuse the exact
    stepper; switching back restores dWorldQuickStep."""
    from odegpu.batch import Batch
    from odegpu._lib import OdeGpuError
    sc = S.box_drop(seed=0)
    B = Batch(sc)
    B.set_stepper(True)
    with pytest.raises(OdeGpuError, match="dWorldStep"):
        B.step_tap()
    B.set_stepper(False)
    B.step(1)
    B.close()
