"""Parity at the workloads' full sizes: the 4096-world batch (the bench
workload) over 200 steps, 1024 hinge chains over 100 steps with the plane at
z = -2, 2048 vehicles on the 256 x 256 heightfield over 300 steps, and the
10,000-sphere world.

Every step of the oracle's FP64 rollout is re-injected into the GPU (rounded
to FP32, the GPU's storage) and into the oracle, and both step once from that
identical input. Contacts, rows, islands with rows and the dRand seed after
the step agree in every world at every step; the only accepted differences
are decisions that the oracle itself flips when its input moves by FP32-sized
amounts (ties at FP32 resolution), and, on the heightfield, the recorded
inputs where the reference's own FP32 and FP64 builds disagree (the GPU must
give the FP32 build's count there), together at most 0.1% of the world-steps. At the
listed steps the state after the step agrees within the one-step tolerances
of test_gpu_parity.py plus 1e-4 of the oracle's value (the stated relative
target; fast-spinning wheels carry tens of rad/s) in every world whose
integer outputs agree."""
import numpy as np
import pytest

from odegpu import scene as S
from gpu_helpers import rollout_parity, round32
import oracle_lib as O

pytestmark = pytest.mark.gpu

# pos (m), q, lvel (m/s), avel (rad/s): one FP32 step against one FP64 step
TOL = (2e-5, 2e-5, 2e-3, 2e-3)


def _batch(sc):
    from odegpu.batch import Batch
    return Batch(sc)


def test_batched_4096_worlds_200_steps():
    """The bench workload itself: batched_worlds(4096, seed=1), steps 0-199,
    state checked at steps 0, 150 and 199 (settled piles, ~130 rows/world)."""
    sc = S.batched_worlds(n_worlds=4096, seed=1)
    r = rollout_parity(sc, 200, _batch, state_steps=(0, 150, 199), tol=TOL)
    print("batched 4096:", r)
    assert r["state_worlds_checked"] > 3 * 4096 * 0.99


def test_hinge_chains_1024_plane_at_minus_2():
    """1024 eight-link hinge chains with per-step torques, plane at z = -2
    (end links reach it): 100 steps."""
    sc = S.hinge_chains(n_worlds=1024, steps=100, plane_z=-2.0)
    r = rollout_parity(sc, 100, _batch, state_steps=(0, 50, 99), tol=TOL)
    print("hinge chains 1024:", r)


def test_vehicles_2048_cars_300_steps():
    """2048 cars on the 256 x 256 fractal heightfield with per-step steering
    stops and drive torques: 300 steps. The suspension rows (ERP 0.4, CFM
    0.01 on a 1000 kg chassis) make the chassis velocity about 3x as
    sensitive to the FP32 input as a rigid contact, hence 5e-3 m/s beside
    the relative 1e-4. A wheel's spin takes the friction impulse of a quarter
    of the car (~25 N s per step) through its 0.35 m radius and 0.98 kg m^2
    inertia: the 1e-3 relative difference that 20 unconverged FP32 Gauss-
    Seidel iterations leave in that impulse is ~9e-3 rad/s, hence 1e-2
    rad/s for angular velocity."""
    sc = S.vehicles(n_worlds=2048, steps=300)
    r = rollout_parity(sc, 300, _batch, state_steps=(0, 150, 299), tol=(2e-5, 2e-5, 5e-3, 1e-2),
                       accept=_reference_single_build_cases())
    print("vehicles 2048:", r)


def _reference_single_build_cases():
    """The world-steps of the vehicle rollout where the reference's dSINGLE
    and dDOUBLE builds disagree on a geom's heightfield contacts
    (tests/golden/vehicle_hf_cases.npz, made from the reference by
    make_vehicle_hf_cases.py and replayed on CPU by test_oracle.py). The
    GPU's heightfield collider computes in FP32 like the dSINGLE build: there
    its contact count must be the dSINGLE build's."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "vehicle_hf_cases.npz"))
    want = {(int(k), int(w)): int(n) for k, w, n in zip(g["step"], g["world"], g["contacts_single"])}

    def accept(k, w, counts):
        return want.get((k, w)) == int(counts[0])
    return accept


def _pairs(rec, gi, gk):
    return [(int(a), int(b)) for a, b in zip(rec[:, gi], rec[:, gk])]


def test_sphere_pile_10k_one_step_from_oracle_state():
    """The 10,000-sphere world (large-world pipeline): one step from the
    oracle's state at steps 0 and 100. Contacts are compared pair by pair:
    a contact present on one side only must be a grazing one (|depth| below
    2e-6 m, a few FP32 units at the pile's coordinates); the RNG seed and the
    row count agree when the contact sets do; positions within 2e-5 m,
    velocities within 5e-3 m/s (5e-2 rad/s for angular velocity, the linear
    tolerance over the smallest radius), as for the 600-sphere pile."""
    from odegpu.batch import Batch
    sc = S.sphere_pile(n=10000)
    x, seeds, _ = O.step_worlds_from(sc, 0, 0, counts=False)
    B = Batch(sc)
    done = 0
    for k in range(101):
        if k in (0, 100):
            x32 = round32(x)
            cont, after = O.step_world_contacts(sc, 0, k, x32, int(seeds[0]))
            B.set_state(x32)
            B.set_seeds(seeds)
            B.set_step_index(k)
            B.step(1)
            assert B.status()[0] == 0
            nc, nr, ni = B.counts()
            g = B.contacts(0, cap=200000)
            assert len(g) == nc[0]
            # oracle contacts by geom pair; GPU contacts by body pair (geom i
            # is on body i - 5 for the 5 static planes first, see scene)
            gb = sc.geom_body
            o_pairs = {}
            for c in cont:
                key = (int(gb[int(c[7])]), int(gb[int(c[8])]))
                o_pairs.setdefault(key, []).append(c[6])
            g_pairs = {}
            for c in g:
                key = (int(c[7]), int(c[8]))
                g_pairs.setdefault(key, []).append(c[6])
            for key in set(o_pairs) | set(g_pairs):
                a, b = o_pairs.get(key, []), g_pairs.get(key, [])
                if len(a) != len(b):
                    extra = sorted(a)[: len(a) - len(b)] if len(a) > len(b) else sorted(b)[: len(b) - len(a)]
                    assert max(abs(float(v)) for v in extra) < 2e-6, (k, key, a, b)
            if len(cont) == nc[0]:
                _, so, co = O.step_worlds_from(sc, k, 1, state=x32, seeds=seeds)
                assert nr[0] == co[0, 0, 1] and ni[0] == co[0, 0, 2], (k, nr, ni, co[0, 0])
                assert B.seeds()[0] == so[0]
            st = B.state()
            e_pos = np.abs(st[:, 0:3] - after[:, 0:3]).max()
            e_lv = np.abs(st[:, 7:10] - after[:, 7:10]).max()
            e_av = np.abs(st[:, 10:13] - after[:, 10:13]).max()
            print(f"sphere pile step {k}: contacts gpu {nc[0]} oracle {len(cont)}, "
                  f"errors pos {e_pos:.3g} lvel {e_lv:.3g} avel {e_av:.3g}")
            assert e_pos < 2e-5 and e_lv < 5e-3 and e_av < 5e-2, (k, e_pos, e_lv, e_av)
            done += 1
        if k < 100:
            x, seeds, _ = O.step_worlds_from(sc, k, 1, state=x, seeds=seeds, counts=False)
    B.close()
    assert done == 2
