"""Heightfield collider (dCollideHeightfield, ode/src/heightfield.cpp:1677-1853)
and the vehicle batch on the CUDA path: single collider calls against the
reference's golden records, and one-step parity of the vehicle scene
(hinge2 suspension, per-step steering stops and wheel torques, heightfield
contacts) against the FP64 oracle.

Contact counts must match exactly; contact records (FP32 against the FP64
reference) within 1e-4 m / 1e-4 (normals) / 1e-4 m (depth)."""
import os

import numpy as np
import pytest

from odegpu import scene as S
from gpu_helpers import oracle_states, stacked_state, seeds_before, state_err

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ATOL = 1e-4


def _q_from_R(R):
    """Unit quaternion (w, x, y, z) of a rotation matrix."""
    R = np.asarray(R, float).reshape(3, 3)
    t = np.trace(R)
    if t > 0:
        s = 2.0 * np.sqrt(1.0 + t)
        q = [0.25 * s, (R[2, 1] - R[1, 2]) / s, (R[0, 2] - R[2, 0]) / s, (R[1, 0] - R[0, 1]) / s]
    else:
        i = int(np.argmax(np.diag(R)))
        j, k = (i + 1) % 3, (i + 2) % 3
        s = 2.0 * np.sqrt(1.0 + R[i, i] - R[j, j] - R[k, k])
        v = [0.0, 0.0, 0.0]
        v[i] = 0.25 * s
        v[j] = (R[j, i] + R[i, j]) / s
        v[k] = (R[k, i] + R[i, k]) / s
        q = [(R[k, j] - R[j, k]) / s] + v
    q = np.array(q)
    return q / np.linalg.norm(q)


def _kat_scene(g, idx):
    """The golden calls idx as worlds of their own: the heightfield first in
    creation order (so the batch calls dCollide in the same argument order),
    then a body carrying the call's geom."""
    h = g["heights"]
    sp = float(g["spacing"])
    b = S.SceneBuilder()
    surf = b.add_surface(0, 0.5)
    hf = b.add_heightfield(h, sp * (h.shape[1] - 1), sp * (h.shape[0] - 1), pos=g["hf_pos"],
                           R=np.asarray(g["hf_R"]).reshape(3, 3))
    for i in idx:
        w = b.new_world(max_contacts=int(g["flags"][i]), seed=1)
        b.add_geom(w, S.GEOM_HEIGHTFIELD, -1, (hf,), surf)
        bi = b.add_body(w, tuple(g["pos2"][i]), 1.0, np.eye(3) * 0.1, q=tuple(_q_from_R(g["R2"][i])))
        b.add_geom(w, int(g["t2"][i]), bi, tuple(g["p2"][i]), surf)
    return b.build()


def _compare_kats(g, idx, contacts_of, count_mism, scale=1.0):
    worst = 0.0
    for w, i in enumerate(idx):
        c = contacts_of(w)
        nc = int(g["nc"][i])
        if len(c) != nc:
            count_mism.append((i, len(c), nc))
            continue
        if nc:
            worst = max(worst, float(np.abs(c[:, :7] - g["out"][i][:nc, :7]).max()) / scale)
    return worst


@pytest.mark.parametrize("fixture", ["hf_kats", "hf_big_kats"])
def test_heightfield_kats_on_gpu(fixture):
    """Each golden dCollide(heightfield, geom) call as a world of its own; the
    contacts of the first step are the call's. hf_big_kats holds geoms of
    several metres on a 0.25 m field (zones of up to ~60 samples per axis,
    beyond the lane's 10 x 10 arrays): those worlds collide through their
    heightfield workspace, and a sample of them also through the large-world
    pipeline (one world per batch). Records within 1e-4 (relative to the
    coordinates' scale, up to ~12 m, for the large geoms)."""
    from odegpu.batch import Batch
    g = np.load(os.path.join(GOLDEN, f"{fixture}.npz"))
    n = len(g["t2"])
    idx = list(range(n))
    B = Batch(_kat_scene(g, idx))
    B.step(1)
    assert (B.status() == 0).all(), B.status()
    count_mism = []
    scale = 1.0 if fixture == "hf_kats" else 12.0
    worst = _compare_kats(g, idx, B.contacts, count_mism, scale)
    B.close()
    if fixture == "hf_big_kats":
        for i in range(0, n, 10):
            Lw = Batch(_kat_scene(g, [i]), large_world=True)
            Lw.step(1)
            assert Lw.status()[0] == 0, (i, Lw.status())
            worst = max(worst, _compare_kats(g, [i], Lw.contacts, count_mism, scale))
            Lw.close()
    assert not count_mism, f"contact counts differ: {count_mism[:10]}"
    assert worst < ATOL, worst
    assert (g["nc"] > 0).sum() > n // 2


POS_ATOL = 2e-5
Q_ATOL = 2e-5
VEL_ATOL = 2e-3


def test_vehicles_one_step_from_oracle_state():
    """Vehicle batch: from the oracle's FP64 state at several steps, one GPU
    step against the oracle's next state; contact counts and RNG state exact."""
    from odegpu.batch import Batch
    sc = S.vehicles(n_worlds=12, steps=60, hf_samples=64)
    n = 60
    runs = oracle_states(sc, n)
    B = Batch(sc)
    worst = dict(pos=0, q=0, lvel=0, avel=0)
    nc_mismatch = 0
    for k in (0, 10, 20, 35, 59):
        B.set_state(stacked_state(runs, k))
        B.set_seeds(seeds_before(sc, runs, k))
        B.set_step_index(k)
        B.step(1)
        g = B.state()
        nc, _, _ = B.counts()
        ref_nc = np.array([r["ncontacts"][k] for r in runs])
        nc_mismatch += int(np.sum(nc != ref_nc))
        e = state_err(g, stacked_state(runs, k + 1))
        for key in worst:
            worst[key] = max(worst[key], e[key])
        if np.array_equal(nc, ref_nc):
            ref_seeds = np.array([r["seeds"][k] for r in runs], np.uint32)
            assert np.array_equal(B.seeds(), ref_seeds), f"RNG state differs at step {k}"
    assert (B.status() == 0).all(), B.status()
    B.close()
    assert nc_mismatch == 0, f"contact counts differ in {nc_mismatch} world-steps"
    assert worst["pos"] < POS_ATOL and worst["q"] < Q_ATOL, worst
    assert worst["lvel"] < VEL_ATOL and worst["avel"] < VEL_ATOL, worst
