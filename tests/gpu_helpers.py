"""Shared helpers for the GPU parity tests: run the oracle to a step, inject
its state into a GPU batch, step once, compare."""
from __future__ import annotations

import numpy as np

import oracle_lib as O


def oracle_states(scene, n_steps, max_rec=512):
    """Per world: dict(state [n+1, nb, 13], ncontacts [n], seeds [n], contacts)."""
    fn = O.oracle().oracle_run_world
    return [O.run_world(fn, scene, w, n_steps, max_rec=max_rec) for w in range(scene.n_worlds)]


def stacked_state(runs, step):
    return np.concatenate([r["state"][step] for r in runs], axis=0)


def seeds_before(scene, runs, step):
    if step == 0:
        return np.array([scene.world_params[w].seed for w in range(scene.n_worlds)], np.uint32)
    return np.array([r["seeds"][step - 1] for r in runs], np.uint32)


def state_err(gpu, ref):
    """Max abs errors of pos / quaternion (sign-aligned) / lvel / avel."""
    q_g, q_r = gpu[:, 3:7], ref[:, 3:7]
    sgn = np.sign(np.sum(q_g * q_r, axis=1, keepdims=True))
    sgn[sgn == 0] = 1
    return dict(pos=np.abs(gpu[:, 0:3] - ref[:, 0:3]).max(initial=0),
                q=np.abs(q_g * sgn - q_r).max(initial=0),
                lvel=np.abs(gpu[:, 7:10] - ref[:, 7:10]).max(initial=0),
                avel=np.abs(gpu[:, 10:13] - ref[:, 10:13]).max(initial=0))
