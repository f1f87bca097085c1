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


def round32(x):
    """A state as the GPU stores it (FP32), back in FP64."""
    return np.asarray(x, np.float64).astype(np.float32).astype(np.float64)


def world_errors(gpu, ref, body_off, rtol=0.0):
    """Per world max abs error of pos / sign-aligned quaternion / lvel / avel
    beyond rtol * |ref| (each component's error less rtol times its
    reference value, clipped at 0): array [n_worlds, 4]. With rtol = 0 it is
    the plain max abs error."""
    q_g, q_r = gpu[:, 3:7], ref[:, 3:7]
    sgn = np.sign(np.sum(q_g * q_r, axis=1, keepdims=True))
    sgn[sgn == 0] = 1
    d = np.abs(np.concatenate([gpu[:, 0:3] - ref[:, 0:3], q_g * sgn - q_r, gpu[:, 7:13] - ref[:, 7:13]], axis=1))
    r = np.abs(np.concatenate([ref[:, 0:3], q_r, ref[:, 7:13]], axis=1))
    d = np.maximum(d - rtol * r, 0.0)
    e = np.stack([d[:, 0:3].max(axis=1), d[:, 3:7].max(axis=1), d[:, 7:10].max(axis=1), d[:, 10:13].max(axis=1)],
                 axis=1)
    return np.maximum.reduceat(e, np.asarray(body_off[:-1]), axis=0)


ILL_ULPS = (16, 64, 256)


def ill_conditioned(scene, w, step, x_world, seed, want, trials=8, seed_rng=0):
    """Does the oracle's own (contacts, rows, islands) of world w at `step`
    change when its starting positions and orientations move by a few FP32
    units in the last place? Tried at 16, 64 and 256 units (at most 1.5e-5
    relative: 15 micrometres at a metre); returns the smallest level that
    flips a count, or 0 when none does. A decision that flips under input
    changes of that size is a tie at FP32 resolution, which FP32 arithmetic
    inside the step (ODE's own dSINGLE build as much as the GPU) may break
    the other way than FP64."""
    rng = np.random.default_rng(seed_rng)
    x32 = np.asarray(x_world, np.float64).astype(np.float32)
    for ulps in ILL_ULPS:
        for _ in range(trials):
            xp = x32.copy()
            sp = np.spacing(np.abs(xp[:, 0:7])).astype(np.float32)
            xp[:, 0:7] += (rng.integers(-ulps, ulps + 1, size=xp[:, 0:7].shape) * sp).astype(np.float32)
            _, _, c = O.step_worlds_from(scene, step, 1, state=xp.astype(np.float64), seeds=[seed],
                                         w_begin=w, w_end=w + 1, threads=1)
            if not np.array_equal(c[0, 0], want):
                return ulps
    return 0


def pair_diff(scene, B, w, step, x_world, seed):
    """Contacts per body pair that differ between the GPU's last step of
    world w and one oracle step from the same state: {(b1, b2): (gpu, oracle)}."""
    from collections import Counter
    cont, _ = O.step_world_contacts(scene, w, step, x_world, seed)
    g0 = int(scene.geom_off[w])
    gb = scene.geom_body[g0:int(scene.geom_off[w + 1])]
    oc = Counter((int(gb[int(c[7])]), int(gb[int(c[8])])) for c in cont)
    gc = Counter((int(c[7]), int(c[8])) for c in B.contacts(w))
    return {k: (gc.get(k, 0), oc.get(k, 0)) for k in set(oc) | set(gc) if gc.get(k, 0) != oc.get(k, 0)}


def rollout_parity(scene, n_steps, make_batch, state_steps=(), tol=None, rtol=1e-4, max_ill_frac=1e-3,
                   accept=None):
    """Every step of the oracle's own FP64 rollout of `scene` is rounded to
    FP32 (what the GPU stores) and stepped once by the GPU and once by the
    oracle from that identical input. Per world and step, contacts, rows,
    islands with rows and the dRand seed after the step must be equal; a
    difference is accepted only where the oracle's own counts flip under
    FP32-sized perturbations of the input (ill_conditioned) or where
    accept(step, world, gpu_counts) vouches for the GPU's counts (a recorded
    answer of the reference's own FP32 build at that input), and such cases
    stay below max_ill_frac of the world-steps. At the steps in state_steps
    the GPU's state after the step must agree with the oracle's within
    tol + rtol * |oracle| (pos, q, lvel, avel) in every world whose integer
    outputs agree. Returns a summary dict."""
    B = make_batch(scene)
    off = np.asarray(scene.body_off)
    x, seeds, _ = O.step_worlds_from(scene, 0, 0, counts=False)
    nw = scene.n_worlds
    ill, bad, worst, checked = [], [], np.zeros(4), 0
    for k in range(n_steps):
        x32 = round32(x)
        xo, so, co = O.step_worlds_from(scene, k, 1, state=x32, seeds=seeds)
        B.set_state(x32)
        B.set_seeds(seeds)
        B.set_step_index(k)
        B.step(1)
        nc, nr, ni = B.counts()
        g_counts = np.stack([nc, nr, ni], axis=1)
        ok = (g_counts == co[:, 0]).all(axis=1) & (B.seeds() == so)
        assert (B.status() == 0).all(), (k, np.nonzero(B.status())[0][:8])
        for w in np.nonzero(~ok)[0]:
            xw = x32[off[w]:off[w + 1]]
            lvl = ill_conditioned(scene, int(w), k, xw, int(seeds[w]), co[w, 0], seed_rng=k * nw + int(w))
            if lvl:
                ill.append((k, int(w), lvl))
            elif accept is not None and accept(k, int(w), g_counts[w]):
                ill.append((k, int(w), "reference FP32 build"))
            else:
                bad.append((k, int(w), g_counts[w].tolist(), co[w, 0].tolist(),
                            pair_diff(scene, B, int(w), k, xw, int(seeds[w]))))
        if k in state_steps:
            e = world_errors(B.state(), xo, off, rtol)[ok]
            worst = np.maximum(worst, e.max(axis=0, initial=0))
            checked += int(ok.sum())
            if tol is not None:
                lim = np.asarray(tol)
                over = np.nonzero((e > lim).any(axis=1))[0]
                assert len(over) == 0, (k, e[over][:4], lim)
        x, seeds, _ = O.step_worlds_from(scene, k, 1, state=x, seeds=seeds, counts=False)
    B.close()
    assert not bad, bad[:8]
    assert len(ill) <= max_ill_frac * n_steps * nw, (len(ill), ill[:8])
    levels = {u: sum(1 for c in ill if c[2] == u) for u in ILL_ULPS + ("reference FP32 build",)}
    return dict(world_steps=n_steps * nw, ill_conditioned=len(ill), ill_by_ulps=levels,
                worst_beyond_rtol=worst.tolist(), state_worlds_checked=checked)
