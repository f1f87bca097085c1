"""Worlds of one scene split over GPUs: contiguous world blocks per rank.

Worlds are independent (ODE steps each world on its own), so a batch shards
by worlds with no exchange inside the step: every rank builds a Batch of its
block of the scene (parameters replicated, per-step controls sliced) and
steps it alone; state and gradients are gathered only when the caller asks.

    blocks = world_blocks(scene.n_worlds, world_size, weights=bodies_per_world(scene))
    sub = slice_scene(scene, *blocks[rank])
    B = ShardedBatch(scene)            # under torch.distributed
    B.step(100)
    full = B.gather_state()            # [nb_total, 13] on rank 0, None elsewhere

The blocks follow the scene's world order, so concatenating the ranks'
outputs in rank order gives the unsplit batch's layout.
"""
from __future__ import annotations

import numpy as np

from .scene import Scene


def bodies_per_world(scene):
    return np.diff(np.asarray(scene.body_off)).astype(np.int64)


def world_blocks(n_worlds, n_shards, weights=None):
    """Contiguous [begin, end) world ranges, one per shard, each as close as
    possible to an equal share of the total weight (bodies per world by
    default: the step's cost grows with them). Every shard gets at least one
    world when n_worlds >= n_shards."""
    if n_shards < 1:
        raise ValueError("n_shards must be >= 1")
    w = np.ones(n_worlds) if weights is None else np.asarray(weights, np.float64)
    if len(w) != n_worlds:
        raise ValueError("one weight per world")
    cum = np.concatenate([[0.0], np.cumsum(w)])
    total = cum[-1]
    cuts = [0]
    for s in range(1, n_shards):
        c = int(np.searchsorted(cum, total * s / n_shards, side="left"))
        # keep at least one world per shard on both sides of the cut
        c = max(c, cuts[-1] + (1 if n_worlds >= n_shards else 0))
        c = min(c, n_worlds - (n_shards - s if n_worlds >= n_shards else 0))
        cuts.append(c)
    cuts.append(n_worlds)
    return [(cuts[s], cuts[s + 1]) for s in range(n_shards)]


def slice_scene(scene, w_begin, w_end):
    """The scene's worlds [w_begin, w_end) as a scene of their own: offsets
    rebased, world parameters (seeds included), surfaces and heightfields
    shared, per-step controls cut to the block's joints and bodies."""
    if not (0 <= w_begin <= w_end <= scene.n_worlds):
        raise ValueError(f"bad world range [{w_begin}, {w_end}) of {scene.n_worlds}")
    a = scene.to_arrays()
    b0, b1 = int(scene.body_off[w_begin]), int(scene.body_off[w_end])
    g0, g1 = int(scene.geom_off[w_begin]), int(scene.geom_off[w_end])
    j0, j1 = int(scene.joint_off[w_begin]), int(scene.joint_off[w_end])
    out = {}
    for k, v in a.items():
        if k in ("joint_torque", "joint_stop"):       # [S][nj_total](...)
            out[k] = v[:, j0:j1]
        elif k == "body_force":                       # [S][nb_total][6]
            out[k] = v[:, b0:b1]
        elif k in ("body_off", "geom_off", "joint_off"):
            out[k] = np.ascontiguousarray(v[w_begin:w_end + 1] - v[w_begin])
        elif k.startswith("body_"):
            out[k] = v[b0:b1]
        elif k.startswith("geom_"):
            out[k] = v[g0:g1]
        elif k.startswith("joint_"):
            out[k] = v[j0:j1]
        elif k == "world_params":
            out[k] = v[w_begin:w_end]
        else:                                         # surfaces, heightfields
            out[k] = v
    return Scene.from_arrays(out)


def _dist():
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return None
    return dist


def gather_blocks(local, dst=0, group=None):
    """Concatenate every rank's numpy array along axis 0 in rank order on
    rank dst (None elsewhere); without an initialised process group, the
    array itself. Works with the gloo and nccl backends (nccl through the
    current CUDA device)."""
    import torch
    dist = _dist()
    if dist is None or dist.get_world_size(group) == 1:
        return np.asarray(local)
    ws = dist.get_world_size(group)
    rank = dist.get_rank(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else "cpu"
    x = np.ascontiguousarray(local)
    # collectives carry signed and floating types: unsigned words travel as
    # their signed bit patterns
    back = None
    if x.dtype in (np.uint32, np.uint64, np.uint16, np.uint8):
        back = x.dtype
        x = x.view({1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}[x.dtype.itemsize])
    n = torch.tensor([x.shape[0]], dtype=torch.int64, device=dev)
    ns = [torch.zeros_like(n) for _ in range(ws)]
    dist.all_gather(ns, n, group=group)
    ns = [int(v.item()) for v in ns]
    m = max(ns)
    t = torch.zeros((m,) + x.shape[1:], dtype=torch.from_numpy(x[:0]).dtype, device=dev)
    if x.shape[0]:
        t[: x.shape[0]] = torch.from_numpy(x).to(dev)
    parts = [torch.zeros_like(t) for _ in range(ws)]
    dist.all_gather(parts, t, group=group)
    if rank != dst:
        return None
    out = np.concatenate([p[:k].cpu().numpy() for p, k in zip(parts, ns)], axis=0)
    return out.view(back) if back is not None else out


class ShardedBatch:
    """This rank's block of a scene as a Batch on this rank's GPU.

    rank / world_size default to the initialised process group (one block
    when there is none); the block is chosen by world_blocks with bodies per
    world as weights. step / state / set_state act on the block; gather_state
    and gather_bodies collect per-body arrays of all blocks in the scene's
    order on one rank."""

    def __init__(self, scene, rank=None, world_size=None, device=None, group=None, **batch_kw):
        from .batch import Batch
        dist = _dist()
        if rank is None:
            rank = dist.get_rank(group) if dist else 0
        if world_size is None:
            world_size = dist.get_world_size(group) if dist else 1
        self.rank, self.world_size, self.group = rank, world_size, group
        self.blocks = world_blocks(scene.n_worlds, world_size, weights=bodies_per_world(scene))
        self.w_begin, self.w_end = self.blocks[rank]
        self.scene = slice_scene(scene, self.w_begin, self.w_end)
        if device is None:
            import os
            device = int(os.environ.get("LOCAL_RANK", "0"))
        self.batch = Batch(self.scene, device=device, **batch_kw)

    def step(self, n=1):
        self.batch.step(n)

    def state(self):
        return self.batch.state()

    def set_state(self, st):
        self.batch.set_state(st)

    def gather_state(self, dst=0):
        return gather_blocks(self.batch.state(), dst=dst, group=self.group)

    def gather_bodies(self, local, dst=0):
        """A per-body array of this block ([nb_block, ...], e.g. a gradient
        with respect to the initial state) gathered over all blocks."""
        return gather_blocks(local, dst=dst, group=self.group)

    def close(self):
        self.batch.close()
