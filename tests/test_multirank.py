"""The multi-rank path of bench.py on CPU (gloo, world size 2): every rank
steps its own shard of worlds (rank-seeded scene, no collective in the step)
and the timed region is the maximum over ranks. The step here is the oracle
on the host; the GPU run uses the same functions with NCCL."""
import os
import socket
import sys
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world_size, port, outdir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world_size)
    import time
    import bench
    import oracle_lib as O
    from odegpu import scene as S
    sc = S.batched_worlds(n_worlds=3, seed=bench.rank_scene_seed(rank))
    t0 = time.perf_counter()
    final = [O.run_world(O.oracle().oracle_run_world, sc, w, 5)["state"][-1] for w in range(sc.n_worlds)]
    t_local = time.perf_counter() - t0 + 0.01 * rank      # ranks end at different times
    t_max = bench.max_over_ranks(t_local)
    np.savez(os.path.join(outdir, f"r{rank}.npz"), final=np.concatenate(final), t_local=t_local, t_max=t_max,
             nb=sc.nb_total)
    tdist.barrier()
    tdist.destroy_process_group()


def test_two_ranks_shard_and_reduce_max():
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(2, _free_port(), d), nprocs=2, join=True, start_method="spawn")
        r = [np.load(os.path.join(d, f"r{k}.npz")) for k in range(2)]
    # every rank saw the slowest rank's time
    t_max = max(float(x["t_local"]) for x in r)
    assert all(abs(float(x["t_max"]) - t_max) < 1e-12 for x in r)
    # distinct shards: different scenes, different results
    assert r[0]["final"].shape != r[1]["final"].shape or not np.allclose(r[0]["final"], r[1]["final"])
    # the aggregate rate counts every rank's worlds over the slowest rank's time
    units = 3 * 5
    rate = units * 2 / t_max
    assert rate < units * 2 / float(r[0]["t_local"]) + 1e-9


def _split_worker(rank, world_size, port, outdir):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world_size)
    import oracle_lib as O
    from odegpu import scene as S
    from odegpu.shard import bodies_per_world, gather_blocks, slice_scene, world_blocks
    out = {}
    for name, sc in (("batched", S.batched_worlds(n_worlds=37, seed=9)),
                     ("vehicles", S.vehicles(n_worlds=6, steps=20, hf_samples=64))):
        b0, b1 = world_blocks(sc.n_worlds, world_size, weights=bodies_per_world(sc))[rank]
        sub = slice_scene(sc, b0, b1)
        x, seeds, counts = O.step_worlds_from(sub, 0, 20, threads=2)
        xs = gather_blocks(x)
        ss = gather_blocks(seeds)
        cs = gather_blocks(counts)
        if rank == 0:
            out[name + "_state"], out[name + "_seeds"], out[name + "_counts"] = xs, ss, cs
        else:
            assert xs is None and ss is None and cs is None
    if rank == 0:
        np.savez(os.path.join(outdir, "gathered.npz"), **out)
    tdist.barrier()
    tdist.destroy_process_group()


def test_scene_split_over_two_ranks_equals_unsplit_run():
    """odegpu.shard: a scene cut into two contiguous world blocks (balanced by
    bodies), each block stepped on its own rank (the oracle stands in for the
    GPU step on CPU), the blocks' states, seeds and per-step counts gathered
    to rank 0 in rank order: bit-identical to stepping the unsplit scene.
    Covers plain worlds and worlds with a shared heightfield and per-step
    controls."""
    sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
    import oracle_lib as O
    from odegpu import scene as S
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_split_worker, args=(2, _free_port(), d), nprocs=2, join=True, start_method="spawn")
        g = dict(np.load(os.path.join(d, "gathered.npz")))
    for name, sc in (("batched", S.batched_worlds(n_worlds=37, seed=9)),
                     ("vehicles", S.vehicles(n_worlds=6, steps=20, hf_samples=64))):
        x, seeds, counts = O.step_worlds_from(sc, 0, 20, threads=2)
        assert np.array_equal(g[name + "_state"], x), name
        assert np.array_equal(g[name + "_seeds"], seeds), name
        assert np.array_equal(g[name + "_counts"], counts), name


def test_world_blocks_cover_and_balance():
    sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
    from odegpu import scene as S
    from odegpu.shard import bodies_per_world, world_blocks
    sc = S.batched_worlds(n_worlds=4096, seed=1)
    w = bodies_per_world(sc)
    for n in (1, 2, 3, 8):
        bl = world_blocks(sc.n_worlds, n, weights=w)
        assert bl[0][0] == 0 and bl[-1][1] == sc.n_worlds
        assert all(a[1] == b[0] for a, b in zip(bl, bl[1:]))
        loads = [w[a:b].sum() for a, b in bl]
        assert max(loads) - min(loads) <= 2 * w.max(), (n, loads)
