"""Sample-range sharding of one frame (rayna_gb300/shard.py) on CPU, with
two gloo ranks and the oracle standing in for each rank's device.

Each rank traces its own samples of every pixel with the frame's random
streams (the oracle's f32 policy, which follows the device's counter
assignment), scales the partial mean to sum / samples as rg_set_sample_range
does, and the sum-reduce of the two partials must equal the one-rank frame.
The gradient reduction is checked the same way.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _scene():
    from rayna_gb300 import presets
    from rayna_gb300.scene import RenderOpts
    scene, cam, _ = presets.random_spheres(seed=0)
    return scene, cam, RenderOpts(width=24, height=16, samples=7, ray_depth=6)


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import binding as ob
    from rayna_gb300 import shard
    from rayna_gb300.scene import flatten
    scene, cam, opts = _scene()
    flat = flatten(scene)
    first, count = shard.sample_range(rank, world, opts.samples)
    frames = 2
    acc = np.zeros((opts.width, opts.height, 3))
    for f in range(frames):  # two frames, each one accumulation step of sum / samples
        st, m, _, _ = ob.render_window(flat, cam, opts, (0, 0, opts.width, opts.height), seed=100 + f,
                                       policy=ob.POLICY_GPU_F32, samples=(first, count))
        assert st == 0
        acc += m * count / opts.samples
    total, n = shard.reduce_accumulation(acc, frames, dist)
    grads = {"albedo": np.full((3, 3), rank + 1.0), "density": np.array([2.0 * rank]), "loss": 1.0 + rank}
    g = shard.allreduce_gradients(grads, dist)
    q.put((rank, first, count, total / n, g))
    dist.destroy_process_group()


def test_sample_range_split():
    from rayna_gb300 import shard
    assert [shard.sample_range(r, 3, 8) for r in range(3)] == [(0, 3), (3, 3), (6, 2)]
    assert [shard.sample_range(r, 2, 1) for r in range(2)] == [(0, 1), (1, 0)]
    with pytest.raises(ValueError):
        shard.sample_range(2, 2, 8)


def test_two_ranks_sum_to_the_one_rank_frame():
    pytest.importorskip("torch")
    import multiprocessing as mp
    from oracle import binding as ob
    from rayna_gb300.scene import flatten
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted((q.get(timeout=300) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    scene, cam, opts = _scene()
    flat = flatten(scene)
    whole = np.zeros((opts.width, opts.height, 3))
    for f in range(2):
        st, m, _, _ = ob.render(flat, cam, opts, seed=100 + f, policy=ob.POLICY_GPU_F32)
        whole += m
    whole /= 2
    assert [(o[1], o[2]) for o in out] == [(0, 4), (4, 3)]
    for _, _, _, mean, g in out:
        np.testing.assert_allclose(mean, whole, rtol=1e-12, atol=1e-12)
        np.testing.assert_array_equal(g["albedo"], np.full((3, 3), 1.5))
        np.testing.assert_array_equal(g["density"], [1.0])
        assert g["loss"] == 1.5
