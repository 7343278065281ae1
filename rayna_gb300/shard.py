"""One frame split across devices by sample range, and the reductions it needs.

The reference renders a frame as a sum over every pixel's samples, folded
into its accumulation buffer (render/renderer.rs:313-336,
render/accum_buffer.rs:37-42). Samples are independent: each is keyed by
(frame, pixel, sample) in the counter-based random streams, so N devices can
share one frame by taking disjoint sample ranges with the same frame keys.
Each device's accumulation then holds the sum over its samples divided by the
pixel's full sample count (rg_set_sample_range); the exchange is one
sum-reduce of those sums, with the frame count equal on every device. The
adjoint adds one sum-reduce of the gradient vector. The scene is replicated.

Every rank must render the same frames with the same keys: give each rank's
Renderer the same `seed` and call render() the same number of times.
"""
from __future__ import annotations

import numpy as np


def sample_range(rank: int, world: int, samples: int) -> tuple[int, int]:
    """Samples [first, first + count) of `samples` that `rank` of `world`
    traces: contiguous, the first `samples % world` ranks one more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    base, extra = divmod(int(samples), int(world))
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def _allreduce_sum(arr: np.ndarray, dist, group=None) -> np.ndarray:
    import torch
    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64).copy())
    dev = None
    if dist.get_backend(group) == "nccl":
        dev = torch.device("cuda", torch.cuda.current_device())
        t = t.to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def reduce_accumulation(sums: np.ndarray, frames: int, dist=None, group=None) -> tuple[np.ndarray, int]:
    """Sum-reduces the accumulation sums of every rank's sample range (f64
    on the wire). Returns (summed sums, frames); raises if the ranks hold
    different frame counts. Without `dist` it returns its input."""
    if dist is None:
        return np.asarray(sums, np.float64), int(frames)
    import torch
    f = torch.tensor([int(frames), -int(frames)], dtype=torch.int64)
    if dist.get_backend(group) == "nccl":
        f = f.to(torch.device("cuda", torch.cuda.current_device()))
    dist.all_reduce(f, op=dist.ReduceOp.MAX, group=group)
    hi, lo = int(f[0]), -int(f[1])
    if hi != lo:
        raise RuntimeError(f"ranks hold different frame counts ({lo}..{hi})")
    return _allreduce_sum(sums, dist, group), int(frames)


def render_sharded(renderer, frames: int, dist=None, group=None) -> np.ndarray:
    """Renders `frames` frames of `renderer` with this rank's share of every
    pixel's samples and returns the whole frames' running mean, (w, h, 3),
    the same on every rank."""
    world = dist.get_world_size(group) if dist is not None else 1
    rank = dist.get_rank(group) if dist is not None else 0
    first, count = sample_range(rank, world, renderer.options.samples)
    if count == 0:
        raise ValueError("more ranks than samples per pixel")
    renderer.set_sample_range(first, count if world > 1 else 0)
    for _ in range(int(frames)):
        renderer.render()
    sums, n = renderer.get_accumulation()
    total, n = reduce_accumulation(sums, n, dist, group)
    return total / max(n, 1)


def allreduce_gradients(grads: dict, dist=None, group=None, average: bool = True) -> dict:
    """Sum-reduces (or averages) every array of a gradient dict from
    Renderer.backward over the ranks; 'loss' is summed likewise."""
    if dist is None:
        return grads
    world = dist.get_world_size(group)
    out = {}
    for k, v in grads.items():
        a = _allreduce_sum(np.atleast_1d(np.asarray(v, np.float64)), dist, group)
        if average:
            a = a / world
        out[k] = float(a[0]) if np.isscalar(v) or np.ndim(v) == 0 else a.reshape(np.shape(v))
    return out
