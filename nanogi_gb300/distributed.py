"""Sample sharding across processes (one GPU per process).

Paths are independent (src/nanogi.cpp:281-319), so N samples split into disjoint ranges,
one per rank, each rendered with the same Philox seed. Every sample keeps its global index,
so a sharded render traces exactly the paths of a single-process render. The only exchange
is one sum of the W*H*3 FP64 film at the end of the job, the counterpart of the reference's
per-thread film gather (src/nanogi.cpp:429-437).

Shards are cut at whole-image passes (multiples of W*H samples). The pixel stratification
then matches the single-process render exactly, and the summed film is identical up to the
order of floating-point additions.
"""
from __future__ import annotations

from typing import Callable


def shard_range(num_samples: int, width: int, height: int, world: int, rank: int) -> tuple[int, int]:
    """(offset, count) of rank's samples: whole passes dealt out evenly, remainder to the last rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world / rank")
    wh = width * height
    passes = num_samples // wh
    base, extra = divmod(passes, world)
    start_pass = rank * base + min(rank, extra)
    my_passes = base + (1 if rank < extra else 0)
    offset = start_pass * wh
    count = my_passes * wh
    if rank == world - 1:
        count = num_samples - offset
    return offset, count


def reduce_film(film, group=None):
    """Sums a film (torch tensor, any device the backend supports) over all ranks in place."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(film, op=dist.ReduceOp.SUM, group=group)
    return film


def render_sharded(render_raw: Callable[[int, int], "object"], num_samples: int, width: int, height: int,
                   rank: int, world: int, group=None):
    """Renders rank's shard with render_raw(offset, count) -> raw-sum film (torch tensor),
    sums the films over ranks and normalises by W*H/N as RenderProcess does."""
    offset, count = shard_range(num_samples, width, height, world, rank)
    film = render_raw(offset, count)
    reduce_film(film, group)
    if num_samples > 0:
        film *= (width * height) / num_samples
    return film


def render_device_sharded(scene, renderer, film, rank: int, world: int, group=None, stream: int = 0):
    """GPU shard: adds this rank's samples into the device film, then sums over ranks.

    renderer: nanogi_gb300.Renderer with the job's TOTAL num_samples; film: zeroed torch
    CUDA float64 tensor of shape (H, W, 3). Returns the normalised film.
    """
    import copy

    def raw(offset, count):
        r = copy.copy(renderer)
        r.sample_offset = renderer.sample_offset + offset
        r.num_samples = count
        if count > 0:
            r.render_device(scene, film.data_ptr(), stream)
        return film

    return render_sharded(raw, renderer.num_samples, renderer.width, renderer.height, rank, world, group)
