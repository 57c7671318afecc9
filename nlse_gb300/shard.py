"""Sharding whole fields across ranks (one process per GPU).

Fields never interact during propagation, so ranks split a batch into
contiguous blocks of whole fields, advance them independently (no collective
on the data path) and gather the results once at the end.
"""

from __future__ import annotations

import torch


def field_block(n_fields: int, rank: int, world: int) -> slice:
    """Contiguous, balanced block of fields of `rank` (the first n % world ranks
    take one more)."""
    if world <= 0 or not 0 <= rank < world or n_fields < 0:
        raise ValueError("need 0 <= rank < world and n_fields >= 0")
    base, extra = divmod(n_fields, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def gather_fields(local: torch.Tensor, n_fields: int, group=None) -> torch.Tensor:
    """All ranks' blocks (leading dimension) in rank order, on every rank.

    One all_gather of equal-size buffers (blocks padded to the largest);
    complex tensors travel as their real view.
    """
    import torch.distributed as dist

    world = dist.get_world_size(group)
    sizes = [field_block(n_fields, r, world) for r in range(world)]
    longest = max(s.stop - s.start for s in sizes)
    x = torch.view_as_real(local) if local.is_complex() else local
    buf = torch.zeros((longest,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
    buf[: x.shape[0]] = x
    parts = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=group)
    out = torch.cat([p[: s.stop - s.start] for p, s in zip(parts, sizes)])
    return torch.view_as_complex(out) if local.is_complex() else out
