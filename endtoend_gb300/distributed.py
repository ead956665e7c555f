"""Beam sharding over several GPUs, one process per GPU (host side).

The reference splits beams over devices in contiguous blocks, the remainder
going to the first devices (CCCS/dosecalc-beam/main.cu:241-261), computes each
device's dose and sums the device volumes (cuda_sum_device_float_dose,
CCCS/dosecalc-beam/nvbbRayConvolve_host.cu:775-837).  Here every rank is a
process with its own engine context; the dose sum is one all-reduce of the
dose volume.  The EndtoEnd loss gradient needs that summed dose on every rank
(the same all-reduce), after which each rank runs the adjoint of its own
beams and the fluence gradients are gathered.

The per-rank compute is passed in as callables (the engine's device calls on
a GPU rank), so the exchange logic is the same whatever computes the local
part.  torch.distributed carries the collectives: NCCL between GPU ranks,
gloo between CPU processes.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, Tuple

import torch
import torch.distributed as dist


def beam_shards(nbeams: int, world: int) -> List[Tuple[int, int]]:
    """(first beam, count) of every rank: nbeams // world each, the remainder
    one more on the first ranks, contiguous in beam order (main.cu:241-261)."""
    if world <= 0 or nbeams < 0:
        raise ValueError("world must be positive and nbeams non-negative")
    base, extra = divmod(nbeams, world)
    out, start = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        out.append((start, n))
        start += n
    return out


def _world(group) -> Tuple[int, int]:
    if not dist.is_available() or not dist.is_initialized():
        return 0, 1
    return dist.get_rank(group), dist.get_world_size(group)


def sharded_dose(local_dose: Callable[[Sequence], torch.Tensor], beams: Sequence, group=None) -> torch.Tensor:
    """Summed dose of all beams: this rank's shard through local_dose(beams
    of the shard) -> dose volume tensor, then one all-reduce (sum)."""
    rank, world = _world(group)
    first, n = beam_shards(len(beams), world)[rank]
    dose = local_dose(list(beams[first:first + n]))
    if world > 1:
        dist.all_reduce(dose, op=dist.ReduceOp.SUM, group=group)
    return dose


def sharded_loss_and_grad(local_dose: Callable[[Sequence], torch.Tensor],
                          local_adjoint: Callable[[Sequence, torch.Tensor], torch.Tensor],
                          dose_loss: Callable[[torch.Tensor], Tuple[float, torch.Tensor]], beams: Sequence,
                          fluence_sizes: Sequence[int], group=None) -> Tuple[float, torch.Tensor, torch.Tensor]:
    """Loss, dL/d(fluence) of every beam (concatenated in beam order) and the
    summed dose.

    local_dose(shard) -> the shard's dose; dose_loss(dose) -> (loss, dL/d dose),
    evaluated on the summed dose (identical on every rank); local_adjoint(shard,
    dL/d dose) -> the shard's fluence gradient, concatenated; fluence_sizes:
    the beamlet count of every beam.  The shards' gradients are gathered so
    every rank returns the full gradient."""
    rank, world = _world(group)
    shards = beam_shards(len(beams), world)
    dose = sharded_dose(local_dose, beams, group)
    loss, gdose = dose_loss(dose)
    first, n = shards[rank]
    g_local = local_adjoint(list(beams[first:first + n]), gdose).reshape(-1)
    if world == 1:
        return loss, g_local, dose
    lens = [int(sum(fluence_sizes[f:f + k])) for f, k in shards]
    if g_local.numel() != lens[rank]:
        raise ValueError("local_adjoint returned %d values for %d beamlets" % (g_local.numel(), lens[rank]))
    width = max(lens) if lens else 0
    padded = torch.zeros(width, dtype=g_local.dtype, device=g_local.device)
    padded[:g_local.numel()] = g_local
    parts = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(parts, padded, group=group)
    grad = torch.cat([p[:lens[r]] for r, p in enumerate(parts)])
    return loss, grad, dose
