"""Data parallelism over GPUs for the expectation / apply path.

One process per GPU.  The unit of work is a state column: every method of
PauliString / PauliOp / SummedPauliOp treats the columns of a (2^n, S) state
batch independently (the reference loops over them inside one call, e.g.
SummedPauliOp::expectation_value, fast_pauli/cpp/include/__summed_pauli_op.hpp:556-588),
so ranks take disjoint column ranges and exchange nothing on the data path.
Only timings (and, for a caller that wants the whole result on one rank,
the output columns) cross ranks.

The helpers take the ``torch.distributed`` module (or ``None`` for one
process) so that the same code runs under NCCL on GPUs and under gloo on CPU.
"""

from __future__ import annotations


def column_shard(n_states: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous column range [begin, end) of ``rank`` out of ``world``; the
    first ``n_states % world`` ranks take one column more.  Ranks past the
    last column get an empty range."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} out of range for world size {world}")
    if n_states < 0:
        raise ValueError("n_states must be >= 0")
    base, extra = divmod(n_states, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def shard_columns(states, world: int, rank: int):
    """This rank's columns of a (2^n, S) state batch (a view; numpy arrays
    and torch tensors alike).  A 1-D state is one column: rank 0 keeps it,
    the others get an empty (2^n, 0) batch."""
    if states.ndim == 1:
        return states if rank == 0 else states.reshape(-1, 1)[:, :0]
    b, e = column_shard(states.shape[1], world, rank)
    return states[:, b:e]


def _device_for(dist):
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def max_over_ranks(value: float, dist=None) -> float:
    """Max of a per-rank float (a step time) over all ranks; the value
    itself without a process group."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=_device_for(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None) -> float:
    """Sum of a per-rank count (units processed) over all ranks."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=_device_for(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def gather_columns(local, n_states: int, dist=None, dst: int = 0):
    """Reassemble the (rows, n_states) result on rank ``dst`` from every
    rank's (rows, shard) block, in column order; other ranks get ``None``.
    ``local`` is a torch tensor on the backend's device.  This is a result
    collection step, not part of the timed data path."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return local
    import torch

    world, rank = dist.get_world_size(), dist.get_rank()
    if local.is_complex():  # collectives move the (re, im) pairs as reals
        full = gather_columns(torch.view_as_real(local.contiguous()), n_states, dist, dst)
        return None if full is None else torch.view_as_complex(full.contiguous())
    rows = local.shape[0]
    widest = column_shard(n_states, world, 0)[1]
    # equal-size blocks for the collective; each rank pads its own
    buf = torch.zeros((rows, widest) + tuple(local.shape[2:]), dtype=local.dtype, device=local.device)
    buf[:, : local.shape[1]] = local
    blocks = [torch.empty_like(buf) for _ in range(world)] if rank == dst else None
    dist.gather(buf, gather_list=blocks, dst=dst)
    if rank != dst:
        return None
    parts = []
    for r in range(world):
        b, e = column_shard(n_states, world, r)
        parts.append(blocks[r][:, : e - b])
    return torch.cat(parts, dim=1)
