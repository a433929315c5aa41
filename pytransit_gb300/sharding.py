"""Population sharding over ranks (one process per GPU).

Every parameter vector of a RoadRunner evaluation is independent: its own
orbit, limb-darkening profile and light curve (the reference's rr_full
parallel loop over npv, pytransit/models/roadrunner/rrmodel.py:229-290, and
its per-pv OpenCL/numba workers).  A population of npv vectors therefore
splits into contiguous blocks, one per rank, and the data path needs no
exchange.  The only collectives are the caller's: a barrier, a max over ranks
of a step time, and, when one rank wants the whole population's flux, a
gather of the blocks.

These helpers take any model whose ``evaluate(k, ldc, t0, p, a, i, e, w)``
follows the reference's call (RoadRunnerModel, TSModel, EclipseModel ...) and
any process group (NCCL on GPUs, gloo on CPU).
"""
from typing import Optional, Sequence, Tuple

import numpy as np

__all__ = ['pv_block', 'shard_parameters', 'evaluate_sharded', 'max_over_ranks', 'barrier']


def pv_block(npv: int, rank: int, world: int) -> Tuple[int, int]:
    """[start, stop) of rank's block of a population of npv parameter vectors:
    contiguous, sizes differ by at most one, the first npv % world ranks take
    the larger blocks; a rank past npv gets an empty block."""
    if world < 1 or not 0 <= rank < world or npv < 0:
        raise ValueError(f"pv_block: need npv >= 0 and 0 <= rank < world (npv={npv}, rank={rank}, world={world})")
    q, r = divmod(npv, world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def _npv_of(p) -> int:
    # The reference takes npv from the orbital period (rrmodel.py:229).
    return int(np.atleast_1d(np.asarray(p)).size)


def shard_parameters(start: int, stop: int, k, ldc, t0, p, a, i, e=0.0, w=0.0) -> tuple:
    """The block [start, stop) of the evaluate() arguments.  A per-pv argument
    (leading axis npv; limb darkening as an [npv, npb, ncoef] array) is sliced,
    everything else (scalars, shared limb-darkening coefficients) is passed on
    unchanged."""
    npv = _npv_of(p)
    if not 0 <= start <= stop <= npv:
        raise ValueError(f"shard_parameters: block [{start}, {stop}) outside a population of {npv}")

    def cut(x, per_pv_ndim=1):
        x = np.asarray(x)
        if npv > 1 and x.ndim >= per_pv_ndim and x.shape[0] == npv:
            return x[start:stop]
        return x

    return (cut(k), cut(ldc, 3), cut(t0), cut(np.atleast_1d(p)), cut(a), cut(i), cut(e), cut(w))


def _as_block(res, nloc: int) -> np.ndarray:
    """Evaluation result as [nloc, ...]: the models squeeze a single vector's
    leading axis away, as the reference does."""
    res = np.asarray(res.detach().cpu().numpy() if hasattr(res, 'detach') else res, dtype=np.float64)
    if nloc == 1 and (res.ndim == 0 or res.shape[0] != 1 or res.ndim == 1):
        res = res[None]
    return res


def evaluate_sharded(model, k, ldc, t0, p, a, i, e=0.0, w=0.0, gather: bool = True, group=None):
    """Evaluate this rank's block of the population with ``model``.

    Without an initialised process group this is ``model.evaluate``.  With
    one, rank r evaluates pv_block(npv, r, world); with gather=True every rank
    returns the whole population's flux in pv order, squeezed as the model
    squeezes it, else (block_flux [nloc, ...], (start, stop)).
    """
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return model.evaluate(k, ldc, t0, p, a, i, e, w)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    npv = _npv_of(p)
    start, stop = pv_block(npv, rank, world)
    local = None
    if stop > start:
        local = _as_block(model.evaluate(*shard_parameters(start, stop, k, ldc, t0, p, a, i, e, w)), stop - start)
    if not gather:
        return local, (start, stop)
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    blocks = [b for b in parts if b is not None]
    full = np.concatenate(blocks, axis=0)
    return np.squeeze(full) if npv == 1 else full


def _collective_device(group=None):
    import torch
    import torch.distributed as dist
    if dist.get_backend(group) == 'nccl':
        return torch.device('cuda', torch.cuda.current_device())
    return torch.device('cpu')


def max_over_ranks(x: float, group=None) -> float:
    """The maximum of a host scalar (a step time) over the ranks; x itself
    without a process group."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_collective_device(group))
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def barrier(group=None) -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.barrier(group=group)
