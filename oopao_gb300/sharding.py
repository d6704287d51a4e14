"""Interaction-matrix columns sharded over ranks (one process per GPU).

The columns of an interaction matrix (modes, push-pull pairs) are
independent (``OOPAO/calibration/InteractionMatrix.py:99-167`` loops over
them), so a multi-GPU build partitions them: every rank measures a
contiguous, balanced slice of the M2C columns on its own GPU, and one gather
of the slices (the only collective) assembles D on every rank.  With
``torch.distributed`` on NCCL the gather moves device tensors; on gloo it
moves host tensors.
"""
import numpy as np
import torch

from .tools import OopaoError


def column_shards(n_cols, world):
    """Balanced contiguous [start, stop) column ranges, one per rank (the
    first n_cols % world ranks take one column more)."""
    if world < 1 or n_cols < 0:
        raise OopaoError('column_shards: world must be >= 1 and n_cols >= 0')
    base, extra = divmod(n_cols, world)
    out, s = [], 0
    for r in range(world):
        e = s + base + (1 if r < extra else 0)
        out.append((s, e))
        s = e
    return out


def gather_columns(local, n_rows, shards, group=None):
    """All-gather column slices [n_rows, stop-start] (numpy or tensor) into the
    full [n_rows, n_cols] float64 numpy matrix on every rank."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    width = max(e - s for s, e in shards)
    backend = dist.get_backend(group)
    dev = torch.device('cuda', torch.cuda.current_device()) if backend == 'nccl' else torch.device('cpu')
    loc = torch.as_tensor(np.asarray(local.cpu() if torch.is_tensor(local) else local, dtype=np.float64))
    s, e = shards[rank]
    if loc.shape != (n_rows, e - s):
        raise OopaoError('gather_columns: rank %d holds %s, expected %s' % (rank, tuple(loc.shape), (n_rows, e - s)))
    pad = torch.zeros((n_rows, width), dtype=torch.float64, device=dev)
    pad[:, :e - s] = loc.to(dev)
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return np.concatenate([parts[r][:, :shards[r][1] - shards[r][0]].cpu().numpy() for r in range(world)], axis=1)


def sharded_interaction_matrix(ngs, tel, dm, wfs, M2C, stroke, group=None, single_pass=True, method='batched',
                               column_fn=None):
    """D [nSignal, nModes] of ``InteractionMatrix`` built column-sharded over
    the ranks of `group`; every rank returns the full float64 D.
    `column_fn(M2C_slice) -> D_slice` replaces the local measurement (default:
    this rank's ``InteractionMatrix(..., invert=False).D``)."""
    import torch.distributed as dist
    M2C = np.asarray(M2C)
    n = M2C.shape[1]
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    shards = column_shards(n, world)
    s, e = shards[rank]
    if column_fn is None:
        from .calibration import InteractionMatrix

        def column_fn(m):
            if m.shape[1] == 0:
                return np.zeros((wfs.nSignal, 0))
            return np.asarray(InteractionMatrix(ngs, tel, dm, wfs, m, stroke, single_pass=single_pass,
                                                method=method, invert=False).D)
    local = column_fn(M2C[:, s:e])
    n_rows = np.asarray(local).shape[0]
    return gather_columns(local, n_rows, shards, group)


def max_over_ranks(value, group=None):
    """Maximum of a float over the ranks (the timing rule of the benchmark)."""
    import torch.distributed as dist
    backend = dist.get_backend(group)
    dev = torch.device('cuda', torch.cuda.current_device()) if backend == 'nccl' else torch.device('cpu')
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
