"""One bunch, or a train of bunches, split over several GPUs (one process
per GPU).

No counterpart in the reference, which tracks a bunch in one process.

Single bunch, sharded by particles.  Every rank holds a contiguous range
of the bunch's macroparticles (``shard_range``) as its own ``Particles``
(same charge per macroparticle, same optics) and runs the whole turn on
it: the element maps act particle by particle, and the slicing pass
writes the rank's partial slice columns.  The only exchange is in the
slicing: each rank folds its columns into compensated per-slice sums
(``phk_slice_sums``: count, sum x, sum y as high and low parts, 6 S
doubles), an all-gather gives every rank all ranks' sums in rank order,
and ``phk_slice_merge`` adds them rank 0 first.  The totals are the
columns' sums to about 2^-106 of the largest partial sum, so every rank
sees the same slice moments, equal to those of one rank holding all the
columns; the wake and its kicks are then computed on every rank from
those moments (replicated) and kick the rank's own particles.  This
replaces the per-slice sums of the reference's slicing
(particles/slicing.py:443-470, cobra_functions/stats.pyx:235-253) that a
bunch split over processes has to combine.  Cuts must be fixed (a
slicer with ``z_cuts``): bunch-dependent cuts and uniform-charge slices
need statistics of the whole bunch and are refused.

Trains of bunches (the batched form): ``pack_bunches`` assigns whole
bunches to ranks by greedy bin packing of their macroparticle counts
(largest first, each to the least-loaded rank), so that no bunch spans
two ranks and no exchange is needed; each rank runs ``BatchedTurn`` on
its bunches.

The exchange goes through ``torch.distributed`` (NCCL between GPUs, gloo
on the host); ``Shards(group=None)`` in a process without a process group
is a single shard.
"""
import numpy as np
import torch


def shard_range(n, rank, world):
    """Particles [start, stop) of shard ``rank`` of ``world``: contiguous,
    sizes differing by at most one, the larger shards first."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError('rank %r outside a world of %r' % (rank, world))
    base, extra = divmod(int(n), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def pack_bunches(sizes, world):
    """Bunch indices per rank: greedy bin packing of the bunches'
    macroparticle counts (largest first; ties to the lower bunch index),
    each to the rank with the fewest particles so far (ties to the lower
    rank).  Every rank's list is in ascending bunch order."""
    if world < 1:
        raise ValueError('world must be >= 1')
    sizes = np.asarray(sizes, dtype=np.int64)
    order = sorted(range(len(sizes)), key=lambda b: (-int(sizes[b]), b))
    load = [0] * world
    out = [[] for _ in range(world)]
    for b in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(b)
        load[r] += int(sizes[b])
    return [sorted(x) for x in out]


class Shards(object):
    """The ranks a bunch is split over: a ``torch.distributed`` process
    group (the default group when ``group`` is None and one is
    initialised), or a single shard."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.group = group
        if dist.is_available() and dist.is_initialized():
            self.rank = dist.get_rank(group)
            self.world = dist.get_world_size(group)
        else:
            if group is not None:
                raise ValueError('a process group was given but '
                                 'torch.distributed is not initialised')
            self.rank, self.world = 0, 1

    def range(self, n):
        return shard_range(n, self.rank, self.world)

    def all_gather(self, t):
        """[world, *t.shape]: every rank's ``t``, rank 0 first."""
        t = t.contiguous()
        if self.world == 1:
            return t.unsqueeze(0)
        import torch.distributed as dist
        flat = t.reshape(-1)
        out = torch.empty(self.world * flat.numel(), dtype=t.dtype,
                          device=t.device)
        dist.all_gather_into_tensor(out, flat, group=self.group)
        return out.view((self.world,) + tuple(t.shape))


def shard(bunch, shards):
    """Mark ``bunch`` (this rank's particles) as one shard of a bunch split
    over ``shards``: its slicings merge the slice sums of every shard."""
    bunch._shard = shards
    return bunch


def merged_slice_moments(beam, acc, counts, mean_x, mean_y, moments_out,
                         stream):
    """Slice counts, means and wake moments of the whole sharded bunch from
    this shard's accumulation ``acc`` (an AccumRequest that has run)."""
    import ctypes
    from . import _native as N
    S = acc.dslicer.n_slices
    local = torch.empty(2, 3, S, dtype=torch.float64, device=beam._device)
    a = acc.struct()
    N.call('phk_slice_sums', ctypes.byref(a), local.data_ptr(), stream)
    gathered = beam._shard.all_gather(local)
    N.call('phk_slice_merge', gathered.data_ptr(), gathered.shape[0], S,
           counts.data_ptr(), 0 if mean_x is None else mean_x.data_ptr(),
           0 if mean_y is None else mean_y.data_ptr(),
           0 if moments_out is None else moments_out.data_ptr(), stream)
