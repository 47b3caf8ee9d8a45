"""Multi-GPU layout of a tracking job.

Particles are independent during tracking, so a job shards by particles
(or, for dynamic-aperture scans, by whole error seeds) with no exchange on
the data path: each rank tracks its own contiguous slice and results are
gathered afterwards.
"""


def shard_range(n, rank, world):
    """Contiguous [lo, hi) slice of n items owned by `rank` of `world`;
    the slices cover [0, n) exactly once and differ in size by at most 1."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("invalid rank / world size")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi
