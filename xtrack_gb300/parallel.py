"""Multi-GPU layout of a tracking job: one beam split over the ranks.

Particles are independent during tracking, so a job shards by particles
(or, for dynamic-aperture scans, by whole error seeds) with no exchange on
the data path: each rank tracks a contiguous particle_id range of the beam
on its own GPU, and the per-particle results are gathered afterwards. The
gather is a host-side exchange over a gloo process group (torch.distributed),
not a device collective: the ranks may sit on different boxes with one GPU
each.
"""
import numpy as np
import torch

from .particles import PER_PARTICLE_FIELDS, Particles

# Per-particle fields the push writes (and therefore the gather returns).
TRACKED_FIELDS = ("x", "px", "y", "py", "zeta", "delta", "ptau", "rpp", "rvv", "s", "ax", "ay",
                  "state", "at_element", "at_turn")


def shard_range(n, rank, world):
    """Contiguous [lo, hi) slice of n items owned by `rank` of `world`;
    the slices cover [0, n) exactly once and differ in size by at most 1."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("invalid rank / world size")
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return lo, hi


def shard_slots(particles, rank, world):
    """Slots of `particles` whose particle_id falls in the rank's range of
    the sorted ids (ids need not be stored in order)."""
    ids = particles.particle_id.cpu().numpy()
    order = np.argsort(ids, kind="stable")
    lo, hi = shard_range(len(order), rank, world)
    return order[lo:hi]


def take_shard(particles, slots, device=None):
    """A new Particles holding the given slots of `particles` on `device`."""
    d = particles.to_dict()
    for f in PER_PARTICLE_FIELDS:
        d[f] = d[f][slots]
    return Particles.from_dict(d, device=device if device is not None else particles.device)


def _gloo_group(group):
    import torch.distributed as dist
    if group is not None:
        return group
    if dist.get_backend() == "gloo":
        return None
    return dist.new_group(backend="gloo")


def gather_shards(particles, shard, slots, group=None):
    """Writes every rank's tracked shard back into `particles` on every rank
    (host-side all-gather over gloo): each rank passes its own shard and the
    slots it was taken from."""
    import torch.distributed as dist
    g = _gloo_group(group)
    world = dist.get_world_size(g)
    n_fields = len(TRACKED_FIELDS)
    rows = [shard.to_numpy()[f] for f in TRACKED_FIELDS]
    packed = np.stack([r.view(np.float64) if r.dtype == np.int64 else r for r in rows])
    width = torch.tensor([packed.shape[1]], dtype=torch.int64)
    widths = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(widths, width, group=g)
    wmax = int(max(int(w) for w in widths))
    buf = torch.zeros((n_fields + 1, wmax), dtype=torch.float64)
    buf[:n_fields, :packed.shape[1]] = torch.from_numpy(packed)
    buf[n_fields, :len(slots)] = torch.from_numpy(np.asarray(slots, dtype=np.int64).view(np.float64))
    parts = [torch.zeros_like(buf) for _ in range(world)]
    dist.all_gather(parts, buf, group=g)
    full = particles.to_numpy()
    out = {f: full[f].copy() for f in TRACKED_FIELDS}
    for r, part in enumerate(parts):
        w = int(widths[r])
        a = part.numpy()
        sl = a[n_fields, :w].view(np.int64)
        for k, f in enumerate(TRACKED_FIELDS):
            v = a[k, :w]
            out[f][sl] = v.view(np.int64) if out[f].dtype == np.int64 else v
    for f in TRACKED_FIELDS:
        setattr(particles, f, torch.from_numpy(out[f]))
    return particles


def track_sharded(line, particles, group=None, device=None, track=None, **track_kw):
    """Line.track of one beam over the ranks of a torch.distributed job.

    Every rank passes the same full `particles`; rank r tracks the r-th
    contiguous particle_id range (shard_range) on `device` (default: the
    beam's device) with ``line.track(shard, **track_kw)``, or with
    ``track(line, shard, **track_kw)`` when given, and the tracked
    coordinates, state, at_turn and at_element of all ranks are gathered
    back into `particles` on every rank. The results equal one unsharded
    call: particles never interact during tracking. Turn-by-turn monitors
    record per shard and are not gathered, so they are rejected here."""
    import torch.distributed as dist
    if track_kw.get("turn_by_turn_monitor"):
        raise ValueError("track_sharded: turn-by-turn monitors are per shard; track each shard "
                         "with line.track to record them")
    g = _gloo_group(group)
    rank, world = dist.get_rank(g), dist.get_world_size(g)
    slots = shard_slots(particles, rank, world)
    shard = take_shard(particles, slots, device=device)
    if track is None:
        line.track(shard, **track_kw)
    else:
        track(line, shard, **track_kw)
    return gather_shards(particles, shard, slots, group=g)
