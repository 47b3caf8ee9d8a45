"""Launch autotuner of the push: block size, staging chunk of the element
table, compaction period and CUDA-graph replay.

None of these change results (the kernels compute every particle the same
way under every tuning); they change only the time. The search is a
coordinate descent from the library's default tuning: each parameter in
turn is set to every candidate value while the others keep their best
values so far, and each candidate is timed on a copy of the caller's
particles over a short probe run (CUDA events on the current stream, best
of ``repeats``).

Results are kept in a JSON cache keyed by the device, the lattice (a hash of
its element records and configuration), the arithmetic mode and the
problem size rounded to a power of two, so a later run with the same key
applies the stored tuning without timing anything.
"""
import hashlib
import json
import os

import numpy as np

SPACE = {
    "block_size": (32, 64, 128, 256),
    "chunk_bytes": (0, 12288, 16384, 32768, 49152, 98304),
    "compact_every": (0, 1, 8, 64),
    "use_graph": (0, 1),
}
ORDER = ("block_size", "chunk_bytes", "compact_every", "use_graph")


def _pow2_bucket(n):
    n = max(int(n), 1)
    return 1 << (n - 1).bit_length()


def tuning_key(tracker, n_particles, num_turns, device_name=None):
    """Cache key of a tracking problem."""
    h = hashlib.sha1()
    recs = getattr(tracker, "_records", None)
    if recs is None and hasattr(tracker, "_seeds"):
        for t in tracker._seeds:
            h.update(np.ascontiguousarray(t._records).tobytes())
    elif recs is not None:
        h.update(np.ascontiguousarray(recs).tobytes())
    h.update(bytes(tracker._cfg))
    if device_name is None:
        import torch
        props = torch.cuda.get_device_properties(tracker.device)
        device_name = f"{props.name}/{props.multi_processor_count}"
    return "|".join([device_name, h.hexdigest()[:16], tracker.arith,
                     f"n{_pow2_bucket(n_particles)}", f"t{_pow2_bucket(num_turns)}"])


def load_cache(path):
    if path and os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def save_cache(path, cache):
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _cuda_timer(tracker, particles, num_turns, repeats, lattice_index=None):
    import torch

    def run(tuning):
        tracker.set_tuning(**tuning)
        best = float("inf")
        for _ in range(repeats + 1):           # the first run warms up
            p = particles.copy()
            stream = torch.cuda.current_stream(p.device)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if lattice_index is None:
                tracker._track(p, num_turns=num_turns)
            else:
                tracker.track(p, lattice_index=lattice_index, num_turns=num_turns)
            e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        tracker.device_status()
        return best
    return run


def autotune(tracker, particles, num_turns, cache_path=None, refresh=False, probe_turns=None,
             repeats=2, space=None, timer=None, device_name=None, lattice_index=None):
    """Finds and applies the fastest tuning of ``tracker`` for tracking
    ``particles`` over ``num_turns`` turns. Returns ``(tuning, report)``;
    ``report['source']`` is 'cache' or 'search'.

    ``probe_turns`` (default ``min(num_turns, 16)``) turns are timed per
    candidate on copies of ``particles``; ``particles`` itself is not
    tracked. A ``BatchTracker`` takes the particles' ``lattice_index``.
    ``timer(tuning) -> ms`` replaces the CUDA-event timer."""
    space = dict(SPACE if space is None else space)
    key = tuning_key(tracker, particles._capacity, num_turns, device_name=device_name)
    cache = load_cache(cache_path)
    if not refresh and key in cache:
        tuning = dict(cache[key]["tuning"])
        tracker.set_tuning(**tuning)
        return tuning, {"source": "cache", "key": key, "timings": cache[key].get("timings", [])}
    if probe_turns is None:
        probe_turns = min(int(num_turns), 16)
    if timer is None:
        timer = _cuda_timer(tracker, particles, probe_turns, repeats, lattice_index)
    best = dict(tracker.get_tuning())
    timings = []
    seen = {}

    def measure(t):
        k = tuple(sorted(t.items()))
        if k not in seen:
            seen[k] = float(timer(dict(t)))
            timings.append({"tuning": dict(t), "ms": seen[k]})
        return seen[k]

    best_ms = measure(best)
    for name in ORDER:
        for v in space.get(name, ()):
            cand = dict(best)
            cand[name] = v
            ms = measure(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    tracker.set_tuning(**best)
    if cache_path:
        cache[key] = {"tuning": best, "ms": best_ms, "probe_turns": probe_turns,
                      "timings": timings}
        save_cache(cache_path, cache)
    return best, {"source": "search", "key": key, "ms": best_ms, "timings": timings}
