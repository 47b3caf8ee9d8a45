"""Tracker: host side of the push (xtrack/tracker.py).

Builds the device lattice from the line's raw element records once
(replacing TrackerData + kernel compilation, tracker.py:38-147, 437-501),
and drives ``xtg_track`` with the reference's split of a run into a first
partial turn, middle turns and a last partial turn (tracker.py:1270-1436),
its monitor set-up (tracker.py:1445-1480) and its end-of-turn flags.
"""
import ctypes
import time as _time

import numpy as np
import torch

from . import _abi
from .monitors import MultiElementMonitor, ParticlesMonitor

ARITH = {"exact": _abi.ARITH_EXACT, "fast": _abi.ARITH_FAST}


class TrackFlags:
    """Runtime flag register (xtrack/track_flags.py:5-12)."""
    _bits = {"XS_FLAG_BACKTRACK": 0, "XS_FLAG_KILL_CAVITY_KICK": 2,
             "XS_FLAG_IGNORE_GLOBAL_APERTURE": 3, "XS_FLAG_IGNORE_LOCAL_APERTURE": 4,
             "XS_FLAG_SR_TAPER": 5, "XS_FLAG_SR_KICK_SAME_AS_FIRST": 6}

    def __init__(self, **kwargs):
        object.__setattr__(self, "flags", {k: False for k in self._bits})
        for k, v in kwargs.items():
            setattr(self, k, v)

    def get_flags_register(self):
        reg = 0
        for k, b in self._bits.items():
            if self.flags[k]:
                reg |= 1 << b
        return np.uint64(reg)

    def __getattr__(self, name):
        flags = object.__getattribute__(self, "flags")
        if name in flags:
            return flags[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name not in self.flags:
            raise KeyError(f"Unknown flag '{name}'")
        if name in ("XS_FLAG_SR_TAPER", "XS_FLAG_SR_KICK_SAME_AS_FIRST") and value:
            raise NotImplementedError("synchrotron-radiation flags are not supported")
        self.flags[name] = bool(value)


class Tracker:
    def __init__(self, line, device=None, arith="exact"):
        if arith not in ARITH:
            raise ValueError("arith must be 'exact' or 'fast'")
        self.line = line
        self.arith = arith
        self.device = torch.device(device) if device is not None else torch.device("cuda")
        if self.device.type != "cuda":
            raise RuntimeError("xtrack_gb300 tracks on a CUDA device only "
                               f"(got device {self.device})")
        self._lib = _abi.load_library()
        self.track_flags = TrackFlags()
        # Line.freeze_longitudinal(True): every call freezes zeta, ptau,
        # delta, rpp and rvv (the reference's FREEZE_VAR_<name> config)
        self.frozen_longitudinal = False
        self.num_elements = len(line.element_names)
        self._records = line._element_records()
        cfg = line.config
        self._cfg = _abi.XtgConfig()
        self._cfg.use_exact_drifts = 1 if cfg.XTRACK_USE_EXACT_DRIFTS else 0
        self._cfg.cavity_preserve_angle = 1 if cfg.XTRACK_CAVITY_PRESERVE_ANGLE else 0
        lim = cfg.XTRACK_GLOBAL_XY_LIMIT
        self._cfg.has_global_xy_limit = 0 if lim is None or lim is False else 1
        self._cfg.global_xy_limit = float(lim) if self._cfg.has_global_xy_limit else 0.0
        self._cfg.arith = ARITH[arith]
        self.line_length = float(line.get_length())
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _abi.check(self._lib.xtg_lattice_create(
                self._records.ctypes.data_as(ctypes.c_void_p), len(self._records),
                ctypes.byref(self._cfg), ctypes.byref(handle)), self._lib)
        self._handle = handle
        self.record_last_track = None
        self.record_multi_element_last_track = None
        self.time_last_track = None

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            try:
                self._lib.xtg_lattice_destroy(h)
            except Exception:
                pass
            self._handle = None

    # ------------------------------------------------------------------
    def flops_per_particle(self, ele_start=0, num_elements=None):
        """Canonical FP64 FLOPs one particle spends on the given elements."""
        if num_elements is None:
            num_elements = self.num_elements - ele_start
        n = ctypes.c_int64()
        f = ctypes.c_double()
        _abi.check(self._lib.xtg_lattice_info(self._handle, ctypes.byref(n), ele_start,
                                              num_elements, ctypes.byref(f)), self._lib)
        return f.value

    def get_tuning(self):
        t = _abi.XtgTuning()
        _abi.check(self._lib.xtg_get_tuning(self._handle, ctypes.byref(t)), self._lib)
        return {f: getattr(t, f) for f, _ in _abi.XtgTuning._fields_}

    def set_tuning(self, **kw):
        """block_size (32/64/128/256), compact_every (turns), chunk_bytes (0: no
        shared-memory staging), use_graph. Results do not depend on them."""
        cur = self.get_tuning()
        unknown = set(kw) - set(cur)
        if unknown:
            raise KeyError(f"unknown tuning keys {unknown}")
        cur.update(kw)
        t = _abi.XtgTuning(**{k: int(v) for k, v in cur.items()})
        _abi.check(self._lib.xtg_set_tuning(self._handle, ctypes.byref(t)), self._lib)
        return cur

    def device_status(self):
        """Synchronizes and raises if a bounded wait inside a kernel gave up."""
        _abi.check(self._lib.xtg_device_status(self._handle), self._lib)

    # ------------------------------------------------------------------
    def _get_monitor(self, particles, turn_by_turn_monitor, num_turns):
        """tracker.py:1445-1480."""
        if turn_by_turn_monitor is None or turn_by_turn_monitor is False:
            return 0, None
        if turn_by_turn_monitor is True:
            mon = ParticlesMonitor(start_at_turn=0, stop_at_turn=num_turns,
                                   particle_id_range=particles.get_active_particle_id_range(),
                                   device=particles.device)
            return 1, mon
        if turn_by_turn_monitor == "ONE_TURN_EBE":
            mon = ParticlesMonitor(start_at_turn=0, stop_at_turn=len(self.line.element_names) + 1,
                                   particle_id_range=particles.get_active_particle_id_range(),
                                   device=particles.device, ebe_mode=1)
            return 2, mon
        if isinstance(turn_by_turn_monitor, ParticlesMonitor):
            return (2 if turn_by_turn_monitor.ebe_mode == 1 else 1), turn_by_turn_monitor
        raise ValueError("Please provide a valid monitor object")

    def _set_multi_element_monitor(self, mem):
        st = self._lib.xtg_set_multi_element_monitor(
            self._handle, ctypes.byref(mem._xtg_struct()) if mem is not None else None)
        _abi.check(st, self._lib)

    def _launch(self, pstruct, num_turns, ele_start, num_ele_track, flag_end, flag_monitor,
                mstruct, flags, stream):
        st = self._lib.xtg_track(
            self._handle, ctypes.byref(pstruct), int(num_turns), int(ele_start),
            int(num_ele_track), int(flag_end), int(1 if self.line.reset_s_at_end_turn else 0),
            int(flag_monitor), int(self.num_elements), self.line_length,
            ctypes.byref(mstruct) if mstruct is not None else None,
            int(flags), ctypes.c_void_p(stream))
        _abi.check(st, self._lib)

    def _get_multi_element_monitor(self, multi_element_monitor_at, particles, num_turns):
        """tracker.py:1482-1525."""
        if multi_element_monitor_at is None or len(multi_element_monitor_at) == 0:
            return None
        names = list(self.line.element_names)
        if isinstance(multi_element_monitor_at, str):
            if multi_element_monitor_at != "_all_":
                raise ValueError("multi_element_monitor_at must be a list of names or '_all_'")
            multi_element_monitor_at = names
        index = {n: i for i, n in reversed(list(enumerate(names)))}
        missing = [n for n in multi_element_monitor_at if n not in index]
        if missing:
            raise ValueError(f"Elements not found in line: {set(missing)}")
        obs = [index[n] for n in multi_element_monitor_at]
        mapping = np.full(len(names) + 1, -1, dtype=np.int64)
        mapping[obs] = np.arange(len(obs), dtype=np.int64)
        start, end = particles.get_active_particle_id_range()
        return MultiElementMonitor(start_at_turn=0, stop_at_turn=num_turns or 1,
                                   part_id_start=start, part_id_end=end,
                                   at_element_mapping=mapping,
                                   obs_names=[names[i] for i in obs], device=particles.device)

    def _track(self, particles, ele_start=0, ele_stop=None, num_elements=None, num_turns=None,
               turn_by_turn_monitor=None, freeze_longitudinal=False, time=False,
               with_progress=False, backtrack=False, _force_no_end_turn_actions=False,
               multi_element_monitor_at=None):
        if particles.device.type != "cuda":
            raise RuntimeError("particles must live on a CUDA device")
        if with_progress:
            return self._track_with_progress(particles, ele_start, ele_stop, num_elements,
                                             num_turns, turn_by_turn_monitor, time,
                                             with_progress, backtrack, freeze_longitudinal)
        t0 = None
        if time:
            torch.cuda.synchronize(particles.device)
            t0 = _time.perf_counter()

        if particles.start_tracking_at_element >= 0:
            if ele_start != 0:
                raise ValueError("The argument ele_start is used, but "
                                 "particles.start_tracking_at_element is set as well.")
            ele_start = particles.start_tracking_at_element
            particles.start_tracking_at_element = -1
        if isinstance(ele_start, str):
            ele_start = self.line.element_names.index(ele_start)
        if ele_start is None:
            ele_start = 0
        if not (0 <= ele_start <= self.num_elements):
            raise ValueError("ele_start out of range")
        L = self.num_elements

        # tracker.py:1270-1333
        num_middle_turns = 0
        num_elements_last_turn = 0
        if num_elements is not None:
            if num_elements < 0:
                raise ValueError("num_elements must be >= 0")
            if ele_stop is not None:
                raise ValueError("Cannot use both num_elements and ele_stop!")
            if num_turns is not None:
                raise ValueError("Cannot use both num_elements and num_turns!")
            if num_elements + ele_start <= L:
                num_elements_first_turn = num_elements
            else:
                num_elements_first_turn = L - ele_start
                num_middle_turns, ele_stop = divmod(ele_start + num_elements, L)
                num_elements_last_turn = ele_stop
                num_middle_turns -= 1
        else:
            if num_turns is None:
                num_turns = 1
            elif num_turns <= 0:
                raise ValueError("num_turns must be > 0")
            if ele_stop is None:
                num_elements_first_turn = L - ele_start
                num_middle_turns = num_turns - 1
            else:
                if isinstance(ele_stop, str):
                    ele_stop = self.line.element_names.index(ele_stop)
                if not (0 <= ele_stop <= L):
                    raise ValueError("ele_stop out of range")
                if ele_stop <= ele_start:
                    num_turns += 1
                if num_turns == 1:
                    num_elements_first_turn = ele_stop - ele_start
                else:
                    num_elements_first_turn = L - ele_start
                    num_middle_turns = num_turns - 2
                    num_elements_last_turn = ele_stop

        if self.line.skip_end_turn_actions or _force_no_end_turn_actions:
            flag_end_first, flag_end_middle = False, False
        else:
            flag_end_first = (num_elements_first_turn + ele_start == L)
            flag_end_middle = True

        monitor_turns = num_middle_turns + (2 if num_elements_last_turn > 0 else 1)
        flag_monitor, monitor = self._get_monitor(particles, turn_by_turn_monitor, monitor_turns)
        mstruct = monitor._xtg_struct() if monitor is not None else None

        flags = self.track_flags.get_flags_register()
        if backtrack:
            flags = np.uint64(int(flags) | (1 << _abi.FLAG_BACKTRACK))
        if freeze_longitudinal or self.frozen_longitudinal:
            flags = np.uint64(int(flags) | (1 << _abi.FLAG_FREEZE_LONGITUDINAL))

        mem = self._get_multi_element_monitor(multi_element_monitor_at, particles, monitor_turns)
        pstruct = particles._xtg_struct()
        stream = torch.cuda.current_stream(particles.device).cuda_stream
        with torch.cuda.device(particles.device):
            if mem is not None:
                self._set_multi_element_monitor(mem)
            try:
                if (ele_start == 0 and num_elements_first_turn == L and flag_end_first == flag_end_middle
                        and num_middle_turns > 0):
                    # the first turn is a whole turn with the middle turns'
                    # arguments: one call, the same result (the reference's
                    # split exists for a partial first turn), and a turn-by-
                    # turn monitor's records of a particle are written in one
                    # pass instead of two
                    self._launch(pstruct, 1 + num_middle_turns, 0, L, flag_end_middle, flag_monitor,
                                 mstruct, flags, stream)
                else:
                    self._launch(pstruct, 1, ele_start, num_elements_first_turn, flag_end_first,
                                 flag_monitor, mstruct, flags, stream)
                    if num_middle_turns > 0:
                        self._launch(pstruct, num_middle_turns, 0, L, flag_end_middle, flag_monitor,
                                     mstruct, flags, stream)
                if num_elements_last_turn > 0:
                    self._launch(pstruct, 1, 0, num_elements_last_turn, False, flag_monitor,
                                 mstruct, flags, stream)
            finally:
                if mem is not None:
                    self._set_multi_element_monitor(None)

        self.record_last_track = monitor
        self.record_multi_element_last_track = mem
        if time:
            torch.cuda.synchronize(particles.device)
            self.time_last_track = _time.perf_counter() - t0
        return None

    def _track_with_progress(self, particles, ele_start, ele_stop, num_elements, num_turns,
                             turn_by_turn_monitor, time, with_progress, backtrack,
                             freeze_longitudinal=False):
        """tracker.py:313-381: batches of turns, same result as one call."""
        if turn_by_turn_monitor not in (None, False):
            raise NotImplementedError("with_progress together with a monitor is not supported")
        if num_elements is not None or ele_stop is not None:
            raise NotImplementedError("with_progress supports whole turns only")
        batch = 100 if with_progress is True else int(with_progress)
        num_turns = 1 if num_turns is None else num_turns
        t0 = _time.perf_counter()
        done = 0
        first = True
        while done < num_turns:
            n = min(batch, num_turns - done)
            self._track(particles, ele_start=ele_start if first else 0, num_turns=n,
                        backtrack=backtrack, freeze_longitudinal=freeze_longitudinal)
            first = False
            done += n
        if time:
            torch.cuda.synchronize(particles.device)
            self.time_last_track = _time.perf_counter() - t0
