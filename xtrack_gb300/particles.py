"""Particles structure-of-arrays held as PyTorch tensors.

Mirrors ``xtrack.Particles`` (xtrack/particles/particles.py): the same
per-particle fields (particles.py:26-83), the same constructor keywords and
the same derivation of the energy variables (particles.py:1900-2069), so a
script that builds ``xt.Particles(p0c=..., x=..., delta=...)`` builds the
same numbers here. Arrays live on one torch device; the CUDA push borrows
their device pointers.
"""
import numpy as np
import torch

from . import _abi

PROTON_MASS_EV = 938272088.16        # particles/masses.py:12 (PDG 2024)
ELECTRON_MASS_EV = 510998.95         # particles/masses.py:8
LAST_INVALID_STATE = -999999999      # particles.py:24
CLIGHT = 299792458.0

DOUBLE_FIELDS = (
    "p0c", "gamma0", "beta0", "s", "zeta", "x", "y", "px", "py",
    "ptau", "delta", "rpp", "rvv", "chi", "charge_ratio", "weight",
    "ax", "ay", "spin_x", "spin_y", "spin_z", "anomalous_magnetic_moment")
INT_FIELDS = ("pdg_id", "particle_id", "at_element", "at_turn", "state", "parent_particle_id")
PER_PARTICLE_FIELDS = DOUBLE_FIELDS + INT_FIELDS
SCALAR_FIELDS = ("q0", "mass0", "t_sim")

_ACCEPTED = set(PER_PARTICLE_FIELDS) | set(SCALAR_FIELDS) | {
    "energy0", "tau", "pzeta", "mass_ratio", "kinetic_energy0", "rigidity0",
    "start_tracking_at_element", "name"}


def default_device():
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


class Particles:
    """Structure of arrays of particle coordinates (see xtrack.Particles).

    Parameters follow xtrack: ``x, px, y, py, zeta, delta`` (or ``ptau`` /
    ``pzeta``), reference ``p0c`` (or ``energy0``, ``gamma0``, ``beta0``,
    ``kinetic_energy0``, ``rigidity0``), ``mass0`` [eV], ``q0`` [e],
    ``chi``/``charge_ratio``/``mass_ratio``, ``s``, ``at_turn``,
    ``at_element``, ``state``, ``particle_id``, ``weight``. Scalars broadcast.
    ``_capacity`` reserves extra slots (state LAST_INVALID_STATE).
    ``device`` selects the torch device (default: cuda when available).
    """

    def __init__(self, _capacity=None, device=None, _no_reorganize=False, **kwargs):
        unknown = set(kwargs) - _ACCEPTED
        if unknown:
            raise NameError(f"Invalid argument(s) provided: {unknown}")
        self.device = torch.device(device) if device is not None else default_device()

        # number of particles from the array-valued inputs (particles.py:609-623)
        input_length = 1
        for name, val in kwargs.items():
            if name in SCALAR_FIELDS or name in ("start_tracking_at_element", "name"):
                continue
            if np.isscalar(val) or np.ndim(val) == 0 or len(val) == 1:
                continue
            if len(val) != input_length and input_length > 1:
                raise ValueError("All per particle vars have to be of the same length.")
            input_length = len(val)
        if _capacity is None:
            _capacity = input_length
        if _capacity <= 0:
            raise ValueError("Explicitly provided `_capacity` has to be greater than zero.")
        if _capacity < input_length:
            raise ValueError(f"Capacity ({_capacity}) has to be greater or equal to the "
                             f"number of particles ({input_length}).")
        n = input_length
        self._capacity = int(_capacity)

        arr = {}
        for f in DOUBLE_FIELDS:
            arr[f] = np.full(_capacity, float(LAST_INVALID_STATE), dtype=np.float64)
        for f in INT_FIELDS:
            arr[f] = np.full(_capacity, LAST_INVALID_STATE, dtype=np.int64)

        def vec(val, dtype=np.float64):
            a = np.asarray(val, dtype=dtype)
            if a.ndim == 0 or a.size == 1:
                return np.full(n, a.reshape(-1)[0] if a.ndim else a.item(), dtype=dtype)
            return a.astype(dtype)

        arr["state"][:n] = vec(kwargs.get("state", 1), np.int64)
        pid = vec(kwargs.get("particle_id", np.arange(n)), np.int64)
        arr["particle_id"][:n] = pid
        arr["parent_particle_id"][:n] = vec(kwargs.get("parent_particle_id", pid), np.int64)

        self.q0 = float(kwargs.get("q0", 1.0))
        self.mass0 = float(kwargs.get("mass0", PROTON_MASS_EV))
        self.t_sim = float(kwargs.get("t_sim", 0.0))
        self.start_tracking_at_element = int(kwargs.get("start_tracking_at_element", -1))

        # init_independent_per_part_vars (particles.py:1805-1832)
        for f, d in (("s", 0), ("at_turn", 0), ("at_element", 0), ("weight", 1), ("x", 0),
                     ("y", 0), ("px", 0), ("py", 0), ("ax", 0), ("ay", 0),
                     ("anomalous_magnetic_moment", 0), ("spin_x", 0), ("spin_y", 0),
                     ("spin_z", 0), ("pdg_id", 0)):
            dtype = np.int64 if f in INT_FIELDS else np.float64
            arr[f][:n] = vec(kwargs.get(f, d), dtype)

        # _update_chi_charge_ratio (particles.py:2032-2069)
        chi, cr, mr = kwargs.get("chi"), kwargs.get("charge_ratio"), kwargs.get("mass_ratio")
        nargs = sum(v is not None for v in (chi, cr, mr))
        if nargs == 0:
            arr["chi"][:n] = 1.0
            arr["charge_ratio"][:n] = 1.0
        elif nargs == 1:
            raise ValueError("Two of `chi`, `charge_ratio` and `mass_ratio` must be provided.")
        else:
            if chi is None:
                arr["charge_ratio"][:n] = vec(cr)
                arr["chi"][:n] = vec(cr) / vec(mr)
            elif cr is None:
                arr["chi"][:n] = vec(chi)
                arr["charge_ratio"][:n] = vec(chi) * vec(mr)
            else:
                arr["chi"][:n] = vec(chi)
                arr["charge_ratio"][:n] = vec(cr)

        # _update_refs (particles.py:1900-1954)
        mass0 = self.mass0
        p0c, energy0 = kwargs.get("p0c"), kwargs.get("energy0")
        gamma0, beta0 = kwargs.get("gamma0"), kwargs.get("beta0")
        ek0, rig0 = kwargs.get("kinetic_energy0"), kwargs.get("rigidity0")
        if all(v is None for v in (p0c, energy0, gamma0, beta0, ek0, rig0)):
            p0c = 1e9
        if p0c is not None:
            _p0c = vec(p0c)
            _energy0 = np.sqrt(_p0c ** 2 + mass0 ** 2)
            _beta0 = _p0c / _energy0
            _gamma0 = _energy0 / mass0
        elif energy0 is not None:
            _energy0 = vec(energy0)
            _p0c = np.sqrt(_energy0 ** 2 - mass0 ** 2)
            _beta0 = _p0c / _energy0
            _gamma0 = _energy0 / mass0
        elif gamma0 is not None:
            _gamma0 = vec(gamma0)
            _beta0 = np.sqrt(1 - 1 / _gamma0 ** 2)
            _energy0 = mass0 * _gamma0
            _p0c = _energy0 * _beta0
        elif beta0 is not None:
            _beta0 = vec(beta0)
            _gamma0 = 1 / np.sqrt(1 - _beta0 ** 2)
            _energy0 = mass0 * _gamma0
            _p0c = _energy0 * _beta0
        elif ek0 is not None:
            _energy0 = vec(ek0) + mass0
            _p0c = np.sqrt(_energy0 ** 2 - mass0 ** 2)
            _beta0 = _p0c / _energy0
            _gamma0 = _energy0 / mass0
        else:
            _p0c = vec(rig0) * abs(self.q0) * CLIGHT
            _energy0 = np.sqrt(_p0c ** 2 + mass0 ** 2)
            _beta0 = _p0c / _energy0
            _gamma0 = _energy0 / mass0
        arr["p0c"][:n] = _p0c
        arr["beta0"][:n] = _beta0
        arr["gamma0"][:n] = _gamma0

        # _update_energy_deviations (particles.py:1956-2008)
        b0 = arr["beta0"][:n]
        delta, ptau, pzeta = kwargs.get("delta"), kwargs.get("ptau"), kwargs.get("pzeta")
        if all(v is None for v in (delta, ptau, pzeta)):
            mass_ratio = arr["charge_ratio"][:n] / arr["chi"][:n]
            if np.any(mass_ratio != 1.0):
                raise ValueError("Need to provide `delta` or `ptau` with non-default mass ratios.")
            delta = 0.0
        if delta is not None:
            _delta = vec(delta)
            _ptau = np.sqrt(_delta ** 2 + 2 * _delta + 1 / b0 ** 2) - 1 / b0
        elif ptau is not None:
            _ptau = vec(ptau)
            _delta = np.sqrt(_ptau ** 2 + 2 * _ptau / b0 + 1) - 1
        else:
            _ptau = vec(pzeta) * b0
            _delta = np.sqrt(_ptau ** 2 + 2 * _ptau / b0 + 1) - 1
        arr["delta"][:n] = _delta
        arr["ptau"][:n] = _ptau
        delta_beta0 = _delta * b0
        ptau_beta0 = np.sqrt(delta_beta0 ** 2 + 2 * delta_beta0 * b0 + 1) - 1
        arr["rvv"][:n] = (1 + _delta) / (1 + ptau_beta0)
        arr["rpp"][:n] = 1 / (1 + _delta)

        # _update_zeta (particles.py:2010-2030)
        zeta, tau = kwargs.get("zeta"), kwargs.get("tau")
        if zeta is not None:
            arr["zeta"][:n] = vec(zeta)
        elif tau is not None:
            arr["zeta"][:n] = b0 * vec(tau)
        else:
            arr["zeta"][:n] = 0.0

        self._set_arrays(arr)
        if "name" in kwargs:
            self.name = kwargs["name"]

    # ------------------------------------------------------------------
    def _set_arrays(self, arr):
        for f in PER_PARTICLE_FIELDS:
            t = torch.from_numpy(np.ascontiguousarray(arr[f])).to(self.device)
            object.__setattr__(self, "_t_" + f, t)

    def __getattr__(self, name):
        if name in PER_PARTICLE_FIELDS:
            return object.__getattribute__(self, "_t_" + name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in PER_PARTICLE_FIELDS:
            t = object.__getattribute__(self, "_t_" + name)
            if torch.is_tensor(value):
                t.copy_(value.to(t.dtype))
            else:
                t.copy_(torch.as_tensor(np.asarray(value), dtype=t.dtype).to(t.device).expand_as(t))
            return
        object.__setattr__(self, name, value)

    # ------------------------------------------------------------------
    @property
    def energy0(self):
        return torch.sqrt(self.p0c ** 2 + self.mass0 ** 2)

    @property
    def mass_ratio(self):
        return self.charge_ratio / self.chi

    @property
    def mass(self):
        return self.mass_ratio * self.mass0

    @property
    def energy(self):
        return self.energy0 + self.ptau * self.p0c

    @property
    def pzeta(self):
        return self.ptau / self.beta0

    @property
    def tau(self):
        return self.zeta / self.beta0

    @property
    def _num_active_particles(self):
        return int((self.state > 0).sum().item())

    @property
    def _num_lost_particles(self):
        return int(((self.state <= 0) & (self.state > LAST_INVALID_STATE)).sum().item())

    def get_active_particle_id_range(self):
        """Range (python-style, end exclusive) of ids of active particles
        (particles.py:1340-1348)."""
        mask = self.state > 0
        ids = self.particle_id[mask]
        return int(ids.min().item()), int(ids.max().item()) + 1

    def reorganize(self):
        """Moves active particles first, then lost, then unallocated slots
        (particles.py:1198-1259). Returns (n_active, n_lost)."""
        st = self.state
        key = torch.where(st > 0, 0, torch.where(st > LAST_INVALID_STATE, 1, 2))
        order = torch.sort(key, stable=True).indices
        for f in PER_PARTICLE_FIELDS:
            t = object.__getattribute__(self, "_t_" + f)
            t.copy_(t[order])
        return self._num_active_particles, self._num_lost_particles

    def copy(self, device=None):
        out = object.__new__(Particles)
        object.__setattr__(out, "device", torch.device(device) if device is not None else self.device)
        for k in ("_capacity", "q0", "mass0", "t_sim", "start_tracking_at_element"):
            object.__setattr__(out, k, getattr(self, k))
        for f in PER_PARTICLE_FIELDS:
            t = object.__getattribute__(self, "_t_" + f)
            object.__setattr__(out, "_t_" + f, t.to(out.device).clone())
        return out

    def to_dict(self):
        out = {f: object.__getattribute__(self, "_t_" + f).cpu().numpy().copy()
               for f in PER_PARTICLE_FIELDS}
        for k in SCALAR_FIELDS:
            out[k] = getattr(self, k)
        out["_capacity"] = self._capacity
        out["start_tracking_at_element"] = self.start_tracking_at_element
        return out

    @classmethod
    def from_dict(cls, dct, device=None):
        out = object.__new__(cls)
        object.__setattr__(out, "device", torch.device(device) if device is not None else default_device())
        cap = len(dct["x"])
        object.__setattr__(out, "_capacity", cap)
        object.__setattr__(out, "q0", float(dct.get("q0", 1.0)))
        object.__setattr__(out, "mass0", float(dct.get("mass0", PROTON_MASS_EV)))
        object.__setattr__(out, "t_sim", float(dct.get("t_sim", 0.0)))
        object.__setattr__(out, "start_tracking_at_element", int(dct.get("start_tracking_at_element", -1)))
        arr = {}
        for f in DOUBLE_FIELDS:
            arr[f] = np.asarray(dct.get(f, np.zeros(cap)), dtype=np.float64)
        for f in INT_FIELDS:
            arr[f] = np.asarray(dct.get(f, np.zeros(cap, dtype=np.int64)), dtype=np.int64)
        out._set_arrays(arr)
        return out

    def to_numpy(self):
        """Dict of host numpy copies of every per-particle array."""
        return {f: object.__getattribute__(self, "_t_" + f).cpu().numpy() for f in PER_PARTICLE_FIELDS}

    # ------------------------------------------------------------------
    def _xtg_struct(self):
        """C-ABI view (XtgParticles) of the arrays; they must be contiguous."""
        ptrs = {}
        for f in _abi.PARTICLE_DOUBLE_FIELDS + _abi.PARTICLE_INT_FIELDS:
            t = object.__getattribute__(self, "_t_" + f)
            if not t.is_contiguous():
                raise ValueError(f"particle array {f} is not contiguous")
            ptrs[f] = t.data_ptr()
        return _abi.particles_struct_from_ptrs(self._capacity, self.q0, self.mass0, self.t_sim, ptrs)

    def __len__(self):
        return self._capacity

    def __repr__(self):
        return (f"Particles(capacity={self._capacity}, active={self._num_active_particles}, "
                f"device={self.device})")
