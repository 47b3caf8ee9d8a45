"""xtrack_gb300: GB300-native particle push with xtrack's Line.track API.

``import xtrack_gb300 as xt`` gives ``xt.Line``, ``xt.Particles``, the
in-scope beam elements, ``xt.ParticlesMonitor`` and the slicing schemes.
Tracking runs hand-written FP64 CUDA kernels for sm_103a through the C-ABI
library ``libxtrack_gb300.so`` (see include/xtrack_gb300.h).
"""
from .particles import Particles, PROTON_MASS_EV, ELECTRON_MASS_EV, LAST_INVALID_STATE
from .elements import (Marker, Drift, Multipole, Bend, Quadrupole, Sextupole, Octupole,
                       Cavity, LimitEllipse, LimitRect, LimitRectEllipse, LimitPolygon, DipoleEdge,
                       BeamElement)
from .elements import *  # noqa: F401,F403  (slice classes)
from .monitors import (ParticlesMonitor, LastTurnsMonitor, BeamPositionMonitor, BeamSizeMonitor,
                       BeamProfileMonitor, MultiElementMonitor)
from .slicing import Strategy, Teapot, Uniform
from .line import Line, TrackerConfig, freeze_longitudinal
from .tracker import Tracker, TrackFlags
from .batch import BatchTracker
from .tuning import autotune
from .serialization import load

__version__ = "0.1.0"
