"""streamsculptor_gb300 — GB300-native (sm_103a) stream generation.

Drop-in for the hot path of jnibauer/streamsculptor: potential classes,
integrate_orbit, gen_stream_*, fields.integrate_field and the perturbation
generators, backed by hand-written CUDA kernels behind a C ABI
(include/streamsculptor_gb300.h, libssgb300.so).  As in the reference,
`main` and `streamhelpers` are flattened into the package namespace and
`potential`, `fields`, `perturbative` are submodules.
"""
from .main import *  # noqa: F401,F403
from .streamhelpers import *  # noqa: F401,F403
from . import potential, fields, perturbative  # noqa: F401
from ._core import CenterTrack  # noqa: F401

__version__ = "0.1.0"
