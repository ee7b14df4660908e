"""GB300-native MNAD modeling / RTM hot path (Python front end of libmnad.so).

* :mod:`mnad.reference_api` -- ``fwd_PDE_exact_MNAD`` / ``Born_adj_MNAD`` with
  the reference MATLAB signatures.
* :mod:`mnad.api` -- contexts, stored wavefields, batched plans.
* :mod:`mnad.workflow` -- seeded synthetic models and acquisition for the
  benchmark configurations.
* :mod:`mnad.build` -- the nvcc build recipe of the library.
"""
from ._lib import MnadError, lib  # noqa: F401
from .api import Context, Plan, Server, ShotJob  # noqa: F401
from .reference_api import Born_adj_MNAD, fwd_PDE_exact_MNAD  # noqa: F401
from . import drivers  # noqa: F401,E402

__all__ = ["Context", "Plan", "Server", "ShotJob", "MnadError", "fwd_PDE_exact_MNAD", "Born_adj_MNAD", "lib"]
