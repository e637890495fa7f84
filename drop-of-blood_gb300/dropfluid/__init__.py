"""dropfluid — GB300-native staggered-MAC fluid step of the drop-of-blood
simulator, driven through the C ABI of libdropfluid.so (include/dropfluid.h).

The compute path is hand-written CUDA for sm_103a; this package is the host
side: ctypes binding, the engine-style wrapper, the uniform-block packer and
the seeded benchmark scenes.
"""
from . import abi  # noqa: F401
from . import adjoint  # noqa: F401
from ._lib import DropFluidError, load  # noqa: F401
from .abi import config_closed_box, config_reference  # noqa: F401
from .engine import DropFluid, eval_math  # noqa: F401

__all__ = ["abi", "adjoint", "DropFluid", "DropFluidError", "config_closed_box", "config_reference", "eval_math", "load"]
