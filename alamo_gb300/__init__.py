"""alamo_gb300 — alamo's nodal linear-elastic multigrid path on GB300.

The CUDA library ``_build/libagb.so`` (C ABI: include/agb.h) is the product;
this package is its host-side mirror of the reference's Operator::Elastic /
Solver::Nonlocal::Linear / Newton interface plus the benchmark inputs.
"""
from . import bc, synth  # noqa: F401
from ._lib import LIB_PATH, AgbError, lib, last_error  # noqa: F401
from .elastic import DevicePtr, Elastic, Linear, Newton, default_opts  # noqa: F401

__all__ = ["bc", "synth", "Elastic", "Linear", "Newton", "DevicePtr", "default_opts", "lib", "AgbError",
           "LIB_PATH", "last_error"]
