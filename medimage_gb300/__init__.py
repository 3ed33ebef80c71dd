"""medimage_gb300 -- GB300-native Ambrosio-Tortorelli CT reconstruction engine.

Python host bindings over the C-ABI of ``include/at_engine.h`` and the GoldenC
drop-in symbols of ``include/goldnc.h``, both exported by the in-tree
``medimage_gb300/libat_engine.so`` (built by ``medimage_gb300/build.py``).

There is no CPU fallback: every call goes to the CUDA library, and importing
the bindings raises if the library is missing.
"""
from __future__ import annotations

from .engine import (  # noqa: F401
    AtError,
    ConeGeometry,
    FanGeometry,
    RayGeometry,
    RowAction,
    RowActionParams,
    Params,
    Plan,
    ProjSet,
    Server,
    Solver,
    device_info,
    lib,
    quality,
    reconstruct,
    set_batch_launch_mode,
)
from . import configs, io, phantom  # noqa: F401

__all__ = [
    "AtError",
    "ConeGeometry",
    "FanGeometry",
    "RayGeometry",
    "RowAction",
    "RowActionParams",
    "Params",
    "Plan",
    "ProjSet",
    "Server",
    "Solver",
    "configs",
    "io",
    "device_info",
    "lib",
    "phantom",
    "quality",
    "reconstruct",
    "set_batch_launch_mode",
]
