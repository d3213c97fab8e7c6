"""GB300 (sm_103a) rigid-water force/energy path of Genesis6.

The compute lives in libg6gpu.so (CUDA kernels behind the C ABI of
include/g6gpu.h).  This package is the host side: the ctypes binding, the
system owner (RigidWater), the reference-facing pair-list calls, synthetic
configurations and the build script.
"""
from . import _capi, analysis, config, formats, interaction, replicas  # noqa: F401
from ._capi import G6Error, Thermostat, lib, model_info  # noqa: F401
from .system import RigidWater  # noqa: F401

__all__ = ["RigidWater", "G6Error", "Thermostat", "lib", "model_info", "analysis", "config", "formats", "interaction",
           "replicas"]
