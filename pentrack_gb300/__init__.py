"""pentrack_gb300 -- GB300-native (sm_103a) drop-in for PENTrack's particle-tracking hot path.

The product is libpentrack_gpu.so (C ABI in include/pentrack_gpu.h): CUDA
kernels for the adaptive Dormand-Prince integration, tricubic/harmonic field
evaluation, BVH segment-mesh queries and wall physics.  This package is the
Python host binding over that ABI plus synthetic-workload helpers.
"""
from . import _abi as abi  # noqa: F401
from .engine import ConfigScene, config_run_params, Batch, Engine, EngineError, ParticleSet, Scene, lib, run_params  # noqa: F401

__all__ = ["abi", "Batch", "ConfigScene", "Engine", "EngineError", "ParticleSet", "Scene", "config_run_params", "lib", "run_params"]
