"""powerfit_gb300: GB300-native (sm_103a) exhaustive 6D local cross-correlation
search, a drop-in for PowerFit's correlator.

Public API
----------
``CUDACorrelator``   reference ``GPUCorrelator`` surface (setters, ``scan``, ``lcc``, ``rot``)
``PowerFitter``      reference ``PowerFitter`` surface (devices instead of OpenCL queues)
``BaseCorrelator``   reference contract (preprocessing, argument checks)
``rotations``        rotation sets (``quat_to_rotmat``, ``proportional_orientations``)
``synth``            seeded synthetic maps for tests and benchmarks
"""
from .correlator import BaseCorrelator, CUDACorrelator, PowerFitter, combine_shards, determine_core_indices

__all__ = ["BaseCorrelator", "CUDACorrelator", "PowerFitter", "combine_shards", "determine_core_indices"]
