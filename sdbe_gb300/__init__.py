"""GB300-native SWARM -> R2DBE resampling stage (drop-in for the APHIDS GPU stage).

The compute path is ``libsdbe.so`` (hand-written sm_103a CUDA, C ABI in
``include/sdbe.h``); this package is its host side.
"""
from ._native import SdbeError  # noqa: F401
from .resampler import GroupResult, Resampler, host_buffer, process_multi  # noqa: F401

__all__ = ["Resampler", "GroupResult", "SdbeError", "host_buffer", "process_multi"]
