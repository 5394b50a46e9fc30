"""Inverse polyphase filter bank for PFB-mode SWARM spectra (over the C ABI).

``inverse_pfb`` is the device counterpart of the least-squares inversion set
up in software/prototyping/cuda/pfb_inverse.cu:213-488 (Shaw's method): the
time blocks whose 4-tap Hamming PFB gives the spectra.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .resampler import _addr, _is_device


def inverse_pfb(rs, spec, ntap: int = 4, out=None, stream=None):
    """``spec``: complex64 ``[nblock, 16385]`` on the device (torch CUDA
    tensor or raw address with ``nblock`` given by its shape).  Returns the
    float32 time blocks ``[nblock + ntap - 1, 32768]`` (a torch tensor when
    ``out`` is not given).  Without ``stream`` the call runs on the handle's
    stream and returns when the blocks are ready."""
    import torch

    if not _is_device(spec):
        spec = torch.from_numpy(np.ascontiguousarray(spec, np.complex64)).cuda()
    nblock = int(spec.shape[0])
    if out is None:
        out = torch.empty((nblock + ntap - 1, 2 * (N.CHANNELS)), dtype=torch.float32, device=spec.device)
    st = None if stream is None else C.c_void_p(stream if isinstance(stream, int) else stream.cuda_stream)
    N.check(N.lib().sdbe_inverse_pfb(rs.handle, _addr(spec), nblock, ntap, _addr(out), st), rs.handle)
    if stream is None:  # the handle's stream: wait, so the result is ready for any torch stream
        rs.sync()
    return out
