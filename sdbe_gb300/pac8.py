"""Ingest transforms for SWARM's 8pac output (over the C ABI).

``unpack_8pac`` and ``beng_reform`` are the device counterparts of
``unpack_8pac`` (software/aphids/vdif_8pac.c:47-56) and
``beng_reform_headers`` (software/aphids/beng_reform.c:137-186); the
reference's file-scope T0/TPREV/BPREV become an explicit ``ReformState``.
Buffers are device memory: torch CUDA tensors or raw addresses.
"""
from __future__ import annotations

import ctypes as C

from . import _native as N
from .resampler import _addr


def _stream(stream):
    if stream is None:
        return None
    return C.c_void_p(stream if isinstance(stream, int) else stream.cuda_stream)


def new_state() -> N.ReformState:
    st = N.ReformState()
    N.check(N.lib().sdbe_reform_init(C.byref(st)))
    return st


def unpack_8pac(src, n_units: int, dst, stream=None):
    """n_units 8504-B units at ``src`` -> 8*n_units 1056-B packets at ``dst``."""
    N.check(N.lib().sdbe_unpack_8pac(_addr(src), n_units, _addr(dst), _stream(stream)))


def beng_reform(state: N.ReformState, pkts, n_pkts: int, stream=None) -> N.ReformState:
    """Rewrite new-format headers of ``n_pkts`` packets in place; updates and
    returns ``state`` (the call synchronizes the stream)."""
    N.check(N.lib().sdbe_beng_reform(C.byref(state), _addr(pkts), n_pkts, _stream(stream)))
    return state
