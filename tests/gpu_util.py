"""Helpers for the GPU tests: device buffers through torch, C-ABI calls."""
import ctypes as C

import numpy as np

from oracle import sdbe_oracle as O


def torch_mod():
    import torch

    return torch


def dev(arr: np.ndarray):
    torch = torch_mod()
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def empty(nbytes: int, dtype="uint8"):
    torch = torch_mod()
    dt = {"uint8": torch.uint8, "float32": torch.float32, "int32": torch.int32, "int8": torch.int8}[dtype]
    itemsize = torch.tensor([], dtype=dt).element_size()
    return torch.empty(nbytes // itemsize, dtype=dt, device="cuda")


def zeros(nbytes: int, dtype="uint8"):
    t = empty(nbytes, dtype)
    t.zero_()
    return t


def ptr(t) -> int:
    return int(t.data_ptr())


def host(t) -> np.ndarray:
    torch_mod().cuda.synchronize()
    return t.cpu().numpy()


def rel_rms(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(np.mean((got - ref) ** 2) / np.mean(ref ** 2)))


def crel_rms(got, ref):
    got = np.asarray(got, np.complex128)
    ref = np.asarray(ref, np.complex128)
    return float(np.sqrt(np.mean(np.abs(got - ref) ** 2) / np.mean(np.abs(ref) ** 2)))


def codes_of(payload_bytes: np.ndarray) -> np.ndarray:
    return O.unpack2bit(np.ascontiguousarray(payload_bytes).reshape(-1).view("<u4"))


def packed_to_complex(words: np.ndarray) -> np.ndarray:
    """Packed nibble spectra [n, 2048] u32 -> complex [n, 16385] (Nyquist 0)."""
    w = np.asarray(words, np.uint32)
    nib = (w[..., None] >> (4 * np.arange(8, dtype=np.uint32))) & 0xF
    nib = nib.reshape(w.shape[0], -1)
    re = (nib >> 2).astype(np.float64) - 2
    im = (nib & 3).astype(np.float64) - 2
    out = np.zeros((w.shape[0], O.BENG_CHANNELS), np.complex128)
    out[:, :O.BENG_CHANNELS_] = re + 1j * im
    return out
