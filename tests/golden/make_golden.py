"""Generate golden fixtures by running the reference's own Python code.

Run where a Smithsonian/sdbe checkout exists, with ``SDBE_REFERENCE`` set to
it (``SDBE_REFERENCE=<checkout> python tests/golden/make_golden.py``); the
fixtures it writes are committed so tests never need the reference at run
time.

The reference prototypes are Python 2.  They are loaded here unchanged except
for one exact semantic shim: every ``/`` becomes ``_py2div(a, b)``, which is
Python 2's division (floor division when both operands are integers, true
division otherwise).  Two helpers emulate the numpy of that era where the code
relies on it (float shapes accepted by ``zeros``).  Fixtures produced:

* ``dbe_frame_decode.npz``  -- ``swarm.DBEFrame.from_bin`` on seeded B-engine
  packets: c, f, b and the complex samples of p0/p1 for channels 0..7
  (``prototyping/swarm.py:36-66``, ``prototyping/vdif.py:182-211``).
* ``quantize_pack.npz``     -- ``sdbe_preprocess.quantize_to_2bit``
  (``prototyping/sdbe_preprocess.py:668-692``) then ``vdif.VDIFFrame.to_bin``
  (``prototyping/vdif.py:98-141,213-242``): codes, payload and header bytes.
* ``reorder_mar2015.npz``   -- the numpy check of the Mar-2015 reorder,
  statements of ``prototyping/cuda/reorder.py:284-293`` run on seeded data.
* ``fft_resample_2496.npz`` -- the numpy check of the batched FFT resampler,
  statements of ``prototyping/cuda/resample.py:130-134`` (39 snapshots,
  2496 -> 4096 MS/s, zero-pad), a strided sample of the result and its
  checksum; the reference compares cuFFT output divided by
  ``cpu_C.shape[-1]*2*BENG_CHANNELS_`` against it (``resample.py:138``).
"""
from __future__ import annotations

import ast
import os
import sys
import types

import numpy as np

REF = os.environ.get("SDBE_REFERENCE", "")
PROTO = os.path.join(REF, "software", "prototyping")
OUT = os.path.dirname(os.path.abspath(__file__))


def _py2div(a, b):
    ints = (int, np.integer)
    if isinstance(a, ints) and isinstance(b, ints) and not isinstance(a, bool):
        return a // b
    return a / b


class _Py2Div(ast.NodeTransformer):
    def visit_BinOp(self, node):
        self.generic_visit(node)
        if isinstance(node.op, ast.Div):
            return ast.copy_location(
                ast.Call(func=ast.Name(id="_py2div", ctx=ast.Load()),
                         args=[node.left, node.right], keywords=[]), node)
        return node


def load_py2_module(path: str, name: str):
    src = open(path).read()
    tree = ast.fix_missing_locations(_Py2Div().visit(ast.parse(src, path)))
    mod = types.ModuleType(name)
    mod.__file__ = path
    mod.__dict__["_py2div"] = _py2div
    sys.modules[name] = mod
    exec(compile(tree, path, "exec"), mod.__dict__)
    return mod


def extract_function(path: str, fname: str, env: dict):
    tree = ast.parse(open(path).read(), path)
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == fname:
            m = ast.fix_missing_locations(_Py2Div().visit(ast.Module(body=[node], type_ignores=[])))
            env.setdefault("_py2div", _py2div)
            exec(compile(m, path, "exec"), env)
            return env[fname]
    raise KeyError(fname)


def extract_statements(path: str, first: int, last: int):
    """Compile source lines [first, last] of a file on their own.

    The rest of these prototype files holds Python 2 ``print`` statements, so
    only the cited lines are parsed.  Indented lines (inside a function body)
    are wrapped in ``if True:`` so their own indentation is kept.
    """
    lines = open(path).read().splitlines(keepends=True)[first - 1:last]
    src = "".join(lines)
    if lines and lines[0][:1] in (" ", "\t"):
        src = "if True:\n" + src
    tree = ast.fix_missing_locations(_Py2Div().visit(ast.parse(src, path)))
    return compile(tree, path, "exec")


def make_beng_packets(rng, n):
    words = rng.integers(0, 2**32, size=(n, 264), dtype=np.uint64).astype(np.uint32)
    c = rng.integers(0, 256, n)
    f = rng.integers(0, 8, n)
    b = rng.integers(0, 2**40, n, dtype=np.int64)
    words[:, 0] &= 0x3FFFFFFF  # valid, non-legacy
    words[:, 2] = (words[:, 2] & ~np.uint32(0xFFFFFF)) | np.uint32(1056 // 8)
    words[:, 3] = (words[:, 3] & ~np.uint32(0x7C000000)) | np.uint32(1 << 26)  # 2 bits/sample
    words[:, 4] = (b >> 8).astype(np.uint32)
    words[:, 5] = (c | (rng.integers(0, 256, n) << 8) | (f << 16) | ((b & 0xFF) << 24)).astype(np.uint32)
    return words.view(np.uint8).reshape(n, 1056)


def golden_dbe_frame(rng):
    load_py2_module(os.path.join(PROTO, "vdif.py"), "vdif")
    swarm = load_py2_module(os.path.join(PROTO, "swarm.py"), "swarm")
    pk = make_beng_packets(rng, 24)
    cs, fs, bs = [], [], []
    p0 = np.zeros((len(pk), 8, 128), np.complex64)
    p1 = np.zeros((len(pk), 8, 128), np.complex64)
    for i, row in enumerate(pk):
        fr = swarm.DBEFrame.from_bin(row.tobytes())
        cs.append(fr.c), fs.append(fr.f), bs.append(fr.b)
        for ch in range(8):
            p0[i, ch] = fr.bdata["p0"]["ch%d" % ch]
            p1[i, ch] = fr.bdata["p1"]["ch%d" % ch]
    np.savez_compressed(os.path.join(OUT, "dbe_frame_decode.npz"), packets=pk,
                        c=np.array(cs), f=np.array(fs), b=np.array(bs, dtype=np.int64), p0=p0, p1=p1)


def golden_quantize_pack(rng):
    vdif = sys.modules.get("vdif") or load_py2_module(os.path.join(PROTO, "vdif.py"), "vdif")
    env = {"np": np}
    q2 = extract_function(os.path.join(PROTO, "sdbe_preprocess.py"), "quantize_to_2bit", env)
    n = 32768
    th = 0.98
    xs = rng.standard_normal(n)
    xs[:8] = [-th, 0.0, th, -0.0, -2 * th, 2 * th, 1e-9, -1e-9]
    codes_ref = q2(xs, th)
    frames = []
    headers = []
    for k, (pol, psn, secs, df) in enumerate([(0, 1, 12345, 124999), (1, 2**33 + 7, 7, 3)]):
        fr = vdif.VDIFFrame()
        fr.secs_since_epoch = secs
        fr.ref_epoch = 30
        fr.data_frame = df
        fr.frame_length = 8224 // 8
        fr.bits_per_sample = 2
        fr.thread_id = 0
        fr.station_id = (ord("S") << 8) | ord("m")
        fr.eud_vers = 2
        fr.eud = [pol | (1 << 1) | (0 << 2), 0, psn & 0xFFFFFFFF, psn >> 32]
        fr.data = codes_ref
        b = fr.to_bin()
        frames.append(np.frombuffer(b, np.uint8))
        headers.append(dict(pol=pol, psn=psn, secs=secs, df=df))
    np.savez_compressed(os.path.join(OUT, "quantize_pack.npz"), xs=xs, th=th,
                        codes=np.asarray(codes_ref, np.int8), frames=np.stack(frames),
                        hdr_pol=[h["pol"] for h in headers], hdr_psn=np.array([h["psn"] for h in headers], np.uint64),
                        hdr_secs=[h["secs"] for h in headers], hdr_df=[h["df"] for h in headers],
                        ref_epoch=30, bdc_sideband=1, rx_sideband=0)


def golden_reorder(rng):
    path = os.path.join(PROTO, "cuda", "reorder.py")
    code = extract_statements(path, 284, 293)
    n_frames = 5
    # reorder.py's CPU reference works on [channel][B-frame][snapshot]
    cpu_beng_data = rng.integers(-2, 2, size=(64, n_frames, 128)).astype(np.int8)
    env = {"np": np, "_py2div": _py2div, "cpu_beng_data": cpu_beng_data,
           "cpu_result": np.empty_like(cpu_beng_data)}
    exec(code, env)
    np.savez_compressed(os.path.join(OUT, "reorder_mar2015.npz"),
                        data=cpu_beng_data, result=env["cpu_result"])


def golden_fft_resample(seed=20150401):
    path = os.path.join(PROTO, "cuda", "resample.py")
    code = extract_statements(path, 130, 134)
    rng = np.random.default_rng(seed)
    BENG_CHANNELS_ = 16384
    BENG_CHANNELS = BENG_CHANNELS_ + 1
    num_snapshots = 39
    cpu_in = (rng.integers(-2, 2, (num_snapshots, BENG_CHANNELS))
              + 1j * rng.integers(-2, 2, (num_snapshots, BENG_CHANNELS))).astype(np.complex64)
    cpu_in[:, -1] = 0
    from numpy.fft import irfft, rfft

    def zeros(shape, dtype=float):  # numpy of the era truncated float shapes
        return np.zeros(tuple(int(s) for s in shape), dtype)

    env = {"_py2div": _py2div, "irfft": irfft, "rfft": rfft, "hstack": np.hstack, "zeros": zeros,
           "float32": np.float32, "complex64": np.complex64, "cpu_in": cpu_in,
           "num_snapshots": num_snapshots, "snapshots_per_batch": 39, "batch_size": 1,
           "BENG_CHANNELS_": BENG_CHANNELS_, "BENG_CHANNELS": BENG_CHANNELS,
           "SWARM_RATE": 2496e6, "R2DBE_RATE": 4096e6}
    exec(code, env)
    cpu_C = np.asarray(env["cpu_C"], np.float64).ravel()
    stride = 509
    np.savez_compressed(os.path.join(OUT, "fft_resample_2496.npz"), seed=seed,
                        n_out=cpu_C.size, stride=stride, sample=cpu_C[::stride],
                        sum=cpu_C.sum(), sumsq=(cpu_C ** 2).sum())


def main():
    if not REF:
        sys.exit("set SDBE_REFERENCE to the Smithsonian/sdbe checkout")
    rng = np.random.default_rng(1056)
    golden_dbe_frame(rng)
    golden_quantize_pack(rng)
    golden_reorder(rng)
    golden_fft_resample()
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
