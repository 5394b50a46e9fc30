"""CPU checks of the host-side pieces: synthetic generator, oracle pipeline
properties, and the multi-process sharding of streams over ranks (gloo)."""
import os

import numpy as np
import pytest

from oracle import sdbe_oracle as O


@pytest.fixture(scope="module")
def synth():
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import synth as S

    return S


def test_generator_is_deterministic_and_thread_independent(synth):
    spec = synth.config1()
    spec.n_frames = 3
    a = synth.generate(spec, n_threads=1)
    b = synth.generate(spec, n_threads=3)
    assert np.array_equal(a, b)
    # frames are the same whichever call generates them
    assert np.array_equal(synth.generate(spec, frame_offset=1, n_frames=2), a[2048:])
    spec2 = synth.config1(stream=1)
    spec2.n_frames = 3
    assert not np.array_equal(a, synth.generate(spec2))


def test_generator_layout_and_statistics(synth):
    spec = synth.config1()
    spec.n_frames = 2
    p = synth.generate(spec)
    inv, c, f, b = O.decode_beng_headers(p)
    assert (inv == 0).all() and p.shape == (2 * 2048, 1056)
    assert set(np.unique(b)) == {spec.b_start, spec.b_start + 1}
    cc, counts = O.completion_bitmap(p, spec.b_start, 2)
    assert (cc == 0xFF).all() and (counts == 2048).all()
    b0, b1 = O.vdif_to_beng(p, spec.b_start, 2)
    for beng in (b0, b1):
        vals, cnt = np.unique(beng[..., 1], return_counts=True)
        frac = cnt / cnt.sum()
        assert list(vals) == [-2, -1, 0, 1]
        assert abs(frac[0] - 0.1635) < 0.002 and abs(frac[1] - 0.3365) < 0.002
    # the 10 dB tone at channel 5000 pushes pol 0 real codes to the top level
    assert (b0[:, :, 5000, 1] == 1).mean() > 0.95


def test_impairments_drop_and_displace(synth):
    spec = synth.config1()
    spec.n_frames = 2
    spec.drop_frac, spec.reorder_frac, spec.reorder_max = 0.01, 0.005, 64
    p = synth.generate(spec)
    n = 2 * 2048
    assert n * 0.97 < p.shape[0] < n
    inv, c, f, b = O.decode_beng_headers(p)
    key = (b - spec.b_start) * 2048 + c * 8 + f
    assert len(np.unique(key)) == p.shape[0]            # no duplicates
    assert np.any(np.diff(key) < 0)                      # some displaced
    cc, counts = O.completion_bitmap(p, spec.b_start, 2)
    assert counts.sum() == p.shape[0]


def test_oracle_carry_matches_single_call(synth):
    """Two calls of 2 frames == one call of 4 frames (snapshots carried)."""
    spec = synth.config1()
    spec.n_frames = 4
    p = synth.generate(spec)
    one = O.process_group(p, spec.b_start, 4, 150)
    st = O.StreamState()
    half = 2 * 2048
    a = O.process_group(p[:half], spec.b_start, 2, 150, state=st)
    b = O.process_group(p[half:], spec.b_start + 2, 2, 150, state=st)
    assert one.shape[1] == 3 * 128 and a.shape[1] + b.shape[1] == one.shape[1]
    assert np.array_equal(np.concatenate([a, b], axis=1), one)


def test_oracle_missing_packets_are_zero(synth):
    spec = synth.config1()
    spec.n_frames = 1
    p = synth.generate(spec)
    keep = np.ones(p.shape[0], bool)
    keep[::7] = False
    b0, _ = O.vdif_to_beng(p[keep], spec.b_start, 1)
    inv, c, f, b = O.decode_beng_headers(p[~keep])
    base = O.channel_base_aphids(c, f)
    assert (b0[0][:, base[0]:base[0] + 8] == 0).all()


def _shard_worker(rank, world, port, out_dir):
    import torch.distributed as dist

    from sdbe_gb300 import sharding

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    streams = list(range(7))
    mine = sharding.streams_for_rank(streams, rank, world)
    work = sharding.allgather_counts(len(mine))
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.array([len(mine), sum(work)] + mine))
    dist.destroy_process_group()


def test_streams_shard_over_ranks_gloo(tmp_path):
    import socket

    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.spawn(_shard_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "r0.npy")
    r1 = np.load(tmp_path / "r1.npy")
    assert r0[1] == r1[1] == 7
    assert sorted(list(r0[2:]) + list(r1[2:])) == list(range(7))


def _digest_worker(rank, world, port, out_dir):
    import hashlib

    import torch.distributed as dist

    from oracle import sdbe_oracle as O
    from sdbe_gb300 import sharding, synth

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    specs = [synth.config1(stream=i) for i in range(5)]
    for sp in specs:
        sp.n_frames = 2

    def run(i, sp):  # the stage's CPU restatement on this rank's stream
        out = O.process_group(synth.generate(sp), sp.b_start, sp.n_frames, 150)
        return hashlib.sha256(out.tobytes()).hexdigest()

    got = sharding.process_shard(specs, run, rank, world)
    np.save(os.path.join(out_dir, f"d{rank}.npy"), np.array([f"{k}:{v}" for k, v in sorted(got.items())]))
    dist.destroy_process_group()


def test_shard_results_equal_single_process_gloo(tmp_path, synth):
    """Two ranks over gloo each process their round-robin share of five
    streams and gather the digests of their outputs: every rank holds all
    five, equal to one process running them all."""
    import hashlib
    import socket

    import torch.multiprocessing as mp

    from sdbe_gb300 import sharding

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.spawn(_digest_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    d0, d1 = np.load(tmp_path / "d0.npy"), np.load(tmp_path / "d1.npy")
    specs = [synth.config1(stream=i) for i in range(5)]
    for sp in specs:
        sp.n_frames = 2
    single = sharding.process_shard(
        specs, lambda i, sp: hashlib.sha256(O.process_group(synth.generate(sp), sp.b_start, 2, 150).tobytes()).hexdigest(),
        0, 1)
    want = np.array([f"{k}:{v}" for k, v in sorted(single.items())])
    assert len(want) == 5
    assert np.array_equal(d0, want) and np.array_equal(d1, want)


def test_oracle_mar2015_stream_split_equals_single(synth):
    """Mar-2015 mode holds one frame back; splitting the stream changes nothing."""
    spec = synth.config1()
    spec.n_frames = 5
    spec.channel_map = 1
    p = synth.generate(spec)
    one = O.process_group(p, spec.b_start, 5, 150, channel_map="mar2015")
    st = O.StreamState()
    a = O.process_group(p[:3 * 2048], spec.b_start, 3, 150, state=st, channel_map="mar2015")
    b = O.process_group(p[3 * 2048:], spec.b_start + 3, 2, 150, state=st, channel_map="mar2015")
    assert one.shape[1] == (4 * 128 // 143) * 128
    assert np.array_equal(np.concatenate([a, b], axis=1), one)
