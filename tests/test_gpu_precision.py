"""Precision of both FFT paths against the FP64 oracle (the precision-form config).

For the FP32 radix path and the two FP16 tensor-core paths
(SDBE_PRECISION_TC16: data and DFT matrix split hi + lo; SDBE_PRECISION_TC16_FAST:
data rounded to FP16, DFT matrix split) this measures, on sampled 143-snapshot batches of the 3-tone stream, the
relative RMS error of the resampled series before requantization and the
2-bit code agreement (GPU: its series, FP32 compare with its own
FP64-accumulated thresholds; oracle: FP64 series, FP64 thresholds).  Results
of the paths run so far are written as JSON to the path in
``$SDBE_PRECISION_JSON`` when it is set.
"""
import json
import os

import numpy as np
import pytest

from gpu_util import dev, empty, host, ptr, rel_rms, zeros
from oracle import sdbe_oracle as O

pytestmark = pytest.mark.gpu

# relative RMS of the chain of three transforms against FP64
RMS_TOL = {"fp32": 3e-6, "tc16": 3e-5, "tc16fast": 2e-3}
AGREE_MIN = 0.999
_RESULTS = {}


@pytest.mark.parametrize("path", ["fp32", "tc16", "tc16fast"])
def test_path_rms_and_code_agreement(path):
    import __graft_entry__ as g

    g.build()
    from sdbe_gb300 import Resampler, synth
    from sdbe_gb300 import _native as N

    spec = synth.config2(n_frames=4)
    p = synth.generate(spec)
    nf = 4
    snaps = nf * 128
    words = empty(2 * snaps * 2048 * 4, "int32")
    bitmap, counts, rej = zeros(nf * 256), zeros(nf * 4, "int32"), zeros(4, "int32")
    lib = N.lib()
    N.check(lib.sdbe_unpack(ptr(dev(p)), p.shape[0], spec.b_start, nf, 0, ptr(words), snaps * 2048, 0, ptr(bitmap),
                            ptr(counts), ptr(rej), None))
    beng = O.vdif_to_beng(p, spec.b_start, nf)
    prec = {"fp32": N.PRECISION_FP32, "tc16": N.PRECISION_TC16, "tc16fast": N.PRECISION_TC16_FAST}[path]
    results = []
    with Resampler(trim_mhz=150, max_frames=nf, precision=prec) as rs:
        for b in (0, 2):
            ts = empty(143 * 32768 * 4, "float32")
            y = empty(128 * 32768 * 4, "float32")
            src = int(words.data_ptr()) + b * 143 * 2048 * 4   # pol 0
            N.check(lib.sdbe_swarm_c2r(rs.handle, src, 143, ptr(ts), None), rs.handle)
            N.check(lib.sdbe_resample_chunks(rs.handle, ptr(ts), 128, ptr(y), None), rs.handle)
            got = host(y).reshape(128, 32768).astype(np.float64)
            sp = O.beng_to_complex(beng[0].reshape(-1, 16384, 2))[b * 143:(b + 1) * 143]
            ts_ref = O.swarm_c2r(sp).reshape(-1)
            ref = O.r2dbe_c2r(O.swarm_r2c(ts_ref), rs.skip_chan)
            err = rel_rms(got, ref)
            err_a = rel_rms(host(ts).astype(np.float64), ts_ref)
            off_g, th_g = O.summary_stats(got)
            off_r, th_r = O.summary_stats(ref)
            cg = O.quantize2bit_codes(got.astype(np.float32), th_g, off_g, np.float32)
            cr = O.quantize2bit_codes(ref, th_r, off_r)
            agree = float(np.mean(cg == cr))
            results.append({"batch": b, "rel_rms": err, "rel_rms_stage_a": err_a,
                            "max_abs_rel": float(np.abs(got - ref).max() / ref.std()),
                            "code_agreement": agree, "threshold_rel_diff": abs(th_g - th_r) / th_r})
    _RESULTS[path] = {"samples_per_batch": 128 * 32768, "batches": results}
    if os.environ.get("SDBE_PRECISION_JSON"):
        with open(os.environ["SDBE_PRECISION_JSON"], "w") as f:
            json.dump(_RESULTS, f, indent=1)
    for r in results:
        assert r["rel_rms"] < RMS_TOL[path], r
        assert r["code_agreement"] >= AGREE_MIN, r
