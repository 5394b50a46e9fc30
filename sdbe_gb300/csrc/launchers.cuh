// Kernel launchers shared between the translation units of libsdbe.
#pragma once

#include "sdbe_internal.cuh"

namespace sdbe {
struct ResampleOut {
    uint8_t *out;
    int64_t out_pol_stride, pkt_stride, payload_off, pkt0;
    const float *thr;
    float *fout;
    int64_t fout_pol_stride;
    double *partials;
};

// Work of one persistent FFT launch as segments: each handle (stream pair)
// contributes n_pols x n items (n_pols 1 or 2; the kernels find the pol by
// one comparison), pol-major, starting at global item item0.
// Passed by value as a __grid_constant__ kernel parameter.
constexpr int kMaxSegs = 32;
struct SegA {  // stage A: snapshots snap0 .. snap0+n_snaps of each pol
    const uint32_t *spec;
    float *out;
    int64_t spec_pol_stride, snap0, n_snaps, out_pol_stride, item0;
};
struct SegsA {
    int64_t n_items;
    int n;
    SegA s[kMaxSegs];
};
struct SegB {  // stage BC: n_chunks 36608-sample chunks of each pol
    const float *in;
    int64_t in_pol_stride, item0;
    int n_chunks, skip;
    ResampleOut o;
};
struct SegsB {
    int64_t n_items;
    int n;
    SegB s[kMaxSegs];
};
cudaError_t launch_swarm_c2r_segs(const SegsA &, const Twiddles &, cudaStream_t);
cudaError_t launch_resample_segs(int mode, const SegsB &, const Twiddles &, cudaStream_t);
cudaError_t launch_unpack(const void *, int64_t, uint64_t, int, int, uint32_t *, int64_t, int64_t, uint32_t *,
                          int32_t *, int32_t *, cudaStream_t, const uint8_t *accept = nullptr);
// The packet unpack and zero fill of several calls (one segment each) in one
// launch each: per segment the arguments of launch_unpack / launch_fill_missing.
struct UnpackSeg {
    const uint8_t *pkts;
    int64_t n_pkts;
    uint64_t b_zero;
    int n_frames, map;
    uint32_t *spec;
    int64_t pol_stride, snap0;
    uint32_t *bitmap;
    int32_t *counts, *rejected;
    const uint8_t *accept;
    int64_t blk0, fill0;  // first block of the unpack grid, first thread of the fill grid (set by unpack_segs_add)
};
struct UnpackSegs {
    int n;
    int64_t blocks, fill_threads;
    UnpackSeg s[kMaxSegs];
};
void unpack_segs_add(UnpackSegs &S, const UnpackSeg &g);
cudaError_t launch_unpack_segs(const UnpackSegs &S, cudaStream_t st);
cudaError_t launch_fill_missing_segs(const UnpackSegs &S, cudaStream_t st);
cudaError_t launch_fill_missing(const uint32_t *, int, int, uint32_t *, int64_t, int64_t, cudaStream_t);
cudaError_t launch_vdif_to_beng_ref(const void *, int64_t, uint64_t, int, int, int8_t *, int8_t *, cudaStream_t);
cudaError_t launch_reorder_mar2015(const uint32_t *, int, uint32_t *, cudaStream_t);
cudaError_t launch_beng_to_complex(const int8_t *, int64_t, void *, cudaStream_t);
cudaError_t build_twiddles(Twiddles &, float2 **);
cudaError_t configure_fft_kernels();
cudaError_t launch_swarm_c2r(const uint32_t *, int64_t, int64_t, int64_t, int, float *, int64_t, const Twiddles &,
                             cudaStream_t);
cudaError_t launch_resample(int, const float *, int64_t, int, int64_t, int, const ResampleOut &, const Twiddles &,
                            cudaStream_t);
cudaError_t launch_swarm_r2c(const float *, int64_t, void *, const Twiddles &, cudaStream_t);
cudaError_t launch_r2dbe_c2r(const void *, int64_t, int64_t, int, float *, const Twiddles &, cudaStream_t);
cudaError_t launch_finalize_thresholds(const double *, int, int, float *, cudaStream_t);
struct WinUpd {  // one handle's windowed-threshold step after a wave
    const double *partials;  // [2][nb*128][3]
    double *ring;            // [2][W][3]
    float *thr;
    int64_t t0;              // stream batch of the wave's first batch
    int nb, W, update, pol1, moments;  // moments: partials are (n, mean, M2), else (n, sum, sum of squares)
};
struct WinUpds {
    int n;
    WinUpd u[kMaxSegs];
};
cudaError_t launch_window_update(const WinUpds &, cudaStream_t);
cudaError_t launch_quantize_chunks(const float *, int64_t, int64_t, const float *, uint8_t *, int64_t, int64_t,
                                   int64_t, int64_t, cudaStream_t);
cudaError_t launch_quantize_flat(const float *, uint32_t *, int64_t, float, float, cudaStream_t);
int stats_partial_blocks(int64_t);
cudaError_t launch_stats_partial(const float *, int64_t, double *, int, cudaStream_t);
cudaError_t launch_align_frames(const uint32_t *, int64_t, const uint32_t *, int64_t, int64_t, int64_t, int64_t, void *,
                                int64_t, cudaStream_t);
cudaError_t launch_save_leftover(const uint32_t *, int64_t, const uint32_t *, int64_t, int64_t, int64_t, int64_t, int64_t,
                                 uint32_t *, cudaStream_t);
cudaError_t launch_vdif_headers(void *, int64_t, int64_t, uint32_t, uint32_t, uint64_t, uint32_t, uint32_t, uint32_t,
                                uint32_t, cudaStream_t);
cudaError_t launch_unpack_8pac(const void *, int64_t, void *, cudaStream_t);
cudaError_t launch_beng_reform(void *, int64_t, const sdbe_reform_state &, sdbe_reform_state *, uint32_t *,
                               cudaStream_t);
cudaError_t launch_gather_headers(const void *, int64_t, uint32_t *, cudaStream_t);

}  // namespace sdbe
