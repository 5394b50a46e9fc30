// The resampler handle and helpers shared by the host-side translation units.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

#include "launchers.cuh"
#include "sdbe_internal.cuh"

struct sdbe_resampler {
    sdbe_config cfg{};
    int skip = 0;
    int wave = 4;
    cudaStream_t stream = nullptr;
    sdbe::Twiddles tw{};
    float2 *tw_storage = nullptr;
    int64_t max_snaps = 0;
    uint32_t *spec = nullptr;     // [2][max_snaps][2048] packed spectra
    int64_t spec_pol_stride = 0;  // words
    uint32_t *bitmap = nullptr;   // [max_frames][64]
    int32_t *counts = nullptr;    // [max_frames] per-frame packets, then [1] rejected
    float *ts = nullptr;          // [2][wave*143*32768] stage-A time series
    int64_t ts_pol_stride = 0;
    float *fout = nullptr;        // [2][128*32768] first-batch floats
    double *partials = nullptr;   // [2][128][3]
    float *thr = nullptr;         // device [8], see k_finalize_thresholds
    // host I/O: two staging slots so one call's copies overlap another's compute
    cudaStream_t copy_in = nullptr, copy_out = nullptr, last_stream = nullptr;
    struct Stage {
        uint8_t *pkt = nullptr;
        int64_t pkt_bytes = 0;
        uint8_t *out = nullptr;
        int64_t out_bytes = 0;
        cudaEvent_t pkt_ready = nullptr, pkt_free = nullptr, out_free = nullptr;
    };
    Stage stage[2];
    int stage_idx = 0;
    cudaEvent_t wave_ev = nullptr;
    // output time alignment (SDBE_OUT_ALIGNED)
    bool align_pending = false;
    sdbe_time_template tmpl{};
    int64_t skip_pending = 0;      // payload words still to drop
    uint32_t *left[2] = {nullptr, nullptr};  // [2 pols][2048] leftover words, double-buffered
    int left_idx = 0;
    int64_t n_left = 0;
    uint8_t *pay = nullptr;        // plain payload stream before alignment
    int64_t pay_bytes = 0;
    // group assembly (sdbe_ingest): a ring of 4 open groups of 143 B-frames
    uint32_t *ring = nullptr;      // [2][4*18304][2048] packed spectra
    uint32_t *ring_bitmap = nullptr;  // [4][143][64]
    uint8_t *ing_batch = nullptr;  // device copy of the received batch
    int64_t ing_batch_bytes = 0;
    uint8_t *ing_accept = nullptr; // device accept mask
    int64_t ing_accept_bytes = 0;
    uint8_t *ing_out = nullptr;    // staging for host output
    int64_t ing_out_bytes = 0;
    uint8_t *ing_raw = nullptr;    // device copy of a host 8pac batch
    int64_t ing_raw_bytes = 0;
    uint8_t *ing_hdr = nullptr;    // [n][3] header words (w0, w4, w5) read back for the policy
    int64_t ing_hdr_bytes = 0;
    sdbe_reform_state reform{-1, -1, -1, -1, -1, 0, 0, 0};  // 8pac batches: reform state
    sdbe_reform_state *reform_dev = nullptr;                // kernel's output state
    double *ipfb_tab = nullptr;   // inverse PFB: [2][ntap][32768] band of P P^T and P taps (FP64)
    int ipfb_ntap = 0;
    uint8_t *ipfb_y = nullptr;    // inverse PFB scratch, grown to the largest call: y [nblock][32768] f32
    int64_t ipfb_y_bytes = 0;
    uint8_t *ipfb_scr = nullptr;  // factors [nblock][ntap][32768] f64
    int64_t ipfb_scr_bytes = 0;
    uint8_t *pol_scr = nullptr;   // group assembly on the device: state, result, bins, codes
    int64_t pol_scr_bytes = 0;
    int64_t ing_last_n = 0;       // packets of the last sdbe_ingest batch (their flags in ing_accept)
    int64_t b_first = -1;
    int64_t ing_ref = 0;
    int64_t g_count[4] = {0, 0, 0, 0};
    std::vector<int32_t> g_fcount = std::vector<int32_t>(4 * 143, 0);
    sdbe_ingest_stats ing{};
    bool thresholds_set = false;
    int64_t carry = 0;
    int64_t stream_batch = 0;     // batches quantized since the stream started (window blocks)
    int window = 0;               // SDBE_THRESH_WINDOW: batches per window
    double *wring = nullptr;      // [2][window][3] batch statistics (n, mean, M2)
    double *wpart = nullptr;      // [2][wave*128][3] chunk statistics of one wave
    // SDBE_PRECISION_TC16: pre-tiled FP16 DFT matrices and complex scratch (on first use)
    void *tc_f128 = nullptr, *tc_f143 = nullptr;
    float2 *tc_bufx = nullptr;    // [2][wave*143][16384]
    float2 *tc_bufy = nullptr;    // [2][wave*128][18304]
    void *tcf_tabs = nullptr;     // SDBE_PRECISION_TC16_FAST: DFT matrices and twiddle tables (on first use)
    uint32_t *tcf_bins = nullptr; // its R2C bins [2][wave*128][kTcfBinsLen] half2 (on first use)
    int64_t tcf_bins_bytes = 0;
    void *tcf_half = nullptr;     // FP16 time series of sdbe_resample_chunks inputs (on first use)
    int64_t tcf_half_bytes = 0;
    uint8_t *tcf_chain = nullptr; // tickets and stage counters of the one-launch waves (on first use)
    int64_t tcf_chain_bytes = 0;
    int *tc_status_host = nullptr;  // 1 after a tensor-core barrier time-out (pinned, mapped)
    int *tc_status = nullptr;       // its device address
    int64_t tc_test_timeout_ns = 0; // > 0: the next fast tensor-core launch withholds a signal (test hook)
    // Mar-2015 format: unpacked frames land here first; the last one is held
    // for the next call because output frame f needs input frame f+1.
    uint32_t *raw = nullptr;      // [2][max_frames+1][128][2048]
    int64_t raw_pol_stride = 0;   // words
    int raw_carry = 0;            // 0 or 1 frame held
    uint32_t secs = 0, df = 0, ref_epoch = 0, station = (uint32_t('S') << 8) | uint32_t('m'), bdc = 0, rx = 0;
    uint64_t psn = 1;
    std::string err;
    // profiling (sdbe_profile_enable / sdbe_profile_read)
    bool prof = false;
    struct Timed {
        cudaEvent_t a, b;
        int kind;       // 0 = stage A, 1 = stage BC
        int64_t units;  // snapshots or chunks
    };
    std::vector<Timed> timed;     // pool; first n_timed in use
    size_t n_timed = 0;
    int64_t launches = 0;
};

namespace sdbe {

int fail(sdbe_resampler *h, int code, const std::string &msg);

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

#define SDBE_CK(h, call)                                                                             \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return ::sdbe::fail((h), SDBE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

cudaError_t timed_begin(sdbe_resampler *h, int kind, int64_t units, cudaStream_t st, size_t *slot);
cudaError_t timed_end(sdbe_resampler *h, size_t slot, cudaStream_t st);
int grow(sdbe_resampler *h, uint8_t **buf, int64_t *cap, int64_t need, const char *what);
// A device buffer of at least `bytes` owned by the calling host thread on the
// current device, kept and reused by later calls of that thread (grown when
// too small).  For handle-less entry points that wait for their stream before
// returning, so that one thread's calls never overlap on it.
cudaError_t thread_scratch(size_t bytes, void **out);

// Where the FFT waves write their payload packets.
struct PayloadTarget {
    uint8_t *base;
    int64_t pol_stride, pkt_stride, payload_off;
};

// Batches the next wave may take: up to `wave` of the `remaining`, and with
// windowed thresholds not past the stream's next block boundary.
inline int64_t wave_len(const sdbe_resampler *h, int64_t wave, int64_t remaining) {
    int64_t nb = remaining < wave ? remaining : wave;
    if (h->cfg.threshold_mode == SDBE_THRESH_WINDOW) {
        const int64_t to_block = SDBE_THRESH_BLOCK - h->stream_batch % SDBE_THRESH_BLOCK;
        if (nb > to_block) nb = to_block;
    }
    return nb;
}

// After a wave of nb batches was quantized: the handle's windowed-threshold
// step (appended to U, launched by the caller) and its batch counter.
inline void window_step(sdbe_resampler *h, const double *partials, int64_t nb, bool moments, WinUpds &U) {
    if (h->cfg.threshold_mode == SDBE_THRESH_WINDOW) {
        const int64_t t0 = h->stream_batch;
        U.u[U.n++] = WinUpd{partials, h->wring, h->thr, t0, static_cast<int>(nb), h->window,
                            (t0 + nb) % SDBE_THRESH_BLOCK == 0 ? 1 : 0, h->cfg.pol1_uses_pol0_threshold,
                            moments ? 1 : 0};
    }
    h->stream_batch += nb;
}

inline int window_after_wave(sdbe_resampler *h, const double *partials, int64_t nb, bool moments, cudaStream_t st) {
    WinUpds U{};
    window_step(h, partials, nb, moments, U);
    if (U.n == 0) return SDBE_OK;
    SDBE_CK(h, launch_window_update(U, st));
    h->launches += 1;
    return SDBE_OK;
}

// Group assembly state (the ingest policy of vdif_in_databuf.c:96-167) as the
// device walk reads and writes it: the first b-count, the oldest open group,
// packets per ring slot and per slot and frame, and the statistics (packets,
// invalid, before_start, too_far_ahead, used, overflow, groups_shipped,
// groups_incomplete).
struct PolState {
    long long b_first, ref;
    long long count[4];
    long long st[8];
    int fcount[4 * 143];
};
constexpr int kPolWindow = 16384;    // B-frames a batch may span from the oldest open group
constexpr int kPolMaxGroups = 128;   // groups shipped or touched by one batch (bounded by the window)
struct PolOut {
    PolState s;                      // the state after the batch
    long long base;                  // b-count of the window's first frame (-1: no valid packet yet)
    int n_ships, n_touched, n_capped, window_exceeded;
    long long ships[kPolMaxGroups], touched[kPolMaxGroups];
};
// The policy on the device for a batch (k_policy.cu): header words (w0, w4,
// w5) of n packets at hdr -> accept[n] on the device, the result in res.
int policy_device(sdbe_resampler *h, const uint32_t *hdr, int64_t n, uint8_t *accept, PolOut *res, cudaStream_t st);

// The FFT chain of sdbe_process on a tensor-core handle (k_tc.cu): same
// arguments as fft_chain (on_wave(lo, hi) after the wave that completes
// payload packets [lo, hi) is queued), payload complete when it returns.
int tc_chain(sdbe_resampler *h, const uint32_t *spec, int64_t spec_pol_stride, int64_t n_batches,
             const PayloadTarget &tgt, cudaStream_t st, const std::function<int(int64_t, int64_t)> &on_wave);

// Batches [b0, b0 + nb) of one handle's packed spectra in a tensor-core wave.
struct TcWaveItem {
    sdbe_resampler *h;
    const uint32_t *spec;
    int64_t spec_pol_stride, b0, nb;
    PayloadTarget tgt;
};
// One wave over several tensor-core handles of the same precision, the three
// transforms in shared launches; `first`: each item is its handle's first batch.
int tc_wave_multi(const std::vector<TcWaveItem> &w, bool first, cudaStream_t st);

// Stage A of the fast tensor-core form (k_tcf.cu): per segment, snapshots
// [snap0, snap0 + n_snaps) of n_pols pols -> float time series [n_snaps][32768]
// at out + pol * out_pol_stride; all segments in one launch.
struct TcfASeg {
    const uint32_t *spec;
    int64_t spec_pol_stride, snap0, n_snaps;
    void *out;               // float, or FP16 x 2^-2
    int64_t out_pol_stride;  // elements
};
int tcf_prepare(sdbe_resampler *h, cudaStream_t st);
int tcf_stage_a(sdbe_resampler *h, const TcfASeg *segs, int n_segs, int n_pols, bool half_out, cudaStream_t st);
// Stages B and C of the fast tensor-core form: per segment n_chunks chunks of
// n_pols pols of FP16 time series (x 2^-2) -> R2C bins [skip, skip + 16384]
// (scratch, kTcfBinsLen half2 per chunk) -> mode 0: 2-bit payload (o.out ...),
// 1: floats (o.fout) + per-chunk (n, mean, M2) in o.partials, 3: 2-bit payload
// + per-chunk (n, sum, sum of squares) in o.partials (if not null), 5: floats.
struct TcfBCSeg {
    const void *ts;
    int64_t ts_pol_stride;   // halves
    uint32_t *bins;
    int64_t bins_pol_stride; // bins
    int64_t n_chunks;
    int skip;
    ResampleOut o;
};
int tcf_stage_bc(sdbe_resampler *h, const TcfBCSeg *segs, int n_segs, int n_pols, int mode, cudaStream_t st);
cudaError_t tcf_to_half(const float *in, void *out, int64_t n_floats, cudaStream_t st);
// One wave of the fast tensor-core chain over several handles (as tc_wave_multi).
int tcf_wave_multi(const std::vector<TcWaveItem> &w, bool first, cudaStream_t st);

// sdbe_swarm_c2r / sdbe_resample_chunks of a SDBE_PRECISION_TC16 handle (one pol).
int tc_swarm_c2r(sdbe_resampler *h, const uint32_t *spec, int64_t n_snaps, float *out, cudaStream_t st);
int tc_resample_chunks(sdbe_resampler *h, const float *in, int64_t n_chunks, float *out, cudaStream_t st);
// C2R 32768 of complex spectra [n][spec_stride] in the tensor-core form (z: n x 16384 complex scratch).
int tc_c2r_spectra(sdbe_resampler *h, const float2 *spec, int64_t spec_stride, int64_t n, float2 *z, float *out,
                   cudaStream_t st);

// First-batch threshold path (if thresholds are unset) and the FFT waves over
// n_batches 143-snapshot batches of packed spectra (spec + pol*spec_pol_stride,
// snapshots from 0), payload packets at tgt from packet 0.  on_wave(lo, hi)
// runs after the waves that completed packets [lo, hi) are queued.
template <class OnWave>
int fft_chain(sdbe_resampler *h, const uint32_t *spec, int64_t spec_pol_stride, int64_t n_batches,
              const PayloadTarget &tgt, cudaStream_t st, OnWave on_wave) {
    int64_t b = 0;
    const bool win = h->cfg.threshold_mode == SDBE_THRESH_WINDOW;
    if (n_batches > 0 && !h->thresholds_set) {
        // First batch: floats + FP64 statistics, thresholds set once (.cu:953-986).
        SDBE_CK(h, launch_swarm_c2r(spec, spec_pol_stride, 0, kBatchSnaps, 2, h->ts, h->ts_pol_stride, h->tw, st));
        ResampleOut o{};
        o.fout = h->fout;
        o.fout_pol_stride = static_cast<int64_t>(kChunks) * kNC;
        o.partials = h->partials;
        SDBE_CK(h, launch_resample(1, h->ts, h->ts_pol_stride, h->skip, kChunks, 2, o, h->tw, st));
        SDBE_CK(h, launch_finalize_thresholds(h->partials, kChunks, h->cfg.pol1_uses_pol0_threshold, h->thr, st));
        SDBE_CK(h, launch_quantize_chunks(h->fout, static_cast<int64_t>(kChunks) * kNC, kChunks, h->thr, tgt.base,
                                          tgt.pol_stride, tgt.pkt_stride, tgt.payload_off, 0, st));
        h->thresholds_set = true;
        h->launches += 4;
        h->stream_batch = 0;
        if (int rc = window_after_wave(h, h->partials, 1, true, st)) return rc;
        b = 1;
        if (int rc = on_wave(0, kChunks)) return rc;
    }
    while (b < n_batches) {
        const int64_t nb = wave_len(h, h->wave, n_batches - b);
        size_t slot;
        SDBE_CK(h, timed_begin(h, 0, 2 * nb * kBatchSnaps, st, &slot));
        SDBE_CK(h, launch_swarm_c2r(spec, spec_pol_stride, b * kBatchSnaps, nb * kBatchSnaps, 2, h->ts,
                                    h->ts_pol_stride, h->tw, st));
        SDBE_CK(h, timed_end(h, slot, st));
        SDBE_CK(h, timed_begin(h, 1, 2 * nb * kChunks, st, &slot));
        ResampleOut o{};
        o.out = tgt.base;
        o.out_pol_stride = tgt.pol_stride;
        o.pkt_stride = tgt.pkt_stride;
        o.payload_off = tgt.payload_off;
        o.pkt0 = b * kChunks;
        o.thr = h->thr;
        o.partials = win ? h->wpart : nullptr;
        SDBE_CK(h, launch_resample(win ? 3 : 0, h->ts, h->ts_pol_stride, h->skip, nb * kChunks, 2, o, h->tw, st));
        SDBE_CK(h, timed_end(h, slot, st));
        h->launches += 2;
        if (int rc = window_after_wave(h, h->wpart, nb, false, st)) return rc;
        if (int rc = on_wave(b * kChunks, (b + nb) * kChunks)) return rc;
        b += nb;
    }
    return SDBE_OK;
}

}  // namespace sdbe
