// C ABI of libsdbe: the drop-in for the APHIDS GPU stage
// (software/aphids/vdif_inout_gpu_thread.cu, Smithsonian/sdbe).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "handle.cuh"
#include "launchers.cuh"
#include "sdbe_internal.cuh"

namespace sdbe {
static thread_local std::string g_thread_error;
void set_thread_error(const std::string &msg) { g_thread_error = msg; }
const std::string &thread_error() { return g_thread_error; }
}  // namespace sdbe

using namespace sdbe;

namespace sdbe {

int fail(sdbe_resampler *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    set_thread_error(msg);
    return code;
}

cudaError_t timed_begin(sdbe_resampler *h, int kind, int64_t units, cudaStream_t st, size_t *slot) {
    *slot = SIZE_MAX;
    if (!h->prof) return cudaSuccess;
    if (h->n_timed == h->timed.size()) {
        sdbe_resampler::Timed t{};
        cudaError_t e = cudaEventCreate(&t.a);
        if (e == cudaSuccess) e = cudaEventCreate(&t.b);
        if (e != cudaSuccess) return e;
        h->timed.push_back(t);
    }
    *slot = h->n_timed++;
    h->timed[*slot].kind = kind;
    h->timed[*slot].units = units;
    return cudaEventRecord(h->timed[*slot].a, st);
}

cudaError_t timed_end(sdbe_resampler *h, size_t slot, cudaStream_t st) {
    if (slot == SIZE_MAX) return cudaSuccess;
    return cudaEventRecord(h->timed[slot].b, st);
}

void free_all(sdbe_resampler *h) {
    for (auto &t : h->timed) {
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    cudaFree(h->tw_storage);
    cudaFree(h->spec);
    cudaFree(h->bitmap);
    cudaFree(h->counts);
    cudaFree(h->ts);
    cudaFree(h->fout);
    cudaFree(h->partials);
    cudaFree(h->thr);
    cudaFree(h->raw);
    cudaFree(h->ring);
    cudaFree(h->ring_bitmap);
    cudaFree(h->ing_batch);
    cudaFree(h->ing_accept);
    cudaFree(h->ing_out);
    cudaFree(h->ing_raw);
    cudaFree(h->ing_hdr);
    cudaFree(h->reform_dev);
    cudaFree(h->ipfb_tab);
    cudaFree(h->ipfb_y);
    cudaFree(h->ipfb_scr);
    cudaFree(h->wring);
    cudaFree(h->wpart);
    cudaFree(h->tc_f128);
    cudaFree(h->tc_f143);
    cudaFree(h->tc_bufx);
    cudaFree(h->tc_bufy);
    cudaFree(h->tcf_tabs);
    cudaFree(h->tcf_bins);
    cudaFree(h->tcf_half);
    cudaFree(h->tcf_chain);
    cudaFree(h->pol_scr);
    if (h->tc_status_host) cudaFreeHost(h->tc_status_host);
    cudaFree(h->left[0]);
    cudaFree(h->left[1]);
    cudaFree(h->pay);
    for (auto &sg : h->stage) {
        cudaFree(sg.pkt);
        cudaFree(sg.out);
        if (sg.pkt_ready) cudaEventDestroy(sg.pkt_ready);
        if (sg.pkt_free) cudaEventDestroy(sg.pkt_free);
        if (sg.out_free) cudaEventDestroy(sg.out_free);
    }
    if (h->wave_ev) cudaEventDestroy(h->wave_ev);
    if (h->copy_in) cudaStreamDestroy(h->copy_in);
    if (h->copy_out) cudaStreamDestroy(h->copy_out);
    if (h->stream) cudaStreamDestroy(h->stream);
}

cudaStream_t pick(sdbe_resampler *h, void *stream) {
    return stream ? static_cast<cudaStream_t>(stream) : h->stream;
}

// B-frames of spectra a call adds to the snapshot stream.
int64_t frames_out(const sdbe_resampler *h, int32_t n_frames) {
    if (h->cfg.channel_map != SDBE_MAP_MAR2015) return n_frames;
    const int64_t n_in = h->raw_carry + static_cast<int64_t>(n_frames);
    return n_in >= 2 ? n_in - 1 : 0;
}

int64_t batches_for(const sdbe_resampler *h, int32_t n_frames) {
    return (h->carry + frames_out(h, n_frames) * kSnapsPerFrame) / kBatchSnaps;
}

cudaError_t thread_scratch(size_t bytes, void **out) {
    struct Slot {
        void *p = nullptr;
        size_t bytes = 0;
    };
    thread_local std::vector<Slot> slots;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (static_cast<size_t>(dev) >= slots.size()) slots.resize(static_cast<size_t>(dev) + 1);
    Slot &sl = slots[static_cast<size_t>(dev)];
    if (sl.bytes < bytes) {
        if (sl.p) {
            e = cudaFree(sl.p);
            if (e != cudaSuccess) return e;
        }
        sl.p = nullptr;
        sl.bytes = 0;
        e = cudaMalloc(&sl.p, bytes);
        if (e != cudaSuccess) return e;
        sl.bytes = bytes;
    }
    *out = sl.p;
    return cudaSuccess;
}

int grow(sdbe_resampler *h, uint8_t **buf, int64_t *cap, int64_t need, const char *what) {
    if (*cap >= need) return SDBE_OK;
    if (*buf && cudaDeviceSynchronize() != cudaSuccess) return fail(h, SDBE_ERR_CUDA, "synchronize before regrow");
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    if (cudaMalloc(buf, static_cast<size_t>(need)) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDBE_ERR_NOMEM, std::string("cannot allocate ") + what);
    }
    *cap = need;
    return SDBE_OK;
}


// One sdbe_process call, split so that several handles can share the FFT
// launches (sdbe_process_multi): plan (checks, no side effects), prepare
// (staging, unpack, headers), the FFT chain, complete (alignment, carry, sync).
struct CallPlan {
    sdbe_resampler *h = nullptr;
    cudaStream_t st = nullptr;
    const void *packets = nullptr;
    int64_t n_packets = 0;
    int32_t n_frames = 0;
    uint64_t b_zero = 0;
    void *out = nullptr;
    uint32_t flags = 0;
    bool aligned = false, framed = false, host_in = false, host_out = false;
    int64_t n_frames_out = 0;  // B-frames of spectra this call adds (Mar-2015 holds one back)
    int64_t n_batches = 0, n_pay = 0, n_out = 0, pkt_stride = 0, payload_off = 0, out_pol_stride = 0;
    uint32_t a_secs = 0, a_df = 0, a_epoch = 0;
    uint64_t a_psn = 0;
    int64_t a_skip = 0, a_new_left = 0, a_skip_after = 0;
    sdbe_resampler::Stage *sg = nullptr;
    uint8_t *dev_out = nullptr;
    PayloadTarget pt{};
};

int plan_call(sdbe_resampler *h, const void *packets, int64_t n_packets, int32_t n_frames, uint64_t b_zero, void *out,
              int64_t out_bytes, uint32_t flags, cudaStream_t st, CallPlan &c) {
    if (n_frames < 0 || n_frames > h->cfg.max_frames)
        return fail(h, SDBE_ERR_CAPACITY, "n_frames outside [0, max_frames]");
    if (n_packets < 0 || (n_packets > 0 && !packets)) return fail(h, SDBE_ERR_ARG, "bad packets");
    c.h = h;
    c.st = st;
    c.packets = packets;
    c.n_packets = n_packets;
    c.n_frames = n_frames;
    c.b_zero = b_zero;
    c.out = out;
    c.flags = flags;
    c.aligned = (flags & SDBE_OUT_ALIGNED) != 0;
    c.framed = (flags & (SDBE_OUT_FRAMED | SDBE_OUT_ALIGNED)) != 0;
    c.n_frames_out = frames_out(h, n_frames);
    c.n_batches = batches_for(h, n_frames);
    c.n_pay = c.n_batches * kChunks;  // payload packets per pol the FFTs produce
    // Time alignment (vdif_out_net_thread.c:199-317): first block after a
    // template starts on the next second boundary if it would cross one and
    // skips the sub-packet offset; every block frames whole packets of
    // [leftover | payload] and carries the rest.
    c.a_secs = h->secs;
    c.a_df = h->df;
    c.a_psn = h->psn;
    c.a_epoch = h->ref_epoch;
    int64_t a_skip_total = h->skip_pending;
    c.n_out = c.n_pay;
    if (c.aligned) {
        if (h->align_pending) {
            c.a_secs = h->tmpl.secs_inre;
            c.a_df = h->tmpl.df_num_insec;
            int64_t skip_frames = 0;
            if (static_cast<int64_t>(c.a_df) > 125000 - c.n_pay) {
                skip_frames = 125000 - static_cast<int64_t>(c.a_df);
                c.a_df = 0;
                c.a_secs += 1;
            }
            const double skip_ps = static_cast<double>(h->tmpl.ps_early + 3715791ull);
            const double skip_samples = std::floor(skip_ps * 4096e6 / 1e12);
            a_skip_total += static_cast<int64_t>(std::floor(skip_samples / (8.0 / 2.0) / 4.0)) + skip_frames * kOutWords;
            c.a_psn = 1;
            c.a_epoch = h->tmpl.ref_epoch;
        }
        const int64_t stream_len = h->n_left + c.n_pay * kOutWords - a_skip_total;
        if (stream_len < 0) {
            c.n_out = 0;
            c.a_skip_after = -stream_len;
        } else {
            c.a_skip = a_skip_total;
            c.n_out = stream_len / kOutWords;
            c.a_new_left = stream_len - c.n_out * kOutWords;
        }
    }
    c.pkt_stride = c.framed ? kOutPkt : kOutPktData;
    c.payload_off = c.framed ? 32 : 0;
    c.out_pol_stride = c.n_out * c.pkt_stride;
    if (out_bytes < 2 * c.out_pol_stride) return fail(h, SDBE_ERR_CAPACITY, "output buffer too small");
    if (c.n_out > 0 && !out) return fail(h, SDBE_ERR_ARG, "null output");
    if (h->cfg.threshold_mode == SDBE_THRESH_FIXED && !h->thresholds_set && c.n_batches > 0)
        return fail(h, SDBE_ERR_STATE, "fixed threshold mode needs sdbe_set_state first");
    c.host_in = (flags & SDBE_IN_HOST) && n_packets > 0;
    c.host_out = (flags & SDBE_OUT_HOST) && c.n_out > 0;
    if (!c.host_in && n_packets > 0 && (reinterpret_cast<uintptr_t>(packets) & 15u))
        return fail(h, SDBE_ERR_ARG, "device packet buffer must be 16-byte aligned");
    if (!c.host_out && c.n_out > 0 && (reinterpret_cast<uintptr_t>(out) & 15u))
        return fail(h, SDBE_ERR_ARG, "device output buffer must be 16-byte aligned");
    return SDBE_OK;
}

// Payload packets [lo, hi) of both pols are final: send them to the host on
// the copy stream while the next wave computes.
int ship_call(CallPlan &c, int64_t lo, int64_t hi) {
    sdbe_resampler *h = c.h;
    if (!c.host_out || hi <= lo) return SDBE_OK;
    SDBE_CK(h, cudaEventRecord(h->wave_ev, c.st));
    SDBE_CK(h, cudaStreamWaitEvent(h->copy_out, h->wave_ev, 0));
    SDBE_CK(h, cudaMemcpy2DAsync(static_cast<uint8_t *>(c.out) + lo * c.pkt_stride, c.out_pol_stride,
                                 c.dev_out + lo * c.pkt_stride, c.out_pol_stride, (hi - lo) * c.pkt_stride, 2,
                                 cudaMemcpyDeviceToHost, h->copy_out));
    return SDBE_OK;
}

// With `batch` (sdbe_process_multi, APHIDS map) the call's unpack and zero
// fill join the batch's launches, which the caller makes after every call is
// prepared (and records the staging slots' pkt_free after them).
int prepare_call(CallPlan &c, UnpackSegs *batch = nullptr) {
    sdbe_resampler *h = c.h;
    cudaStream_t st = c.st;
    c.sg = &h->stage[h->stage_idx];
    sdbe_resampler::Stage &sg = *c.sg;
    if (c.host_in || c.host_out) h->stage_idx ^= 1;
    const uint8_t *src = static_cast<const uint8_t *>(c.packets);
    if (c.host_in) {
        int rc = grow(h, &sg.pkt, &sg.pkt_bytes, c.n_packets * kPktBytes, "packet staging");
        if (rc) return rc;
        // the slot's previous packets must have been unpacked before they are overwritten
        SDBE_CK(h, cudaStreamWaitEvent(h->copy_in, sg.pkt_free, 0));
        SDBE_CK(h, cudaMemcpyAsync(sg.pkt, c.packets, c.n_packets * kPktBytes, cudaMemcpyHostToDevice, h->copy_in));
        SDBE_CK(h, cudaEventRecord(sg.pkt_ready, h->copy_in));
        SDBE_CK(h, cudaStreamWaitEvent(st, sg.pkt_ready, 0));
        src = sg.pkt;
    }
    c.dev_out = static_cast<uint8_t *>(c.out);
    if (c.host_out) {
        int rc = grow(h, &sg.out, &sg.out_bytes, 2 * c.out_pol_stride, "output staging");
        if (rc) return rc;
        // the slot's previous payloads must have left for the host before they are overwritten
        SDBE_CK(h, cudaStreamWaitEvent(st, sg.out_free, 0));
        c.dev_out = sg.out;
    }
    // Where the FFT waves write: the output itself, or the plain payload
    // stream that the alignment step frames afterwards.
    c.pt = PayloadTarget{c.dev_out, c.out_pol_stride, c.pkt_stride, c.payload_off};
    if (c.aligned && c.n_pay > 0) {
        int rc = grow(h, &h->pay, &h->pay_bytes, 2 * c.n_pay * kOutPktData, "payload stream");
        if (rc) return rc;
        c.pt = PayloadTarget{h->pay, c.n_pay * kOutPktData, kOutPktData, 0};
    }
    const int map = h->cfg.channel_map;
    const bool mar = map == SDBE_MAP_MAR2015;
    const int32_t n_frames = c.n_frames;
    if (n_frames > 0) {
        // Mar-2015: unpack after the held frame in `raw`; otherwise straight
        // into the snapshot stream after the carried snapshots.
        uint32_t *dst = mar ? h->raw : h->spec;
        const int64_t dst_stride = mar ? h->raw_pol_stride : h->spec_pol_stride;
        const int64_t snap0 = mar ? static_cast<int64_t>(h->raw_carry) * kSnapsPerFrame : h->carry;
        SDBE_CK(h, cudaMemsetAsync(h->bitmap, 0, static_cast<size_t>(n_frames) * 256, st));
        SDBE_CK(h, cudaMemsetAsync(h->counts, 0, (static_cast<size_t>(h->cfg.max_frames) + 1) * sizeof(int32_t), st));
        if (batch && !mar) {
            unpack_segs_add(*batch, UnpackSeg{static_cast<const uint8_t *>(src), c.n_packets, c.b_zero, n_frames, map,
                                              dst, dst_stride, snap0, h->bitmap, h->counts,
                                              h->counts + h->cfg.max_frames, nullptr, 0, 0});
        } else {
            SDBE_CK(h, launch_unpack(src, c.n_packets, c.b_zero, n_frames, map, dst, dst_stride, snap0, h->bitmap,
                                     h->counts, h->counts + h->cfg.max_frames, st));
            if (c.host_in) SDBE_CK(h, cudaEventRecord(sg.pkt_free, st));
            SDBE_CK(h, launch_fill_missing(h->bitmap, n_frames, map, dst, dst_stride, snap0, st));
            h->launches += c.n_packets > 0 ? 2 : 1;
        }
        if (mar) {
            const int n_in = h->raw_carry + n_frames;
            for (int pol = 0; pol < 2 && n_in >= 2; ++pol) {
                SDBE_CK(h, launch_reorder_mar2015(h->raw + pol * h->raw_pol_stride, n_in,
                                                  h->spec + pol * h->spec_pol_stride + h->carry * kGroups, st));
                h->launches += 1;
            }
            if (n_in >= 2) {  // hold the newest frame
                for (int pol = 0; pol < 2; ++pol) {
                    uint32_t *base = h->raw + pol * h->raw_pol_stride;
                    SDBE_CK(h, cudaMemcpyAsync(base, base + static_cast<int64_t>(n_in - 1) * kSnapsPerFrame * kGroups,
                                               static_cast<size_t>(kSnapsPerFrame) * kGroups * sizeof(uint32_t),
                                               cudaMemcpyDeviceToDevice, st));
                }
            }
            h->raw_carry = 1;
        }
    }
    if (c.framed && !c.aligned && c.n_out > 0) {  // headers first, so every shipped wave is complete
        SDBE_CK(h, launch_vdif_headers(c.dev_out, c.n_out, c.out_pol_stride, h->secs, h->df, h->psn, h->ref_epoch,
                                       h->station, h->bdc, h->rx, st));
        h->launches += 1;
        const uint64_t dfs = static_cast<uint64_t>(h->df) + static_cast<uint64_t>(c.n_out);
        h->secs += static_cast<uint32_t>(dfs / 125000u);
        h->df = static_cast<uint32_t>(dfs % 125000u);
        h->psn += static_cast<uint64_t>(c.n_out);
    }
    return SDBE_OK;
}

int complete_call(CallPlan &c, sdbe_result *result) {
    sdbe_resampler *h = c.h;
    cudaStream_t st = c.st;
    if (c.aligned) {
        const uint32_t *pay_w = reinterpret_cast<const uint32_t *>(h->pay);
        const int64_t pay_ws = c.n_pay * kOutWords;
        uint32_t *cur = h->left[h->left_idx], *nxt = h->left[h->left_idx ^ 1];
        if (c.n_out > 0) {
            SDBE_CK(h, launch_align_frames(pay_w, pay_ws, cur, kOutWords, h->n_left, c.a_skip, c.n_out, c.dev_out,
                                           c.out_pol_stride, st));
            SDBE_CK(h, launch_vdif_headers(c.dev_out, c.n_out, c.out_pol_stride, c.a_secs, c.a_df, c.a_psn, c.a_epoch,
                                           h->station, h->bdc, h->rx, st));
            h->launches += 2;
        }
        if (c.a_skip_after == 0) {
            SDBE_CK(h, launch_save_leftover(pay_w, pay_ws, cur, kOutWords, h->n_left, c.a_skip, c.n_out * kOutWords,
                                            c.a_new_left, nxt, st));
            h->launches += c.a_new_left > 0 ? 1 : 0;
            h->left_idx ^= 1;
            h->n_left = c.a_new_left;
        } else {
            h->n_left = 0;
        }
        h->skip_pending = c.a_skip_after;
        h->align_pending = false;
        const uint64_t dfs = static_cast<uint64_t>(c.a_df) + static_cast<uint64_t>(c.n_out);
        h->secs = c.a_secs + static_cast<uint32_t>(dfs / 125000u);
        h->df = static_cast<uint32_t>(dfs % 125000u);
        h->psn = c.a_psn + static_cast<uint64_t>(c.n_out);
        h->ref_epoch = c.a_epoch;
        if (int rc = ship_call(c, 0, c.n_out)) return rc;
    }
    if (c.host_out) SDBE_CK(h, cudaEventRecord(c.sg->out_free, h->copy_out));
    const int64_t total = h->carry + c.n_frames_out * kSnapsPerFrame;
    const int64_t new_carry = total - c.n_batches * kBatchSnaps;
    if (c.n_batches > 0 && new_carry > 0) {
        for (int pol = 0; pol < 2; ++pol) {
            uint32_t *base = h->spec + pol * h->spec_pol_stride;
            SDBE_CK(h, cudaMemcpyAsync(base, base + c.n_batches * kBatchSnaps * kGroups,
                                       new_carry * kGroups * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
        }
    }
    h->carry = new_carry;
    h->last_stream = st;
    const bool need_sync =
        result || (!(c.flags & SDBE_ASYNC) && (c.flags & (SDBE_SYNC | SDBE_IN_HOST | SDBE_OUT_HOST)));
    if (need_sync) {
        SDBE_CK(h, cudaStreamSynchronize(st));
        if (c.host_out) SDBE_CK(h, cudaStreamSynchronize(h->copy_out));
    }
    if (result) {
        std::vector<int32_t> cnt(static_cast<size_t>(h->cfg.max_frames) + 1);
        SDBE_CK(h, cudaMemcpy(cnt.data(), h->counts, cnt.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
        int64_t acc = 0, incomplete = 0;
        for (int32_t f = 0; f < c.n_frames; ++f) {
            acc += cnt[f];
            if (cnt[f] < kPktsPerFrame) ++incomplete;
        }
        result->n_batches = c.n_batches;
        result->n_out_packets = c.n_out;
        result->packets_accepted = acc;
        result->packets_rejected = cnt[h->cfg.max_frames];
        result->frames_incomplete = incomplete;
        result->carry_snapshots = h->carry;
    }
    return SDBE_OK;
}

// fft_chain_multi for tensor-core handles (all of one precision): the first
// batches of every handle that needs thresholds in one wave, then waves of up
// to the smallest handle wave, each transform one launch over all handles.
int tc_chain_multi(std::vector<CallPlan> &cs) {
    cudaStream_t st = cs[0].st;
    const int n = static_cast<int>(cs.size());
    std::vector<int64_t> b(static_cast<size_t>(n), 0);
    std::vector<TcWaveItem> w;
    for (int i = 0; i < n; ++i) {
        sdbe_resampler *h = cs[i].h;
        if (cs[i].n_batches == 0 || h->thresholds_set) continue;
        w.push_back(TcWaveItem{h, h->spec, h->spec_pol_stride, 0, 1, cs[i].pt});
    }
    if (int rc = tc_wave_multi(w, true, st)) return rc;
    for (const auto &it : w)
        for (int i = 0; i < n; ++i)
            if (cs[i].h == it.h) {
                b[i] = 1;
                if (!cs[i].aligned)
                    if (int rc = ship_call(cs[i], 0, kChunks)) return rc;
            }
    int wave = cs[0].h->wave;
    for (const auto &c : cs) wave = std::min(wave, c.h->wave);
    while (true) {
        w.clear();
        std::vector<int> act;
        for (int i = 0; i < n; ++i) {
            if (b[i] >= cs[i].n_batches) continue;
            const int64_t nb = wave_len(cs[i].h, wave, cs[i].n_batches - b[i]);
            w.push_back(TcWaveItem{cs[i].h, cs[i].h->spec, cs[i].h->spec_pol_stride, b[i], nb, cs[i].pt});
            act.push_back(i);
        }
        if (w.empty()) break;
        if (int rc = tc_wave_multi(w, false, st)) return rc;
        for (size_t k = 0; k < act.size(); ++k) {
            const int i = act[k];
            if (!cs[i].aligned)
                if (int rc = ship_call(cs[i], b[i] * kChunks, (b[i] + w[k].nb) * kChunks)) return rc;
            b[i] += w[k].nb;
        }
    }
    return SDBE_OK;
}

// The FFT chain of several handles on one stream: the first-batch threshold
// path of every handle that needs it in one pair of launches, then waves in
// which one stage-A and one stage-BC launch cover every handle's batches.
int fft_chain_multi(std::vector<CallPlan> &cs) {
    if (cs[0].h->cfg.precision != SDBE_PRECISION_FP32) return tc_chain_multi(cs);
    sdbe_resampler *h0 = cs[0].h;
    cudaStream_t st = cs[0].st;
    const int n = static_cast<int>(cs.size());
    std::vector<int64_t> b(static_cast<size_t>(n), 0);
    {
        SegsA A{};
        SegsB B{};
        std::vector<int> first;
        for (int i = 0; i < n; ++i) {
            sdbe_resampler *h = cs[i].h;
            if (cs[i].n_batches == 0 || h->thresholds_set) continue;
            A.s[A.n] = SegA{h->spec, h->ts, h->spec_pol_stride, 0, kBatchSnaps, h->ts_pol_stride, A.n_items};
            A.n_items += 2 * kBatchSnaps;
            ++A.n;
            ResampleOut o{};
            o.fout = h->fout;
            o.fout_pol_stride = static_cast<int64_t>(kChunks) * kNC;
            o.partials = h->partials;
            B.s[B.n] = SegB{h->ts, h->ts_pol_stride, B.n_items, kChunks, h->skip, o};
            B.n_items += 2 * kChunks;
            ++B.n;
            first.push_back(i);
        }
        if (!first.empty()) {
            SDBE_CK(h0, launch_swarm_c2r_segs(A, h0->tw, st));
            SDBE_CK(h0, launch_resample_segs(1, B, h0->tw, st));
            h0->launches += 2;
            WinUpds U{};
            for (int i : first) {
                sdbe_resampler *h = cs[i].h;
                const PayloadTarget &t = cs[i].pt;
                SDBE_CK(h, launch_finalize_thresholds(h->partials, kChunks, h->cfg.pol1_uses_pol0_threshold, h->thr, st));
                SDBE_CK(h, launch_quantize_chunks(h->fout, static_cast<int64_t>(kChunks) * kNC, kChunks, h->thr, t.base,
                                                  t.pol_stride, t.pkt_stride, t.payload_off, 0, st));
                h->thresholds_set = true;
                h->launches += 2;
                h->stream_batch = 0;
                window_step(h, h->partials, 1, true, U);
                b[i] = 1;
                if (!cs[i].aligned)
                    if (int rc = ship_call(cs[i], 0, kChunks)) return rc;
            }
            if (U.n) {
                SDBE_CK(h0, launch_window_update(U, st));
                h0->launches += 1;
            }
        }
    }
    int wave = h0->wave;
    for (const auto &c : cs) wave = std::min(wave, c.h->wave);
    bool any_win = false;
    for (const auto &c : cs) any_win = any_win || c.h->cfg.threshold_mode == SDBE_THRESH_WINDOW;
    while (true) {
        SegsA A{};
        SegsB B{};
        std::vector<std::pair<int, int64_t>> act;  // handle index, batches this wave
        for (int i = 0; i < n; ++i) {
            sdbe_resampler *h = cs[i].h;
            if (b[i] >= cs[i].n_batches) continue;
            const int64_t nb = wave_len(h, wave, cs[i].n_batches - b[i]);
            A.s[A.n] = SegA{h->spec, h->ts, h->spec_pol_stride, b[i] * kBatchSnaps, nb * kBatchSnaps, h->ts_pol_stride,
                            A.n_items};
            A.n_items += 2 * nb * kBatchSnaps;
            ++A.n;
            const PayloadTarget &t = cs[i].pt;
            ResampleOut o{};
            o.out = t.base;
            o.out_pol_stride = t.pol_stride;
            o.pkt_stride = t.pkt_stride;
            o.payload_off = t.payload_off;
            o.pkt0 = b[i] * kChunks;
            o.thr = h->thr;
            o.partials = h->cfg.threshold_mode == SDBE_THRESH_WINDOW ? h->wpart : nullptr;
            B.s[B.n] = SegB{h->ts, h->ts_pol_stride, B.n_items, static_cast<int>(nb * kChunks), h->skip, o};
            B.n_items += 2 * nb * kChunks;
            ++B.n;
            act.emplace_back(i, nb);
        }
        if (act.empty()) break;
        size_t slot;
        SDBE_CK(h0, timed_begin(h0, 0, A.n_items, st, &slot));
        SDBE_CK(h0, launch_swarm_c2r_segs(A, h0->tw, st));
        SDBE_CK(h0, timed_end(h0, slot, st));
        SDBE_CK(h0, timed_begin(h0, 1, B.n_items, st, &slot));
        SDBE_CK(h0, launch_resample_segs(any_win ? 3 : 0, B, h0->tw, st));
        SDBE_CK(h0, timed_end(h0, slot, st));
        h0->launches += 2;
        WinUpds U{};
        for (auto [i, nb] : act) window_step(cs[i].h, cs[i].h->wpart, nb, false, U);
        if (U.n) {
            SDBE_CK(h0, launch_window_update(U, st));
            h0->launches += 1;
        }
        for (auto [i, nb] : act) {
            if (!cs[i].aligned)
                if (int rc = ship_call(cs[i], b[i] * kChunks, (b[i] + nb) * kChunks)) return rc;
            b[i] += nb;
        }
    }
    return SDBE_OK;
}
}  // namespace sdbe

extern "C" {

int sdbe_create(const sdbe_config *cfg, sdbe_resampler **out) {
    if (!cfg || !out) return fail(nullptr, SDBE_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->max_frames < 1 || cfg->max_frames > (1 << 16))
        return fail(nullptr, SDBE_ERR_ARG, "max_frames must be in [1, 65536]");
    const int skip = static_cast<int>(cfg->trim_mhz * 1e6 / (4576e6 / kNB));  // .cu:269
    if (cfg->trim_mhz < 0 || skip > kMaxSkip) return fail(nullptr, SDBE_ERR_ARG, "trim_mhz must be in [0, 240]");
    if (cfg->threshold_mode != SDBE_THRESH_FIRST_BATCH && cfg->threshold_mode != SDBE_THRESH_FIXED &&
        cfg->threshold_mode != SDBE_THRESH_WINDOW)
        return fail(nullptr, SDBE_ERR_ARG, "unknown threshold_mode");
    if (cfg->threshold_window < 0 || cfg->threshold_window > (1 << 16))
        return fail(nullptr, SDBE_ERR_ARG, "threshold_window in [0, 65536]");
    if (cfg->channel_map != SDBE_MAP_APHIDS && cfg->channel_map != SDBE_MAP_MAR2015)
        return fail(nullptr, SDBE_ERR_ARG, "unknown channel_map");
    if (cfg->wave_batches < 0 || cfg->wave_batches > kDefaultWave)
        return fail(nullptr, SDBE_ERR_ARG, "wave_batches in [0, 64]");
    if (cfg->precision != SDBE_PRECISION_FP32 && cfg->precision != SDBE_PRECISION_TC16 &&
        cfg->precision != SDBE_PRECISION_TC16_FAST)
        return fail(nullptr, SDBE_ERR_ARG, "unknown precision");
    if (cfg->stage_launches != 0 && cfg->stage_launches != SDBE_STAGES_FUSED && cfg->stage_launches != SDBE_STAGES_SPLIT)
        return fail(nullptr, SDBE_ERR_ARG, "stage_launches must be 0, SDBE_STAGES_FUSED or SDBE_STAGES_SPLIT");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
        cudaGetLastError();
        return fail(nullptr, SDBE_ERR_ARG, "no such CUDA device");
    }
    DeviceGuard g(cfg->device);
    if (!g.ok) return fail(nullptr, SDBE_ERR_CUDA, "cudaSetDevice failed");
    sdbe_resampler *h = new sdbe_resampler();
    h->cfg = *cfg;
    h->skip = skip;
    // Default wave: 64 batches (fewer launches: each CTA loads its twiddle
    // tables and waits on its first chunk once per launch; the persistent
    // grid's last round is a smaller share), but no more than one call can
    // produce, so that small handles do not hold 37.5 MB of stage-A scratch
    // per batch they never use.
    const int call_batches = static_cast<int>((kBatchSnaps - 1 + static_cast<int64_t>(cfg->max_frames) * kSnapsPerFrame) /
                                              kBatchSnaps);
    h->wave = cfg->wave_batches > 0 ? cfg->wave_batches : std::max(1, std::min(kDefaultWave, call_batches));
    h->max_snaps = static_cast<int64_t>(cfg->max_frames) * kSnapsPerFrame + kBatchSnaps;
    h->spec_pol_stride = h->max_snaps * kGroups;
    h->ts_pol_stride = static_cast<int64_t>(h->wave) * kBatchSnaps * kNA;
    auto bail = [&](int code, const std::string &m) {
        free_all(h);
        delete h;
        cudaGetLastError();
        return fail(nullptr, code, m);
    };
    if (configure_fft_kernels() != cudaSuccess) return bail(SDBE_ERR_CUDA, "kernel attribute setup failed");
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->copy_in, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&h->copy_out, cudaStreamNonBlocking) != cudaSuccess)
        return bail(SDBE_ERR_CUDA, "stream creation failed");
    bool ev_ok = cudaEventCreateWithFlags(&h->wave_ev, cudaEventDisableTiming) == cudaSuccess;
    for (auto &sg : h->stage)
        ev_ok = ev_ok && cudaEventCreateWithFlags(&sg.pkt_ready, cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&sg.pkt_free, cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&sg.out_free, cudaEventDisableTiming) == cudaSuccess;
    if (!ev_ok) return bail(SDBE_ERR_CUDA, "event creation failed");
    if (build_twiddles(h->tw, &h->tw_storage) != cudaSuccess) return bail(SDBE_ERR_NOMEM, "twiddle tables");
    bool ok = cudaMalloc(&h->spec, 2 * h->spec_pol_stride * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&h->bitmap, static_cast<size_t>(cfg->max_frames) * 256) == cudaSuccess &&
              cudaMalloc(&h->counts, (static_cast<size_t>(cfg->max_frames) + 1) * sizeof(int32_t)) == cudaSuccess &&
              cudaMalloc(&h->ts, 2 * h->ts_pol_stride * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&h->fout, 2 * static_cast<size_t>(kChunks) * kNC * sizeof(float)) == cudaSuccess &&
              cudaMalloc(&h->partials, 2 * kChunks * 3 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&h->thr, 8 * sizeof(float)) == cudaSuccess;
    if (ok && cfg->threshold_mode == SDBE_THRESH_WINDOW) {
        h->window = cfg->threshold_window > 0 ? cfg->threshold_window : 64;
        ok = cudaMalloc(&h->wring, 2 * static_cast<size_t>(h->window) * 3 * sizeof(double)) == cudaSuccess &&
             cudaMalloc(&h->wpart, 2 * static_cast<size_t>(h->wave) * kChunks * 3 * sizeof(double)) == cudaSuccess;
    }
    ok = ok && cudaMalloc(&h->left[0], 2 * kOutWords * sizeof(uint32_t)) == cudaSuccess &&
         cudaMalloc(&h->left[1], 2 * kOutWords * sizeof(uint32_t)) == cudaSuccess;
    if (ok && cfg->channel_map == SDBE_MAP_MAR2015) {
        h->raw_pol_stride = (static_cast<int64_t>(cfg->max_frames) + 1) * kSnapsPerFrame * kGroups;
        ok = cudaMalloc(&h->raw, 2 * h->raw_pol_stride * sizeof(uint32_t)) == cudaSuccess;
    }
    if (!ok) return bail(SDBE_ERR_NOMEM, "device buffer allocation failed");
    if (cudaMemset(h->thr, 0, 8 * sizeof(float)) != cudaSuccess) return bail(SDBE_ERR_CUDA, "memset");
    *out = h;
    return SDBE_OK;
}

int sdbe_destroy(sdbe_resampler *h) {
    if (!h) return SDBE_OK;
    DeviceGuard g(h->cfg.device);
    cudaDeviceSynchronize();
    free_all(h);
    delete h;
    return SDBE_OK;
}

int64_t sdbe_output_bytes(const sdbe_resampler *h, int32_t n_frames, uint32_t flags) {
    if (!h || n_frames < 0) return -1;
    const int64_t n_out = batches_for(h, n_frames) * kChunks;
    if (flags & SDBE_OUT_ALIGNED) return 2 * ((h->n_left + n_out * kOutWords) / kOutWords) * kOutPkt;
    const int64_t pkt = (flags & SDBE_OUT_FRAMED) ? kOutPkt : kOutPktData;
    return 2 * n_out * pkt;
}

int sdbe_process(sdbe_resampler *h, const void *packets, int64_t n_packets, int32_t n_frames, uint64_t b_zero,
                 void *out, int64_t out_bytes, uint32_t flags, void *stream, sdbe_result *result) {
    if (!h) return fail(nullptr, SDBE_ERR_ARG, "null handle");
    DeviceGuard g(h->cfg.device);
    if (!g.ok) return fail(h, SDBE_ERR_CUDA, "cudaSetDevice failed");
    CallPlan c;
    int rc = plan_call(h, packets, n_packets, n_frames, b_zero, out, out_bytes, flags, pick(h, stream), c);
    if (!rc) rc = prepare_call(c);
    if (!rc && h->cfg.precision != SDBE_PRECISION_FP32) {
        rc = tc_chain(h, h->spec, h->spec_pol_stride, c.n_batches, c.pt, c.st,
                      [&](int64_t lo, int64_t hi) { return c.aligned ? SDBE_OK : ship_call(c, lo, hi); });
    } else if (!rc) {
        rc = fft_chain(h, h->spec, h->spec_pol_stride, c.n_batches, c.pt, c.st,
                       [&](int64_t lo, int64_t hi) { return c.aligned ? SDBE_OK : ship_call(c, lo, hi); });
    }
    if (!rc) rc = complete_call(c, result);
    return rc;
}

int sdbe_process_multi(sdbe_resampler *const *hs, const sdbe_stream_desc *d, int32_t n, uint32_t flags, void *stream,
                       sdbe_result *results) {
    if (!hs || !d || n < 1 || n > kMaxSegs) return fail(nullptr, SDBE_ERR_ARG, "need 1..32 handles and descriptors");
    for (int i = 0; i < n; ++i) {
        if (!hs[i]) return fail(nullptr, SDBE_ERR_ARG, "null handle");
        if (hs[i]->cfg.device != hs[0]->cfg.device) return fail(hs[i], SDBE_ERR_ARG, "handles on different devices");
        if (hs[i]->cfg.precision != hs[0]->cfg.precision)
            return fail(hs[i], SDBE_ERR_ARG, "sdbe_process_multi needs handles of one precision");
        for (int j = 0; j < i; ++j)
            if (hs[j] == hs[i]) return fail(hs[i], SDBE_ERR_ARG, "a handle appears twice");
    }
    DeviceGuard g(hs[0]->cfg.device);
    if (!g.ok) return fail(hs[0], SDBE_ERR_CUDA, "cudaSetDevice failed");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : hs[0]->stream;
    std::vector<CallPlan> c(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {  // every check before any work is queued
        int rc = plan_call(hs[i], d[i].packets, d[i].n_packets, d[i].n_frames, d[i].b_zero, d[i].out, d[i].out_bytes,
                           flags, st, c[i]);
        if (rc) return rc;
    }
    // every stream's unpack and zero fill in one launch each
    UnpackSegs U{};
    for (auto &ci : c)
        if (int rc = prepare_call(ci, &U)) return rc;
    if (U.n > 0) {
        SDBE_CK(hs[0], launch_unpack_segs(U, st));
        for (auto &ci : c)
            if (ci.host_in && ci.n_frames > 0 && ci.h->cfg.channel_map != SDBE_MAP_MAR2015)
                SDBE_CK(ci.h, cudaEventRecord(ci.sg->pkt_free, st));
        SDBE_CK(hs[0], launch_fill_missing_segs(U, st));
        hs[0]->launches += U.blocks > 0 ? 2 : 1;
    }
    if (int rc = fft_chain_multi(c)) return rc;
    for (int i = 0; i < n; ++i)
        if (int rc = complete_call(c[i], results ? results + i : nullptr)) return rc;
    return SDBE_OK;
}

int sdbe_header_template(int32_t t0_sec, int32_t t0_clk, uint32_t ref_epoch, sdbe_time_template *out) {
    if (!out) return fail(nullptr, SDBE_ERR_ARG, "null argument");
    constexpr int32_t kClkPerSec = 286000000, kBframeClk = 262144;  // beng_reform.c:25-27
    // get_beng_t0: one B-frame earlier (beng_reform.c:112-126)
    int32_t sec = t0_sec, clk = t0_clk - kBframeClk;
    if (clk < 0) {
        sec -= 1;
        clk += kClkPerSec;
    }
    // fill_vdif_header_template: one B-frame later (beng_reform.c:192-198)
    clk += kBframeClk;
    if (clk > kClkPerSec) {
        sec += 1;
        clk %= kClkPerSec;
    }
    const double frame_full = (125000 * 1.0) * (static_cast<double>(clk) / static_cast<double>(kClkPerSec));
    const double frame_ceil = std::ceil(frame_full);
    const double frac = frame_ceil - frame_full;
    out->secs_inre = static_cast<uint32_t>(sec);
    out->df_num_insec = static_cast<uint32_t>(frame_ceil);
    out->ps_early = static_cast<uint64_t>(std::floor(frac * (1e12 / 125000)));
    out->ref_epoch = ref_epoch;
    out->reserved = 0;
    return SDBE_OK;
}

int sdbe_align_start(sdbe_resampler *h, const sdbe_time_template *t) {
    if (!h || !t) return fail(h, SDBE_ERR_ARG, "null argument");
    if (t->df_num_insec > 125000u) return fail(h, SDBE_ERR_ARG, "df_num_insec must be <= 125000");
    h->tmpl = *t;
    h->align_pending = true;
    h->skip_pending = 0;
    h->n_left = 0;
    return SDBE_OK;
}

int sdbe_sync(sdbe_resampler *h) {
    if (!h) return fail(nullptr, SDBE_ERR_ARG, "null handle");
    DeviceGuard g(h->cfg.device);
    SDBE_CK(h, cudaStreamSynchronize(h->copy_in));
    if (h->last_stream) SDBE_CK(h, cudaStreamSynchronize(h->last_stream));
    SDBE_CK(h, cudaStreamSynchronize(h->stream));
    SDBE_CK(h, cudaStreamSynchronize(h->copy_out));
    return SDBE_OK;
}

int sdbe_get_state(sdbe_resampler *h, sdbe_state *st) {
    if (!h || !st) return fail(h, SDBE_ERR_ARG, "null argument");
    DeviceGuard g(h->cfg.device);
    float thr[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    SDBE_CK(h, cudaDeviceSynchronize());
    if (h->thresholds_set) SDBE_CK(h, cudaMemcpy(thr, h->thr, sizeof(thr), cudaMemcpyDeviceToHost));
    std::memset(st, 0, sizeof(*st));
    st->threshold[0] = thr[4];
    st->threshold[1] = thr[5];
    st->offset[0] = thr[6];
    st->offset[1] = thr[7];
    st->thresholds_set = h->thresholds_set ? 1 : 0;
    st->carry_snapshots = static_cast<int32_t>(h->carry);
    st->secs_inre = h->secs;
    st->df_num_insec = h->df;
    st->edh_psn = h->psn;
    st->ref_epoch = h->ref_epoch;
    st->station_id = h->station;
    st->bdc_sideband = h->bdc;
    st->rx_sideband = h->rx;
    return SDBE_OK;
}

int sdbe_set_state(sdbe_resampler *h, const sdbe_state *st) {
    if (!h || !st) return fail(h, SDBE_ERR_ARG, "null argument");
    if (st->df_num_insec >= 125000u) return fail(h, SDBE_ERR_ARG, "df_num_insec must be < 125000");
    DeviceGuard g(h->cfg.device);
    const bool p1 = h->cfg.pol1_uses_pol0_threshold != 0;
    float thr[8] = {st->threshold[0], p1 ? st->threshold[0] : st->threshold[1],
                    st->offset[0],    p1 ? st->offset[0] : st->offset[1],
                    st->threshold[0], st->threshold[1], st->offset[0], st->offset[1]};
    SDBE_CK(h, cudaDeviceSynchronize());
    SDBE_CK(h, cudaMemcpy(h->thr, thr, sizeof(thr), cudaMemcpyHostToDevice));
    h->thresholds_set = (st->threshold[0] != 0.f || st->threshold[1] != 0.f);
    if (st->carry_snapshots == 0) h->carry = 0;
    h->secs = st->secs_inre;
    h->df = st->df_num_insec;
    h->psn = st->edh_psn;
    h->ref_epoch = st->ref_epoch;
    h->station = st->station_id;
    h->bdc = st->bdc_sideband;
    h->rx = st->rx_sideband;
    return SDBE_OK;
}

int sdbe_reset(sdbe_resampler *h) {
    if (!h) return fail(nullptr, SDBE_ERR_ARG, "null handle");
    h->thresholds_set = false;
    h->carry = 0;
    h->stream_batch = 0;
    h->raw_carry = 0;
    h->n_left = 0;
    h->skip_pending = 0;
    return SDBE_OK;
}

int sdbe_profile_enable(sdbe_resampler *h, int32_t enable) {
    if (!h) return fail(nullptr, SDBE_ERR_ARG, "null handle");
    h->prof = enable != 0;
    return SDBE_OK;
}

int sdbe_profile_read(sdbe_resampler *h, sdbe_profile *out) {
    if (!h || !out) return fail(h, SDBE_ERR_ARG, "null argument");
    DeviceGuard g(h->cfg.device);
    std::memset(out, 0, sizeof(*out));
    for (size_t i = 0; i < h->n_timed; ++i) {
        auto &t = h->timed[i];
        SDBE_CK(h, cudaEventSynchronize(t.b));
        float ms = 0.f;
        SDBE_CK(h, cudaEventElapsedTime(&ms, t.a, t.b));
        if (t.kind == 0) {
            out->stage_a_launches += 1;
            out->stage_a_snapshots += t.units;
            out->stage_a_ms += ms;
        } else if (t.kind == 2) {
            out->fused_launches += 1;
            out->fused_chunks += t.units;
            out->fused_ms += ms;
        } else {
            out->stage_bc_launches += 1;
            out->stage_bc_chunks += t.units;
            out->stage_bc_ms += ms;
        }
    }
    out->launches = h->launches;
    h->n_timed = 0;
    h->launches = 0;
    return SDBE_OK;
}

int sdbe_last_error(const sdbe_resampler *h, char *buf, size_t n) {
    if (!buf || n == 0) return SDBE_ERR_ARG;
    const std::string &m = h ? h->err : thread_error();
    const size_t k = std::min(n - 1, m.size());
    std::memcpy(buf, m.data(), k);
    buf[k] = '\0';
    return SDBE_OK;
}

int sdbe_host_alloc(void **ptr, size_t bytes) {
    if (!ptr) return fail(nullptr, SDBE_ERR_ARG, "null argument");
    if (cudaMallocHost(ptr, bytes) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(nullptr, SDBE_ERR_NOMEM, "cudaMallocHost failed");
    }
    return SDBE_OK;
}

int sdbe_host_free(void *ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) return fail(nullptr, SDBE_ERR_CUDA, "cudaFreeHost failed");
    return SDBE_OK;
}

// The stage entry points' device pointers: the kernels move data in 8- and
// 16-byte vectors (and stage BC bulk-prefetches its input), so a pointer not
// aligned to its kernel's width is refused with SDBE_ERR_ARG here rather
// than faulting the device.
static bool unaligned(const void *p, uintptr_t bytes) { return (reinterpret_cast<uintptr_t>(p) & (bytes - 1)) != 0; }

int sdbe_vdif_to_beng(const void *packets, int64_t n_packets, uint64_t b_zero, int32_t n_frames, int32_t channel_map,
                      int8_t *beng0, int8_t *beng1, void *stream) {
    if (n_frames < 0 || n_packets < 0 || (n_frames > 0 && (!beng0 || !beng1)) || (n_packets > 0 && !packets))
        return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    if ((n_packets > 0 && unaligned(packets, 16)) || unaligned(beng0, 16) || unaligned(beng1, 16))
        return fail(nullptr, SDBE_ERR_ARG, "packets and B-engine buffers must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = static_cast<size_t>(n_frames) * kSnapsPerFrame * kChannels * 2;
    SDBE_CK(nullptr, cudaMemsetAsync(beng0, 0, bytes, st));
    SDBE_CK(nullptr, cudaMemsetAsync(beng1, 0, bytes, st));
    SDBE_CK(nullptr, launch_vdif_to_beng_ref(packets, n_packets, b_zero, n_frames, channel_map, beng0, beng1, st));
    return SDBE_OK;
}

int sdbe_unpack(const void *packets, int64_t n_packets, uint64_t b_zero, int32_t n_frames, int32_t channel_map,
                uint32_t *spec, int64_t pol_stride_words, int64_t snap0, uint32_t *bitmap, int32_t *frame_counts,
                int32_t *rejected, void *stream) {
    if (n_frames < 0 || n_packets < 0 || !spec || !bitmap || !frame_counts || !rejected || snap0 < 0 ||
        (n_packets > 0 && !packets))
        return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    if ((n_packets > 0 && unaligned(packets, 16)) || unaligned(spec, 4))
        return fail(nullptr, SDBE_ERR_ARG, "packets must be 16-byte aligned, spectra 4-byte aligned");
    SDBE_CK(nullptr, launch_unpack(packets, n_packets, b_zero, n_frames, channel_map, spec, pol_stride_words, snap0,
                                   bitmap, frame_counts, rejected, static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

int sdbe_fill_missing(const uint32_t *bitmap, int32_t n_frames, int32_t channel_map, uint32_t *spec,
                      int64_t pol_stride_words, int64_t snap0, void *stream) {
    if (n_frames < 0 || !bitmap || !spec || snap0 < 0) return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    SDBE_CK(nullptr, launch_fill_missing(bitmap, n_frames, channel_map, spec, pol_stride_words, snap0,
                                         static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

int sdbe_beng_to_complex(const int8_t *beng, int64_t n_spectra, void *out_c64, void *stream) {
    if (n_spectra < 0 || (n_spectra > 0 && (!beng || !out_c64))) return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    if (unaligned(beng, 2) || unaligned(out_c64, 8))
        return fail(nullptr, SDBE_ERR_ARG, "B-engine input must be 2-byte, complex output 8-byte aligned");
    SDBE_CK(nullptr, launch_beng_to_complex(beng, n_spectra, out_c64, static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

int sdbe_swarm_c2r(sdbe_resampler *h, const uint32_t *spec, int64_t n_snapshots, float *out, void *stream) {
    if (!h || n_snapshots < 0 || (n_snapshots > 0 && (!spec || !out))) return fail(h, SDBE_ERR_ARG, "bad argument");
    if (unaligned(spec, 16) || unaligned(out, 16)) return fail(h, SDBE_ERR_ARG, "spectra and output must be 16-byte aligned");
    DeviceGuard g(h->cfg.device);
    if (h->cfg.precision != SDBE_PRECISION_FP32) return tc_swarm_c2r(h, spec, n_snapshots, out, pick(h, stream));
    SDBE_CK(h, launch_swarm_c2r(spec, 0, 0, n_snapshots, 1, out, 0, h->tw, pick(h, stream)));
    return SDBE_OK;
}

int sdbe_swarm_r2c(sdbe_resampler *h, const float *in, int64_t n_chunks, void *out_c64, void *stream) {
    if (!h || n_chunks < 0 || (n_chunks > 0 && (!in || !out_c64))) return fail(h, SDBE_ERR_ARG, "bad argument");
    if (unaligned(in, 8) || unaligned(out_c64, 8)) return fail(h, SDBE_ERR_ARG, "input and output must be 8-byte aligned");
    DeviceGuard g(h->cfg.device);
    SDBE_CK(h, launch_swarm_r2c(in, n_chunks, out_c64, h->tw, pick(h, stream)));
    return SDBE_OK;
}

int sdbe_r2dbe_c2r(sdbe_resampler *h, const void *in_c64, int64_t n_chunks, int32_t skip_chan, float *out,
                   void *stream) {
    if (!h || n_chunks < 0 || skip_chan < 0 || skip_chan > kMaxSkip || (n_chunks > 0 && (!in_c64 || !out)))
        return fail(h, SDBE_ERR_ARG, "bad argument");
    if (unaligned(in_c64, 8) || unaligned(out, 8)) return fail(h, SDBE_ERR_ARG, "input and output must be 8-byte aligned");
    DeviceGuard g(h->cfg.device);
    SDBE_CK(h, launch_r2dbe_c2r(in_c64, kMB + 1, n_chunks, skip_chan, out, h->tw, pick(h, stream)));
    return SDBE_OK;
}

int sdbe_resample_chunks(sdbe_resampler *h, const float *in, int64_t n_chunks, float *out, void *stream) {
    if (!h || n_chunks < 0 || (n_chunks > 0 && (!in || !out))) return fail(h, SDBE_ERR_ARG, "bad argument");
    if (unaligned(in, 16) || unaligned(out, 16)) return fail(h, SDBE_ERR_ARG, "input and output must be 16-byte aligned");
    DeviceGuard g(h->cfg.device);
    if (h->cfg.precision != SDBE_PRECISION_FP32) return tc_resample_chunks(h, in, n_chunks, out, pick(h, stream));
    ResampleOut o{};
    o.fout = out;
    SDBE_CK(h, launch_resample(2, in, 0, h->skip, n_chunks, 1, o, h->tw, pick(h, stream)));
    return SDBE_OK;
}

int sdbe_summary_stats(const float *in, int64_t n, double *out_host, void *stream) {
    if (!in || !out_host || n < 2) return fail(nullptr, SDBE_ERR_ARG, "need n >= 2 and non-null pointers");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int blocks = stats_partial_blocks(n);
    void *scr = nullptr;  // this thread's reusable scratch: the call waits for its stream below
    SDBE_CK(nullptr, thread_scratch(static_cast<size_t>(blocks) * 2 * sizeof(double), &scr));
    double *part = static_cast<double *>(scr);
    std::vector<double> hp(static_cast<size_t>(blocks) * 2);
    float shift = 0.f;  // the partial sums are of x - in[0]
    cudaError_t e = launch_stats_partial(in, n, part, blocks, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&shift, in, sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(nullptr, SDBE_ERR_CUDA, std::string("summary_stats: ") + cudaGetErrorString(e));
    double s1 = 0.0, s2 = 0.0;
    for (int b = 0; b < blocks; ++b) {
        s1 += hp[2 * b];
        s2 += hp[2 * b + 1];
    }
    const double nn = static_cast<double>(n);
    const double dmean = s1 / nn;
    out_host[0] = static_cast<double>(shift) + dmean;
    out_host[1] = std::sqrt((s2 - s1 * dmean) / (nn - 1.0));
    return SDBE_OK;
}

int sdbe_quantize2bit(const float *in, uint32_t *out, int64_t n, float thresh, float offset, void *stream) {
    if (n < 0 || (n % 16) != 0 || (n > 0 && (!in || !out))) return fail(nullptr, SDBE_ERR_ARG, "n must be a multiple of 16");
    if (unaligned(in, 16) || unaligned(out, 4)) return fail(nullptr, SDBE_ERR_ARG, "input must be 16-byte, output 4-byte aligned");
    SDBE_CK(nullptr, launch_quantize_flat(in, out, n, thresh, offset, static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

int sdbe_vdif_headers(void *frames, int64_t n_pkts, int64_t pol_stride_bytes, uint32_t secs0, uint32_t df0,
                      uint64_t psn0, uint32_t ref_epoch, uint32_t station_id, uint32_t bdc_sideband,
                      uint32_t rx_sideband, void *stream) {
    if (n_pkts < 0 || (n_pkts > 0 && !frames) || df0 >= 125000u || (pol_stride_bytes & 15) ||
        (reinterpret_cast<uintptr_t>(frames) & 15u))
        return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    SDBE_CK(nullptr, launch_vdif_headers(frames, n_pkts, pol_stride_bytes, secs0, df0, psn0, ref_epoch, station_id,
                                         bdc_sideband, rx_sideband, static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

int sdbe_reorder_mar2015(const uint32_t *spec_in, int32_t n_frames, uint32_t *spec_out, void *stream) {
    if (n_frames < 2 || !spec_in || !spec_out) return fail(nullptr, SDBE_ERR_ARG, "need n_frames >= 2");
    SDBE_CK(nullptr, launch_reorder_mar2015(spec_in, n_frames, spec_out, static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

}  // extern "C"
