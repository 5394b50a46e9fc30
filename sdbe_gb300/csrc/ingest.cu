// Group assembly for packets as received: the ingest thread's windowing,
// limits and flush policy (software/aphids/vdif_in_net_thread.c:255-500,
// vdif_in_databuf.c:96-167) decided on the device from the packet headers
// (k_policy.cu), then the scatter, zero fill and resampling of every shipped
// group.  The host keeps the ring's life cycle: it reads the batch's result
// (ships, touched groups, the state after the batch) and launches the work.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "handle.cuh"

namespace sdbe {
namespace {

constexpr int kRing = 4;                                  // BENG_GROUPS_IN_BUFFER
constexpr int kGroupFrames = 143;                         // BENG_FRAMES_PER_GROUP
constexpr int64_t kGroupPackets = int64_t(kGroupFrames) * kPktsPerFrame;  // 292864
constexpr int64_t kGroupSnaps = int64_t(kGroupFrames) * kSnapsPerFrame;   // 18304 = 128 batches
constexpr int64_t kGroupPkts = int64_t(kGroupFrames) * kSnapsPerFrame / kBatchSnaps * kChunks;  // 16384 per pol

int64_t group_bytes(uint32_t flags) { return 2 * kGroupPkts * ((flags & SDBE_OUT_FRAMED) ? kOutPkt : kOutPktData); }

struct Policy {  // the part of the handle the policy changes
    int64_t b_first, ref;
    int64_t count[kRing];
    std::vector<int32_t> fcount;  // [kRing][143]
    sdbe_ingest_stats st;
};

Policy snapshot(const sdbe_resampler *h) {
    Policy p{h->b_first, h->ing_ref, {}, h->g_fcount, h->ing};
    for (int i = 0; i < kRing; ++i) p.count[i] = h->g_count[i];
    return p;
}

void commit(sdbe_resampler *h, const Policy &p) {
    h->b_first = p.b_first;
    h->ing_ref = p.ref;
    for (int i = 0; i < kRing; ++i) h->g_count[i] = p.count[i];
    h->g_fcount = p.fcount;
    h->ing = p.st;
    h->ing.b_first = p.b_first;
}

int64_t group_start(const Policy &p, int64_t g) { return p.b_first + 1 + kGroupFrames * g; }

void ship(Policy &p, std::vector<int64_t> &ships) {
    const int s = static_cast<int>(p.ref % kRing);
    ships.push_back(p.ref);
    p.st.groups_shipped += 1;
    if (p.count[s] < kGroupPackets) p.st.groups_incomplete += 1;
    p.count[s] = 0;
    std::fill(p.fcount.begin() + s * kGroupFrames, p.fcount.begin() + (s + 1) * kGroupFrames, 0);
    p.ref += 1;
}

// The state after a batch from the device walk.
Policy after_batch(const sdbe_resampler *h, const PolOut &r) {
    Policy p = snapshot(h);
    p.b_first = r.s.b_first;
    p.ref = r.s.ref;
    for (int i = 0; i < kRing; ++i) p.count[i] = r.s.count[i];
    p.fcount.assign(r.s.fcount, r.s.fcount + kRing * kGroupFrames);
    int64_t *st[8] = {&p.st.packets, &p.st.invalid, &p.st.before_start, &p.st.too_far_ahead, &p.st.used,
                      &p.st.overflow, &p.st.groups_shipped, &p.st.groups_incomplete};
    for (int i = 0; i < 8; ++i) *st[i] = r.s.st[i];
    return p;
}

int ensure_ring(sdbe_resampler *h) {
    if (h->ring) return SDBE_OK;
    const size_t words = size_t(2) * kRing * kGroupSnaps * kGroups;
    if (cudaMalloc(&h->ring, words * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc(&h->ring_bitmap, size_t(kRing) * kGroupFrames * 256) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDBE_ERR_NOMEM, "cannot allocate the group ring");
    }
    SDBE_CK(h, cudaMemsetAsync(h->ring_bitmap, 0, size_t(kRing) * kGroupFrames * 256, h->stream));
    return SDBE_OK;
}

// Device work for one policy step: scatter the accepted packets of every
// touched group, ship (zero fill + resample) the shipped ones, in group order.
int run_device(sdbe_resampler *h, const Policy &after, const uint8_t *dev_pkts, int64_t n, const uint8_t *dev_accept,
               const std::vector<int64_t> &ships, const std::vector<int64_t> &touched, uint8_t *dev_out,
               uint32_t flags, cudaStream_t st) {
    const bool framed = (flags & SDBE_OUT_FRAMED) != 0;
    const int64_t gbytes = group_bytes(flags);
    std::vector<int64_t> groups(touched);
    groups.insert(groups.end(), ships.begin(), ships.end());
    std::sort(groups.begin(), groups.end());
    groups.erase(std::unique(groups.begin(), groups.end()), groups.end());
    const int64_t pol_stride = int64_t(kRing) * kGroupSnaps * kGroups;
    const int map = h->cfg.channel_map;
    int64_t out_idx = 0;
    for (int64_t g : groups) {
        const int s = static_cast<int>(g % kRing);
        uint32_t *spec = h->ring + s * kGroupSnaps * kGroups;
        uint32_t *bmp = h->ring_bitmap + static_cast<int64_t>(s) * kGroupFrames * 64;
        const uint64_t b_zero = static_cast<uint64_t>(group_start(after, g));
        if (std::binary_search(touched.begin(), touched.end(), g) && n > 0) {
            SDBE_CK(h, launch_unpack(dev_pkts, n, b_zero, kGroupFrames, map, spec, pol_stride, 0, bmp, nullptr, nullptr,
                                     st, dev_accept));
            h->launches += 1;
        }
        if (std::binary_search(ships.begin(), ships.end(), g)) {
            SDBE_CK(h, launch_fill_missing(bmp, kGroupFrames, map, spec, pol_stride, 0, st));
            uint8_t *gout = dev_out + out_idx * gbytes;
            if (framed) {  // the output thread's headers, counters carried on the handle
                SDBE_CK(h, launch_vdif_headers(gout, kGroupPkts, gbytes / 2, h->secs, h->df, h->psn, h->ref_epoch,
                                               h->station, h->bdc, h->rx, st));
                h->launches += 1;
                const uint64_t dfs = static_cast<uint64_t>(h->df) + static_cast<uint64_t>(kGroupPkts);
                h->secs += static_cast<uint32_t>(dfs / 125000u);
                h->df = static_cast<uint32_t>(dfs % 125000u);
                h->psn += static_cast<uint64_t>(kGroupPkts);
            }
            PayloadTarget pt{gout, gbytes / 2, framed ? kOutPkt : kOutPktData, framed ? 32 : 0};
            int rc = h->cfg.precision != SDBE_PRECISION_FP32
                         ? tc_chain(h, spec, pol_stride, kGroupSnaps / kBatchSnaps, pt, st,
                                    [](int64_t, int64_t) { return SDBE_OK; })
                         : fft_chain(h, spec, pol_stride, kGroupSnaps / kBatchSnaps, pt, st,
                                     [](int64_t, int64_t) { return SDBE_OK; });
            if (rc) return rc;
            SDBE_CK(h, cudaMemsetAsync(bmp, 0, size_t(kGroupFrames) * 256, st));
            h->launches += 1;
            ++out_idx;
        }
    }
    return SDBE_OK;
}

int finish(sdbe_resampler *h, void *out, uint8_t *dev_out, int64_t n_ships, uint32_t flags, cudaStream_t st,
           int32_t *n_groups) {
    if ((flags & SDBE_OUT_HOST) && n_ships > 0)
        SDBE_CK(h, cudaMemcpyAsync(out, dev_out, n_ships * group_bytes(flags), cudaMemcpyDeviceToHost, st));
    SDBE_CK(h, cudaStreamSynchronize(st));
    h->last_stream = st;
    if (n_groups) *n_groups = static_cast<int32_t>(n_ships);
    return SDBE_OK;
}

uint8_t *out_target(sdbe_resampler *h, void *out, int64_t n_ships, uint32_t flags, int *rc) {
    *rc = SDBE_OK;
    if (!(flags & SDBE_OUT_HOST)) return static_cast<uint8_t *>(out);
    if (n_ships == 0) return nullptr;
    *rc = grow(h, &h->ing_out, &h->ing_out_bytes, n_ships * group_bytes(flags), "ingest output staging");
    return h->ing_out;
}

}  // namespace
}  // namespace sdbe

using namespace sdbe;

extern "C" {

int sdbe_ingest(sdbe_resampler *h, const void *packets, int64_t n_packets, void *out, int64_t out_groups,
                uint32_t flags, int32_t *n_groups) {
    if (!h) return fail(nullptr, SDBE_ERR_ARG, "null handle");
    if (n_packets < 0 || (n_packets > 0 && !packets) || out_groups < 0)
        return fail(h, SDBE_ERR_ARG, "bad argument");
    if (h->cfg.channel_map == SDBE_MAP_MAR2015) return fail(h, SDBE_ERR_STATE, "ingest does not support Mar-2015");
    const bool pac8 = (flags & SDBE_IN_8PAC) != 0, in_host = (flags & SDBE_IN_HOST) != 0;
    if (pac8 && !in_host && (reinterpret_cast<uintptr_t>(packets) & 7u))
        return fail(h, SDBE_ERR_ARG, "8pac input must be 8-byte aligned");
    if (!pac8 && !in_host && (reinterpret_cast<uintptr_t>(packets) & 15u))
        return fail(h, SDBE_ERR_ARG, "device packets must be 16-byte aligned");
    if (!(flags & SDBE_OUT_HOST) && out_groups > 0 && (reinterpret_cast<uintptr_t>(out) & 15u))
        return fail(h, SDBE_ERR_ARG, "device output must be 16-byte aligned");
    DeviceGuard g(h->cfg.device);
    if (!g.ok) return fail(h, SDBE_ERR_CUDA, "cudaSetDevice failed");
    cudaStream_t st = h->stream;
    const int64_t n_pk = pac8 ? 8 * n_packets : n_packets;
    const uint8_t *dev_pkts = nullptr;
    sdbe_reform_state reform = h->reform;
    int rc = SDBE_OK;
    uint32_t *hdr = nullptr;
    if (n_pk > 0) {
        // the policy reads the header words on the device: after the 8pac unpack
        // and header reform, or gathered from the packets
        rc = grow(h, &h->ing_hdr, &h->ing_hdr_bytes, n_pk * 12, "ingest header words");
        if (rc) return rc;
        hdr = reinterpret_cast<uint32_t *>(h->ing_hdr);
        if (pac8) {
            const void *src = packets;
            if (in_host) {
                rc = grow(h, &h->ing_raw, &h->ing_raw_bytes, n_packets * kPac8Bytes, "8pac staging");
                if (rc) return rc;
                SDBE_CK(h, cudaMemcpyAsync(h->ing_raw, packets, n_packets * kPac8Bytes, cudaMemcpyHostToDevice, st));
                src = h->ing_raw;
            }
            rc = grow(h, &h->ing_batch, &h->ing_batch_bytes, n_pk * kPktBytes, "ingest batch");
            if (rc) return rc;
            if (!h->reform_dev) SDBE_CK(h, cudaMalloc(&h->reform_dev, sizeof(sdbe_reform_state)));
            SDBE_CK(h, launch_unpack_8pac(src, n_packets, h->ing_batch, st));
            SDBE_CK(h, launch_beng_reform(h->ing_batch, n_pk, h->reform, h->reform_dev, hdr, st));
            SDBE_CK(h, cudaMemcpyAsync(&reform, h->reform_dev, sizeof(reform), cudaMemcpyDeviceToHost, st));
            h->launches += 2;
            dev_pkts = h->ing_batch;
        } else {
            if (in_host) {
                rc = grow(h, &h->ing_batch, &h->ing_batch_bytes, n_pk * kPktBytes, "ingest batch");
                if (rc) return rc;
                SDBE_CK(h, cudaMemcpyAsync(h->ing_batch, packets, n_pk * kPktBytes, cudaMemcpyHostToDevice, st));
                dev_pkts = h->ing_batch;
            } else {
                dev_pkts = static_cast<const uint8_t *>(packets);
            }
            SDBE_CK(h, launch_gather_headers(dev_pkts, n_pk, hdr, st));
            h->launches += 1;
        }
        rc = grow(h, &h->ing_accept, &h->ing_accept_bytes, n_pk, "ingest mask");
        if (rc) return rc;
    }
    PolOut res;
    rc = policy_device(h, hdr, n_pk, h->ing_accept, &res, st);  // waits for the stream
    if (rc) return rc;
    h->ing_last_n = n_pk;
    const int64_t n_ships = res.n_ships;
    if (n_ships > out_groups) {
        if (n_groups) *n_groups = static_cast<int32_t>(n_ships);
        return fail(h, SDBE_ERR_CAPACITY, "output has room for fewer groups than ship");
    }
    if (n_ships > 0 && !out) return fail(h, SDBE_ERR_ARG, "null output");
    rc = ensure_ring(h);
    if (rc) return rc;
    const Policy p = after_batch(h, res);
    const std::vector<int64_t> ships(res.ships, res.ships + n_ships), touched(res.touched, res.touched + res.n_touched);
    uint8_t *dev_out = out_target(h, out, n_ships, flags, &rc);
    if (rc) return rc;
    rc = run_device(h, p, dev_pkts, n_pk, h->ing_accept, ships, touched, dev_out, flags, st);
    if (rc) return rc;
    commit(h, p);
    if (pac8) h->reform = reform;
    return finish(h, out, dev_out, n_ships, flags, st, n_groups);
}

int sdbe_ingest_flush(sdbe_resampler *h, void *out, int64_t out_groups, uint32_t flags, int32_t *n_groups) {
    if (!h) return fail(nullptr, SDBE_ERR_ARG, "null handle");
    Policy p = snapshot(h);
    std::vector<int64_t> ships, touched;
    if (p.b_first >= 0) {
        int64_t last = -1;
        for (int64_t k = p.ref; k < p.ref + kRing; ++k)
            if (p.count[k % kRing] > 0) last = k;
        while (p.ref <= last) ship(p, ships);
    }
    const int64_t n_ships = static_cast<int64_t>(ships.size());
    if (n_ships > out_groups) {
        if (n_groups) *n_groups = static_cast<int32_t>(n_ships);
        return fail(h, SDBE_ERR_CAPACITY, "output has room for fewer groups than ship");
    }
    if (n_ships > 0 && !out) return fail(h, SDBE_ERR_ARG, "null output");
    DeviceGuard g(h->cfg.device);
    if (!g.ok) return fail(h, SDBE_ERR_CUDA, "cudaSetDevice failed");
    int rc = SDBE_OK;
    if (n_ships > 0) rc = ensure_ring(h);
    if (rc) return rc;
    uint8_t *dev_out = out_target(h, out, n_ships, flags, &rc);
    if (rc) return rc;
    rc = run_device(h, p, nullptr, 0, nullptr, ships, touched, dev_out, flags, h->stream);
    if (rc) return rc;
    commit(h, p);
    return finish(h, out, dev_out, n_ships, flags, h->stream, n_groups);
}

int sdbe_ingest_reform_state(const sdbe_resampler *h, sdbe_reform_state *st) {
    if (!h || !st) return SDBE_ERR_ARG;
    *st = h->reform;
    return SDBE_OK;
}

int sdbe_test_ingest_accept(const sdbe_resampler *h, uint8_t *mask, int64_t n) {
    if (!h || n < 0 || (n > 0 && !mask)) return SDBE_ERR_ARG;
    if (n != h->ing_last_n) return fail(const_cast<sdbe_resampler *>(h), SDBE_ERR_ARG, "n is not the last batch's size");
    if (n == 0) return SDBE_OK;
    DeviceGuard g(h->cfg.device);
    if (!g.ok) return SDBE_ERR_CUDA;
    if (cudaMemcpy(mask, h->ing_accept, static_cast<size_t>(n), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(const_cast<sdbe_resampler *>(h), SDBE_ERR_CUDA, "copy of the accept flags failed");
    return SDBE_OK;
}

int sdbe_ingest_get_stats(const sdbe_resampler *h, sdbe_ingest_stats *st) {
    if (!h || !st) return SDBE_ERR_ARG;
    *st = h->ing;
    st->b_first = h->b_first;
    return SDBE_OK;
}

}  // extern "C"
