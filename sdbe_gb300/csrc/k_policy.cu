// Group assembly decisions on the device: the ingest thread's b-count
// windowing, look-ahead flush, frame and group limits and completion shipping
// (get_beng_group_index_offset, insert_vdif_in_beng_group_buffer and
// check_beng_group_complete, software/aphids/vdif_in_databuf.c:96-167, run by
// the ingest loop of vdif_in_net_thread.c:333-490) for one received batch,
// from its packets' header words.
//
// The reference takes a batch's packets in compar_beng order (invalid first,
// then by b-count, stable) one at a time.  The packets of one B-frame (one b)
// are contiguous in that order, and every decision about them depends on the
// policy state and their number only, except which of them a frame that hits
// its 2048-packet limit keeps: the first ones in arrival order.  So:
//   k_pol_scan    the smallest and largest valid b, the invalid packets;
//   k_pol_bin     each packet's frame bin in a window of kPolWindow B-frames
//                 from the oldest open group, and the packets per bin;
//   k_pol_walk    one thread applies the policy per frame in b order: the
//                 packets accepted per frame, the groups shipped and touched,
//                 the statistics and the state after the batch;
//   k_pol_accept  each packet's accept flag where a frame is taken whole;
//   k_pol_rank    the first k packets in arrival order of a frame the limit
//                 cut (one CTA per such frame).
#include <cuda_runtime.h>

#include <cstring>

#include "handle.cuh"

namespace sdbe {
namespace {

constexpr long long kGF = 143;                     // BENG_FRAMES_PER_GROUP
constexpr long long kGP = kGF * kPktsPerFrame;     // packets per complete group
constexpr int kRingSlots = 4;                      // BENG_GROUPS_IN_BUFFER
constexpr int kAhead = 2;                          // MAX_INDEX_LOOK_AHEAD

// scan words: [0] smallest valid b, [1] largest valid b, [2] invalid,
// [3] before the window, [4] beyond the window
constexpr int kScanWords = 5;

__device__ __forceinline__ bool hdr_b(const uint32_t *hdr, int64_t i, unsigned long long *b) {
    const uint32_t w0 = hdr[3 * i], w4 = hdr[3 * i + 1], w5 = hdr[3 * i + 2];
    *b = (static_cast<unsigned long long>(w4) << 8) | (w5 >> 24);
    return (w0 >> 31) == 0;
}

__global__ void k_pol_scan(const uint32_t *__restrict__ hdr, int64_t n, unsigned long long *scan) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    unsigned long long b = 0;
    const bool ok = i < n && hdr_b(hdr, i, &b);
    unsigned long long lo = ok ? b : ~0ull, hi = ok ? b : 0ull;
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long l2 = __shfl_xor_sync(0xffffffffu, lo, o), h2 = __shfl_xor_sync(0xffffffffu, hi, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    const unsigned inval = __popc(__ballot_sync(0xffffffffu, i < n && !ok));
    if ((threadIdx.x & 31) == 0) {
        if (lo != ~0ull) atomicMin(scan, lo);
        if (hi != 0ull) atomicMax(scan + 1, hi);
        if (inval) atomicAdd(scan + 2, static_cast<unsigned long long>(inval));
    }
}

// b of bin 0: the first frame of the oldest open group (the first valid b + 1
// on the stream's first batch); -1 while the stream has no valid packet.
__device__ __forceinline__ long long pol_base(const PolState &s, const unsigned long long *scan) {
    if (s.b_first >= 0) return s.b_first + 1 + kGF * s.ref;
    if (scan[0] == ~0ull) return -1;
    return static_cast<long long>(scan[0]) + 1;
}

// code: bin >= 0, -1 invalid, -2 before the window (before the oldest open
// group), -3 beyond the window
__global__ void k_pol_bin(const uint32_t *__restrict__ hdr, int64_t n, const PolState *__restrict__ st,
                          unsigned long long *scan, int32_t *__restrict__ code, int32_t *__restrict__ nb) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const long long base = pol_base(*st, scan);
    int c = -1;
    unsigned long long b = 0;
    if (i < n && hdr_b(hdr, i, &b) && base >= 0) {
        const long long d = static_cast<long long>(b) - base;
        if (d < 0)
            c = -2;
        else if (d >= kPolWindow)
            c = -3;
        else
            c = static_cast<int>(d);
    }
    if (i < n) {
        code[i] = c;
        if (c >= 0) atomicAdd(nb + c, 1);
    }
    const unsigned before = __popc(__ballot_sync(0xffffffffu, i < n && c == -2));
    const unsigned beyond = __popc(__ballot_sync(0xffffffffu, i < n && c == -3));
    if ((threadIdx.x & 31) == 0) {
        if (before) atomicAdd(scan + 3, static_cast<unsigned long long>(before));
        if (beyond) atomicAdd(scan + 4, static_cast<unsigned long long>(beyond));
    }
}

// The policy, one frame at a time in b order (one warp: the lanes find the
// next non-empty bins, lane 0 decides).  Statistics st[]: packets, invalid,
// before_start, too_far_ahead, used, overflow, groups_shipped,
// groups_incomplete.
__global__ void k_pol_walk(const PolState *__restrict__ in, int64_t n, const unsigned long long *__restrict__ scan,
                           const int32_t *__restrict__ nb, int32_t *__restrict__ acc, int32_t *__restrict__ capped,
                           PolOut *__restrict__ out) {
    const int lane = threadIdx.x;
    __shared__ PolState s;
    __shared__ int n_ships, n_touched, n_capped, bad;
    if (lane == 0) {
        std::memcpy(&s, in, sizeof(PolState));
        n_ships = n_touched = n_capped = bad = 0;
        s.st[0] += n;
        s.st[1] += static_cast<long long>(scan[2]);
        if (s.b_first < 0 && scan[0] != ~0ull) {  // the stream's first valid packet
            s.b_first = static_cast<long long>(scan[0]);
            s.ref = 0;
        }
    }
    __syncwarp();
    const long long base = s.b_first >= 0 ? s.b_first + 1 + kGF * s.ref : -1;
    if (base >= 0) {
        auto ship = [&]() {
            const int sl = static_cast<int>(s.ref % kRingSlots);
            if (n_ships < kPolMaxGroups) out->ships[n_ships] = s.ref;
            else bad = 1;
            ++n_ships;
            s.st[6] += 1;
            if (s.count[sl] < kGP) s.st[7] += 1;
            s.count[sl] = 0;
            for (int f = 0; f < kGF; ++f) s.fcount[sl * kGF + f] = 0;
            s.ref += 1;
        };
        if (lane == 0) s.st[2] += static_cast<long long>(scan[3]);
        const long long span = static_cast<long long>(scan[1]) - base + 1;
        const int nbins = span <= 0 ? 0 : (span < kPolWindow ? static_cast<int>(span) : kPolWindow);
        for (int b0 = 0; b0 < nbins; b0 += 32) {
            const int mine = b0 + lane < nbins ? nb[b0 + lane] : 0;
            unsigned live = __ballot_sync(0xffffffffu, mine > 0);
            if (lane == 0) {
                while (live) {
                    const int k = __ffs(live) - 1;
                    live &= live - 1;
                    const int bin = b0 + k;
                    const long long b = base + bin;
                    const int total = nb[bin];
                    int rem = total, taken = 0;
                    while (rem > 0) {
                        const long long lo = s.b_first + 1 + kGF * s.ref;
                        if (b < lo) {
                            s.st[2] += rem;
                            break;
                        }
                        long long off = (b - lo) / kGF;
                        if (off >= kRingSlots) {
                            // the search ends with its upper bound at the last frame of the
                            // group after the four it checked (vdif_in_databuf.c:107-120)
                            if (b > lo + (kRingSlots + 1) * kGF - 1 + kRingSlots * kGF) {
                                s.st[3] += rem;
                                break;
                            }
                            off = kRingSlots;
                        }
                        if (off > kAhead) {  // force the oldest group out, look again
                            ship();
                            continue;
                        }
                        const long long g = s.ref + off;
                        const int sl = static_cast<int>(g % kRingSlots);
                        const int frame = static_cast<int>(b - (s.b_first + 1 + kGF * g));
                        int room = kPktsPerFrame - s.fcount[sl * kGF + frame];
                        if (kGP - s.count[sl] < room) room = static_cast<int>(kGP - s.count[sl]);
                        if (room > 0) {
                            const int c = rem < room ? rem : room;
                            s.fcount[sl * kGF + frame] += c;
                            s.count[sl] += c;
                            s.st[4] += c;
                            taken += c;
                            rem -= c;
                            if (n_touched == 0 || out->touched[n_touched - 1] != g) {
                                if (n_touched < kPolMaxGroups) out->touched[n_touched] = g;
                                else bad = 1;
                                ++n_touched;
                            }
                        } else {  // offered, over the frame or group limit
                            s.st[4] += 1;
                            s.st[5] += 1;
                            rem -= 1;
                        }
                        if (s.count[s.ref % kRingSlots] == kGP) ship();
                    }
                    acc[bin] = taken;
                    if (taken > 0 && taken < total) capped[n_capped++] = bin;
                }
            }
            __syncwarp();
        }
        if (lane == 0 && scan[4] > 0) {
            // packets beyond the window lie beyond the too-far limit of every
            // state the walk passed through, unless the window's end came
            // within that limit of the last state
            if (s.b_first + 1 + kGF * s.ref + (2 * kRingSlots + 1) * kGF - 1 < base + kPolWindow)
                s.st[3] += static_cast<long long>(scan[4]);
            else
                bad = 1;
        }
    }
    __syncwarp();
    if (lane == 0) {
        std::memcpy(&out->s, &s, sizeof(PolState));
        out->base = base;
        out->n_ships = n_ships;
        out->n_touched = n_touched;
        out->n_capped = n_capped;
        out->window_exceeded = bad;
    }
}

__global__ void k_pol_accept(const int32_t *__restrict__ code, int64_t n, const int32_t *__restrict__ nb,
                             const int32_t *__restrict__ acc, uint8_t *__restrict__ accept) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const int c = code[i];
    accept[i] = (c >= 0 && acc[c] > 0 && acc[c] == nb[c]) ? 1 : 0;
}

// One CTA per frame the limit cut: its first acc[bin] packets in arrival
// order are accepted (a block-wide running count over the batch in order).
__global__ void __launch_bounds__(1024) k_pol_rank(const int32_t *__restrict__ code, int64_t n,
                                                   const int32_t *__restrict__ acc, const int32_t *__restrict__ capped,
                                                   uint8_t *__restrict__ accept) {
    __shared__ int warp_cnt[32];
    __shared__ int run;
    const int bin = capped[blockIdx.x];
    const int k = acc[bin];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) run = 0;
    __syncthreads();
    for (int64_t i0 = 0; i0 < n; i0 += blockDim.x) {
        const int64_t i = i0 + threadIdx.x;
        const bool mine = i < n && code[i] == bin;
        const unsigned m = __ballot_sync(0xffffffffu, mine);
        if (lane == 0) warp_cnt[w] = __popc(m);
        __syncthreads();
        int before = run;
        for (int j = 0; j < w; ++j) before += warp_cnt[j];
        before += __popc(m & ((1u << lane) - 1u));
        if (mine && before < k) accept[i] = 1;
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int j = 0; j < static_cast<int>(blockDim.x >> 5); ++j) t += warp_cnt[j];
            run += t;
        }
        __syncthreads();
        if (run >= k) break;
    }
}

}  // namespace

// The policy on the device for a batch of n packets whose header words (w0,
// w4, w5) are at hdr: the accept flags (accept[n]) and the result (state
// after the batch, ships, touched groups) in host memory.  The handle's state
// is read, not changed.
int policy_device(sdbe_resampler *h, const uint32_t *hdr, int64_t n, uint8_t *accept, PolOut *res, cudaStream_t st) {
    const int64_t need = static_cast<int64_t>(sizeof(PolState) + sizeof(PolOut)) + kScanWords * 8 +
                         3 * static_cast<int64_t>(kPolWindow) * 4 + 4 * (n > 0 ? n : 1);
    if (int rc = grow(h, &h->pol_scr, &h->pol_scr_bytes, need, "the group assembly scratch")) return rc;
    uint8_t *p = h->pol_scr;
    PolState *d_in = reinterpret_cast<PolState *>(p);
    p += sizeof(PolState);
    PolOut *d_out = reinterpret_cast<PolOut *>(p);
    p += sizeof(PolOut);
    unsigned long long *scan = reinterpret_cast<unsigned long long *>(p);
    p += kScanWords * 8;
    int32_t *nb = reinterpret_cast<int32_t *>(p), *acc = nb + kPolWindow, *capped = acc + kPolWindow;
    int32_t *code = capped + kPolWindow;

    PolState s{};
    s.b_first = h->b_first;
    s.ref = h->ing_ref;
    for (int i = 0; i < 4; ++i) s.count[i] = h->g_count[i];
    for (int i = 0; i < 4 * 143; ++i) s.fcount[i] = h->g_fcount[static_cast<size_t>(i)];
    const sdbe_ingest_stats &g = h->ing;
    const int64_t sv[8] = {g.packets, g.invalid, g.before_start, g.too_far_ahead, g.used, g.overflow,
                           g.groups_shipped, g.groups_incomplete};
    for (int i = 0; i < 8; ++i) s.st[i] = sv[i];
    SDBE_CK(h, cudaMemcpyAsync(d_in, &s, sizeof(s), cudaMemcpyHostToDevice, st));
    SDBE_CK(h, cudaMemsetAsync(scan, 0, kScanWords * 8, st));
    SDBE_CK(h, cudaMemsetAsync(scan, 0xFF, 8, st));  // smallest valid b: none yet
    SDBE_CK(h, cudaMemsetAsync(nb, 0, static_cast<size_t>(kPolWindow) * 4, st));
    const unsigned grid = static_cast<unsigned>((n + 255) / 256 > 0 ? (n + 255) / 256 : 1);
    if (n > 0) {
        k_pol_scan<<<grid, 256, 0, st>>>(hdr, n, scan);
        SDBE_CK(h, cudaGetLastError());
        k_pol_bin<<<grid, 256, 0, st>>>(hdr, n, d_in, scan, code, nb);
        SDBE_CK(h, cudaGetLastError());
    }
    k_pol_walk<<<1, 32, 0, st>>>(d_in, n, scan, nb, acc, capped, d_out);
    SDBE_CK(h, cudaGetLastError());
    if (n > 0) {
        k_pol_accept<<<grid, 256, 0, st>>>(code, n, nb, acc, accept);
        SDBE_CK(h, cudaGetLastError());
    }
    h->launches += n > 0 ? 4 : 1;
    SDBE_CK(h, cudaMemcpyAsync(res, d_out, sizeof(PolOut), cudaMemcpyDeviceToHost, st));
    SDBE_CK(h, cudaStreamSynchronize(st));
    if (res->window_exceeded)
        return fail(h, SDBE_ERR_CAPACITY, "the batch spans more B-frames than the group assembly window (16384)");
    if (res->n_capped > 0 && n > 0) {
        k_pol_rank<<<static_cast<unsigned>(res->n_capped), 1024, 0, st>>>(code, n, acc, capped, accept);
        SDBE_CK(h, cudaGetLastError());
        h->launches += 1;
    }
    return SDBE_OK;
}

}  // namespace sdbe
