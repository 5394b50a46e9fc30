// Ingest transforms on the device: 8pac unpack (software/aphids/vdif_8pac.c)
// and the B-engine header reform (software/aphids/beng_reform.c), the
// receive-side pre-pass of vdif_in_net_thread.c:291-298.
#include <cuda_runtime.h>

#include "handle.cuh"

namespace sdbe {

constexpr int kPktU64 = kPktBytes / 8;                        // 132
constexpr int32_t kClkPerSec = 286000000;                     // SWARM_CLK_PER_SEC
constexpr int32_t kBframeClk = 262144;                        // SWARM_BFRAME_CLK
constexpr int32_t kClkTol = 1024;                             // BFRAME_CLK_TOL
constexpr int64_t kMaxOffset = 1000;                          // MAX_COUNTABLE_BFRAME_OFFSET
constexpr int kReformThreads = 1024;

static_assert(sizeof(sdbe_reform_state) == 48, "reform state layout");

// ---------------------------------------------------------------------------
// 8pac unpack: one warp per output packet, 8-byte words (the packets inside a
// unit sit at 8-byte but not 16-byte offsets: 0, then 1064*k).  The header
// words the reference rewrites (vdif_8pac.c:5-41) are fixed in registers.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_unpack_8pac(const uint8_t *__restrict__ src, int64_t n_units,
                                                     uint8_t *__restrict__ dst) {
    const int64_t pkt = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (pkt >= n_units * 8) return;
    const int64_t unit = pkt >> 3;
    const int k = static_cast<int>(pkt & 7);
    const uint8_t *u = src + unit * kPac8Bytes;
    const uint64_t *s = reinterpret_cast<const uint64_t *>(u + 1064 * k);
    uint64_t *d = reinterpret_cast<uint64_t *>(dst + pkt * kPktBytes);
    for (int i = lane; i < kPktU64; i += 32) {
        uint64_t v = __ldcs(s + i);
        if (i < 4) {
            const uint32_t *h1 = reinterpret_cast<const uint32_t *>(u);
            uint32_t lo = static_cast<uint32_t>(v), hi = static_cast<uint32_t>(v >> 32);
            if (i == 0) {
                if (k) lo = (lo & 0x7FFFFFFFu) | (__ldg(h1) & 0x80000000u);                  // fix_8pac_flags
                hi = (hi & 0xFF000000u) | ((8u * (__ldg(h1 + 1) & 0xFFFFFFu) + k) & 0xFFFFFFu);  // data frame
            } else if (i == 1) {
                const int len = static_cast<int>(__ldg(h1 + 2) & 0xFFFFFFu) - 7;               // reset_8pac_size
                lo = (lo & 0xFF000000u) | (static_cast<uint32_t>(len / 8) & 0xFFFFFFu);
            } else if (i == 3) {
                const uint64_t psn = (static_cast<uint64_t>(__ldg(h1 + 7)) << 32) | __ldg(h1 + 6);
                const uint64_t p = 8ull * psn + static_cast<uint64_t>(k);                     // fix_8pac_psn
                lo = static_cast<uint32_t>(p);
                hi = static_cast<uint32_t>(p >> 32);
            }
            v = (static_cast<uint64_t>(hi) << 32) | lo;
        }
        __stcs(d + i, v);
    }
}

// ---------------------------------------------------------------------------
// Header reform.  The reference walks the packets in order with a state of
// T0, TPREV and BPREV; each valid packet's count is BPREV plus the B-frames
// from TPREV to its timestamp, found by stepping one frame at a time with a
// 1024-clock tolerance (beng_reform.c:34-104, 137-186).
//
// One CTA walks tiles of 1024 packets.  When every valid packet of a tile and
// its predecessor have clk < 286e6 and lie a whole number k of frames apart
// with |k| <= 1000, stepping returns exactly k (each step adds 262144 clocks
// to the absolute time and lands on the other timestamp), so the counts are
// BPREV plus a prefix sum: computed with block scans.  Any other tile (jitter,
// corrupt clocks, jumps beyond the cap) is walked by one thread with the
// stepping itself, bounded by the cap, so results match the reference in all
// cases.
// ---------------------------------------------------------------------------
struct Ts {
    int32_t sec, clk;
};

__device__ __forceinline__ Ts read_ts(uint32_t w4, uint32_t w5) {
    const int64_t b = (static_cast<int64_t>(w4) << 21) | static_cast<int64_t>((w5 >> 11) & 0x1FFFFFu);
    return Ts{static_cast<int32_t>((b & 0x001FFFFFE0000000ll) >> 29), static_cast<int32_t>(b & 0x1FFFFFFFll)};
}

__device__ int ts_compare(Ts then, Ts now) {  // _beng_timestamp_compare_then_now, as written
    if (then.sec < now.sec) {
        if (then.sec == now.sec - 1 && then.clk + kClkTol > kClkPerSec && (then.clk + kClkTol) % kClkPerSec >= now.clk)
            return 0;
        return -1;
    }
    if (then.sec > now.sec) {
        if (now.clk + kClkTol > kClkPerSec && (now.clk + kClkTol) % kClkPerSec >= then.clk) return 0;
        return 1;
    }
    if (then.clk + kClkTol < now.clk) return -1;
    if (now.clk + kClkTol < then.clk) return 1;
    return 0;
}

__device__ Ts ts_increment(Ts t) {
    t.clk += kBframeClk;
    if (t.clk > kClkPerSec) {
        t.sec += 1;
        t.clk %= kClkPerSec;
    }
    return t;
}

__device__ int64_t ts_offset(Ts then, Ts now) {  // at most kMaxOffset + 1 steps
    const int cmp = ts_compare(then, now);
    if (cmp == 0) return 0;
    Ts start = cmp < 0 ? then : now;
    const Ts end = cmp < 0 ? now : then;
    const int64_t step = cmp < 0 ? 1 : -1;
    int64_t off = 0;
    while (ts_compare(start, end) < 0) {
        start = ts_increment(start);
        off += step;
        if (off > kMaxOffset || -off > kMaxOffset) break;
    }
    return off;
}

__device__ __forceinline__ void write_old_header(uint32_t *w, uint32_t w5, int32_t off) {
    const uint32_t c = w5 & 0xFFu, f = (w5 >> 8) & 7u, o = static_cast<uint32_t>(off);
    w[5] = (w5 & 0x0000FF00u) | c | (f << 16) | ((o & 0xFFu) << 24);
    w[4] = (o & 0x7FFFFF00u) >> 8;
}

template <class T, class Op>
__device__ T block_scan_inclusive(T v, T *warp_tot, Op op, T identity) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= o) v = op(u, v);
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
        T t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T u = __shfl_up_sync(0xFFFFFFFFu, t, o);
            if (lane >= o) t = op(u, t);
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const T before = warp ? warp_tot[warp - 1] : identity;
    const T r = op(before, v);
    __syncthreads();  // warp_tot reusable
    return r;
}

struct MaxOp {
    __device__ int operator()(int a, int b) const { return a > b ? a : b; }
};
struct SumOp {
    __device__ long long operator()(long long a, long long b) const { return a + b; }
};

__global__ void __launch_bounds__(kReformThreads) k_beng_reform(uint8_t *__restrict__ pkts, int64_t n,
                                                                sdbe_reform_state in, sdbe_reform_state *out,
                                                                uint32_t *__restrict__ hdr) {
    __shared__ sdbe_reform_state s;
    __shared__ Ts s_ts[kReformThreads];
    __shared__ int s_pv[kReformThreads];
    __shared__ int s_first;
    __shared__ int s_scan_i[32];
    __shared__ long long s_scan_l[32];
    const int tid = threadIdx.x;
    if (tid == 0) s = in;
    for (int64_t base = 0; base < n; base += kReformThreads) {
        if (tid == 0) s_first = kReformThreads;
        __syncthreads();
        const int64_t i = base + tid;
        uint32_t *w = reinterpret_cast<uint32_t *>(pkts + i * kPktBytes);
        bool valid = false;
        uint32_t w5 = 0;
        Ts ts{0, 0};
        if (i < n) {
            valid = (w[0] >> 31) == 0u;
            w5 = w[5];
            ts = read_ts(w[4], w5);
        }
        s_ts[tid] = ts;
        if (valid) atomicMin(&s_first, tid);
        __syncthreads();
        if (tid == s_first && s.t0_sec == -1 && s.t0_clk == -1) {  // first valid packet of the stream
            s.t0_sec = s.tprev_sec = ts.sec;
            s.t0_clk = s.tprev_clk = ts.clk;
            s.bprev = 0;
        }
        // index of the previous valid packet in the tile (exclusive max scan)
        s_pv[tid] = block_scan_inclusive<int>(valid ? tid : -1, s_scan_i, MaxOp(), -1);
        __syncthreads();
        const int before = tid ? s_pv[tid - 1] : -1;
        const int last = s_pv[kReformThreads - 1];
        const Ts p = before >= 0 ? s_ts[before] : Ts{s.tprev_sec, s.tprev_clk};
        bool ok = true;
        long long d = 0;
        if (valid) {
            const long long delta = static_cast<long long>(ts.sec - p.sec) * kClkPerSec + (ts.clk - p.clk);
            ok = ts.clk < kClkPerSec && p.clk < kClkPerSec && ts.clk >= 0 && p.clk >= 0 &&
                 delta % kBframeClk == 0 && delta <= kMaxOffset * kBframeClk && -delta <= kMaxOffset * kBframeClk;
            d = delta / kBframeClk;
        }
        const bool slow = __syncthreads_or(valid && !ok) != 0;
        if (!slow) {
            const long long sum = block_scan_inclusive<long long>(valid ? d : 0, s_scan_l, SumOp(), 0);
            const int32_t off = static_cast<int32_t>(static_cast<uint32_t>(static_cast<unsigned long long>(s.bprev + sum)));
            if (valid) write_old_header(w, w5, off);
            __syncthreads();  // everyone has read s.bprev
            if (tid == last) {
                s.tprev_sec = ts.sec;
                s.tprev_clk = ts.clk;
                s.bprev = off;
            }
        } else if (tid == 0) {
            const int64_t end = n - base < kReformThreads ? n - base : kReformThreads;
            for (int64_t j = 0; j < end; ++j) {
                uint32_t *wj = reinterpret_cast<uint32_t *>(pkts + (base + j) * kPktBytes);
                if (wj[0] >> 31) continue;
                const uint32_t w5j = wj[5];
                const Ts now = read_ts(wj[4], w5j);
                int32_t off = static_cast<int32_t>(ts_offset(Ts{s.tprev_sec, s.tprev_clk}, now));
                if (off > kMaxOffset || off < -kMaxOffset) {
                    wj[0] |= 0x80000000u;
                    off = -1;
                    s.marked_invalid += 1;
                } else {
                    off = static_cast<int32_t>(static_cast<uint32_t>(static_cast<unsigned long long>(off + s.bprev)));
                    s.tprev_sec = now.sec;
                    s.tprev_clk = now.clk;
                    s.bprev = off;
                }
                write_old_header(wj, w5j, off);
            }
            s.slow_tiles += 1;
        }
        __syncthreads();
        if (hdr != nullptr && i < n) {
            hdr[3 * i] = w[0];
            hdr[3 * i + 1] = w[4];
            hdr[3 * i + 2] = w[5];
        }
    }
    __syncthreads();
    if (tid == 0) *out = s;
}

// Header words (w0, w4, w5) of plain packets, for the host-side ingest policy.
__global__ void k_gather_headers(const uint8_t *__restrict__ pkts, int64_t n, uint32_t *__restrict__ hdr) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(pkts + i * kPktBytes);
    hdr[3 * i] = __ldg(w);
    hdr[3 * i + 1] = __ldg(w + 4);
    hdr[3 * i + 2] = __ldg(w + 5);
}

cudaError_t launch_unpack_8pac(const void *src, int64_t n_units, void *dst, cudaStream_t st) {
    if (n_units <= 0) return cudaSuccess;
    const int64_t threads = n_units * 8 * 32;
    k_unpack_8pac<<<static_cast<unsigned>((threads + 255) / 256), 256, 0, st>>>(static_cast<const uint8_t *>(src),
                                                                               n_units, static_cast<uint8_t *>(dst));
    return cudaGetLastError();
}

cudaError_t launch_beng_reform(void *pkts, int64_t n, const sdbe_reform_state &in, sdbe_reform_state *out_dev,
                               uint32_t *hdr, cudaStream_t st) {
    k_beng_reform<<<1, kReformThreads, 0, st>>>(static_cast<uint8_t *>(pkts), n, in, out_dev, hdr);
    return cudaGetLastError();
}

cudaError_t launch_gather_headers(const void *pkts, int64_t n, uint32_t *hdr, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_gather_headers<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(static_cast<const uint8_t *>(pkts), n,
                                                                            hdr);
    return cudaGetLastError();
}

}  // namespace sdbe

using namespace sdbe;

extern "C" {

int sdbe_reform_init(sdbe_reform_state *st) {
    if (!st) return SDBE_ERR_ARG;
    *st = sdbe_reform_state{};
    st->t0_sec = st->t0_clk = st->tprev_sec = st->tprev_clk = -1;
    st->bprev = -1;
    return SDBE_OK;
}

int sdbe_unpack_8pac(const void *src, int64_t n_units, void *dst, void *stream) {
    if (n_units < 0 || (n_units > 0 && (!src || !dst))) return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    if ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 7u)
        return fail(nullptr, SDBE_ERR_ARG, "8pac buffers must be 8-byte aligned");
    SDBE_CK(nullptr, launch_unpack_8pac(src, n_units, dst, static_cast<cudaStream_t>(stream)));
    return SDBE_OK;
}

int sdbe_beng_reform(sdbe_reform_state *st, void *pkts, int64_t n_pkts, void *stream) {
    if (!st || n_pkts < 0 || (n_pkts > 0 && !pkts)) return fail(nullptr, SDBE_ERR_ARG, "bad argument");
    if (reinterpret_cast<uintptr_t>(pkts) & 3u) return fail(nullptr, SDBE_ERR_ARG, "packets must be 4-byte aligned");
    if (n_pkts == 0) return SDBE_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void *scr = nullptr;  // this thread's reusable scratch: the call waits for its stream below
    SDBE_CK(nullptr, thread_scratch(sizeof(sdbe_reform_state), &scr));
    sdbe_reform_state *dev = static_cast<sdbe_reform_state *>(scr);
    cudaError_t e = launch_beng_reform(pkts, n_pkts, *st, dev, nullptr, s);
    sdbe_reform_state out{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&out, dev, sizeof(out), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(nullptr, SDBE_ERR_CUDA, std::string("beng_reform: ") + cudaGetErrorString(e));
    *st = out;
    return SDBE_OK;
}

}  // extern "C"
