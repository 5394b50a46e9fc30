// Unpack of 2-bit B-engine VDIF packets into spectra.
//
// Reference: vdif_to_beng, software/aphids/vdif_inout_gpu_thread.cu:404-507.
// Each 1056-B packet carries, for one B-frame b, channel group (c, f) and both
// phased sums, 8 channels x 128 snapshots of 2-bit (real, imag) samples: per
// snapshot two u32 words, bytes 0..3 of the first = channels 3,2,1,0 and of
// the second = channels 7,6,5,4; in each byte bits 0-1/2-3 are pol-1
// imag/real and bits 4-5/6-7 pol-0 imag/real (.cu:464-495).
#include "fft_core.cuh"
#include "launchers.cuh"
#include "sdbe_internal.cuh"

namespace sdbe {

struct PktHeader {
    int64_t frame;
    int group;
    uint32_t c, f;
    bool ok;
};

// B-engine header fields (.cu:353-369, vdif_in_databuf.c:66-74) and the slot
// the packet scatters to.  Packets flagged invalid, with f >= 8 or with b
// outside [b_zero, b_zero + n_frames) are not scattered.
__device__ __forceinline__ PktHeader decode_header(uint32_t w0, uint32_t w4, uint32_t w5, uint64_t b_zero,
                                                   int n_frames, int map) {
    PktHeader h;
    h.c = w5 & 0xFFu;
    h.f = (w5 >> 16) & 0xFFu;
    const uint64_t b = (static_cast<uint64_t>(w4) << 8) | (w5 >> 24);
    h.frame = static_cast<int64_t>(b - b_zero);
    h.ok = ((w0 >> 31) == 0u) && h.f < 8u && h.frame >= 0 && h.frame < n_frames;
    h.group = map == SDBE_MAP_APHIDS ? static_cast<int>((h.c >> 1) * 16u + (h.c & 1u) + 2u * h.f)
                                     : static_cast<int>(8u * h.c + h.f);
    return h;
}

// Two payload words of one snapshot -> packed nibble words for pol 0 and 1
// (nibble = real code << 2 | imag code, channel k of the group at bits 4k).
__device__ __forceinline__ void pack_snapshot(uint32_t wlo, uint32_t whi, uint32_t &p0, uint32_t &p1) {
    const uint32_t x = __byte_perm(wlo, 0u, 0x0123);  // byte k = channel k
    const uint32_t y = __byte_perm(whi, 0u, 0x0123);  // byte k = channel 4 + k
    uint32_t x1 = x & 0x0F0F0F0Fu, y1 = y & 0x0F0F0F0Fu;
    uint32_t x0 = (x >> 4) & 0x0F0F0F0Fu, y0 = (y >> 4) & 0x0F0F0F0Fu;
    x1 |= x1 >> 4;
    y1 |= y1 >> 4;
    x0 |= x0 >> 4;
    y0 |= y0 >> 4;
    p1 = __byte_perm(x1, y1, 0x6420);
    p0 = __byte_perm(x0, y0, 0x6420);
}

constexpr int kTilePkts = 32;

// 32 packets per CTA.  Phase 1: each warp issues the loads of all 4 of its
// packets first (headers broadcast, payloads as coalesced 16-B loads: lane l
// owns snapshots 4l..4l+3), then writes their packed words to a
// [pol][packet][snapshot-quad] tile swizzled by quad ^ packet.  Completion
// bits and per-frame counts are aggregated over the CTA's packets by warp 0
// (one atomic per distinct bitmap word / frame, not one per packet).
// Phase 2: lanes = packets, so each store instruction writes the 32 packets'
// channel groups of one snapshot row (128 contiguous bytes for in-order
// packets).
// Segment of a unpack launch that serves several calls (one per stream
// pair): its blocks start at block blk0 of the grid.
__device__ __forceinline__ const UnpackSeg &unpack_seg(const UnpackSegs &S, int64_t blk) {
    int j = 0;
    while (j + 1 < S.n && blk >= S.s[j + 1].blk0) ++j;
    return S.s[j];
}

__global__ void __launch_bounds__(256) k_unpack_packed(const __grid_constant__ UnpackSegs S) {
    const UnpackSeg &G = unpack_seg(S, blockIdx.x);
    const uint8_t *__restrict__ pkts = G.pkts;
    const int64_t n_pkts = G.n_pkts;
    const uint64_t b_zero = G.b_zero;
    const int n_frames = G.n_frames, map = G.map;
    uint32_t *__restrict__ spec = G.spec;
    const int64_t pol_stride = G.pol_stride, snap0 = G.snap0;
    uint32_t *__restrict__ bitmap = G.bitmap;
    int32_t *__restrict__ counts = G.counts;
    int32_t *__restrict__ rejected = G.rejected;
    const uint8_t *__restrict__ accept = G.accept;
    __shared__ uint4 tile[2][kTilePkts][32];
    __shared__ int64_t s_row[kTilePkts];
    __shared__ int s_group[kTilePkts];
    __shared__ int s_frame[kTilePkts];  // -1 not taken, -2 no packet
    __shared__ uint32_t s_cf[kTilePkts];  // c | f << 8
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t p_base = (static_cast<int64_t>(blockIdx.x) - G.blk0) * kTilePkts;

    uint32_t w0[4], w4[4], w5[4];
    uint4 a[4], b[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int64_t p = p_base + warp * 4 + q;
        if (p < n_pkts) {
            const uint4 *src = reinterpret_cast<const uint4 *>(pkts + p * kPktBytes);
            w0[q] = __ldg(reinterpret_cast<const uint32_t *>(src));
            const uint4 h1 = __ldg(src + 1);
            w4[q] = h1.x;
            w5[q] = h1.y;
            a[q] = __ldcs(src + 2 + 2 * lane);
            b[q] = __ldcs(src + 3 + 2 * lane);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int pl = warp * 4 + q;
        const int64_t p = p_base + pl;
        int64_t row = -1;
        int group = 0, frame = -2;
        uint32_t cf = 0;
        if (p < n_pkts) {
            const PktHeader h = decode_header(w0[q], w4[q], w5[q], b_zero, n_frames, map);
            const bool take = h.ok && (accept == nullptr || accept[p] != 0);
            frame = -1;
            if (take) {
                uint4 o0, o1;
                pack_snapshot(a[q].x, a[q].y, o0.x, o1.x);
                pack_snapshot(a[q].z, a[q].w, o0.y, o1.y);
                pack_snapshot(b[q].x, b[q].y, o0.z, o1.z);
                pack_snapshot(b[q].z, b[q].w, o0.w, o1.w);
                tile[0][pl][lane ^ pl] = o0;
                tile[1][pl][lane ^ pl] = o1;
                row = snap0 + h.frame * kSnapsPerFrame;
                group = h.group;
                frame = static_cast<int>(h.frame);
                cf = h.c | (h.f << 8);
            }
        }
        if (lane == 0) {
            s_row[pl] = row;
            s_group[pl] = group;
            s_frame[pl] = frame;
            s_cf[pl] = cf;
        }
    }
    __syncthreads();

    if (warp == 0) {  // lane = packet of the CTA
        const int frame = s_frame[lane];
        const uint32_t cf = s_cf[lane];
        const bool take = frame >= 0;
        // completion bits: lanes with the same bitmap word OR their bits, the lowest issues the atomic
        const int key = take ? frame * 64 + static_cast<int>((cf & 0xFFu) >> 2) : -1 - (frame == -2);
        const uint32_t bit = take ? 1u << (((cf & 0xFFu) & 3u) * 8u + (cf >> 8)) : 0u;
        const unsigned same = __match_any_sync(0xffffffffu, key);
        uint32_t bits = 0;
        for (int i = 0; i < 32; ++i) {
            const uint32_t bi = __shfl_sync(0xffffffffu, bit, i);
            if ((same >> i) & 1u) bits |= bi;
        }
        const bool leader = lane == __ffs(same) - 1;
        if (take && leader) atomicOr(bitmap + key, bits);
        if (counts != nullptr) {
            const unsigned same_f = __match_any_sync(0xffffffffu, take ? frame : -1);
            if (take && lane == __ffs(same_f) - 1) atomicAdd(counts + frame, __popc(same_f));
        }
        const unsigned rej = __ballot_sync(0xffffffffu, frame == -1);
        if (lane == 0 && rejected != nullptr && rej) atomicAdd(rejected, __popc(rej));
    }

    const int64_t row = s_row[lane];
    const int group = s_group[lane];
    if (row < 0) return;  // no further barriers below
    for (int t = warp; t < 2 * 32; t += 8) {
        const int pol = t >> 5, u = t & 31;
        const uint4 v = tile[pol][lane][u ^ lane];
        uint32_t *dst = spec + pol * pol_stride + (row + 4 * u) * kGroups + group;
        dst[0] = v.x;
        dst[kGroups] = v.y;
        dst[2 * kGroups] = v.z;
        dst[3 * kGroups] = v.w;
    }
}

// Missing packets read as zero (the reference pre-zeroes its buffers,
// .cu:897-898): every (frame, c, f) slot whose completion bit is unset gets
// code 2/2 in all 128 snapshots of both pols.
__global__ void k_fill_missing(const __grid_constant__ UnpackSegs S) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int j = 0;
    while (j + 1 < S.n && t >= S.s[j + 1].fill0) ++j;
    const UnpackSeg &G = S.s[j];
    const uint32_t *__restrict__ bitmap = G.bitmap;
    const int n_frames = G.n_frames, map = G.map;
    uint32_t *__restrict__ spec = G.spec;
    const int64_t pol_stride = G.pol_stride, snap0 = G.snap0;
    const int64_t idx = t - G.fill0;
    if (idx >= static_cast<int64_t>(n_frames) * kPktsPerFrame) return;
    const int64_t frame = idx / kPktsPerFrame;
    const uint32_t cf = static_cast<uint32_t>(idx % kPktsPerFrame);
    const uint32_t c = cf >> 3, f = cf & 7u;
    const uint32_t bit = (bitmap[frame * 64 + (c >> 2)] >> ((c & 3u) * 8u + f)) & 1u;
    if (bit) return;
    const int group = map == SDBE_MAP_APHIDS ? static_cast<int>((c >> 1) * 16u + (c & 1u) + 2u * f)
                                             : static_cast<int>(8u * c + f);
    for (int pol = 0; pol < 2; ++pol) {
        uint32_t *dst = spec + pol * pol_stride + (snap0 + frame * kSnapsPerFrame) * kGroups + group;
        for (int s = 0; s < kSnapsPerFrame; ++s) dst[static_cast<int64_t>(s) * kGroups] = kMissingWord;
    }
}

// Packed nibble word (8 channels) -> 16 int8 bytes (imag, real) per channel,
// value = code - 2 (read_2bit_sample, .cu:387-392).
__device__ __forceinline__ uint4 nibbles_to_int8(uint32_t p) {
    uint32_t o[4];
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        uint32_t acc = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = 2 * w + h;
            const uint32_t nib = (p >> (4 * k)) & 0xFu;
            const uint32_t im = static_cast<uint8_t>(static_cast<int8_t>(static_cast<int>(nib & 3u) - 2));
            const uint32_t re = static_cast<uint8_t>(static_cast<int8_t>(static_cast<int>(nib >> 2) - 2));
            acc |= (im | (re << 8)) << (16 * h);
        }
        o[w] = acc;
    }
    return make_uint4(o[0], o[1], o[2], o[3]);
}

// Reference-layout unpack: int8 [n_frames][128][16384][2] per pol.  One warp
// per packet, lane l owns snapshots 4l..4l+3; each (snapshot, pol) is one
// 16-B store of the packet's 8 channels.
__global__ void __launch_bounds__(256) k_vdif_to_beng_ref(const uint8_t *__restrict__ pkts, int64_t n_pkts,
                                                          uint64_t b_zero, int n_frames, int map,
                                                          int8_t *__restrict__ beng0, int8_t *__restrict__ beng1) {
    const int64_t p = static_cast<int64_t>(blockIdx.x) * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (p >= n_pkts) return;
    const uint4 *src = reinterpret_cast<const uint4 *>(pkts + p * kPktBytes);
    const uint32_t w0 = __ldg(reinterpret_cast<const uint32_t *>(src));
    const uint4 h1 = __ldg(src + 1);
    const PktHeader h = decode_header(w0, h1.x, h1.y, b_zero, n_frames, map);
    if (!h.ok) return;
    const uint4 a = __ldg(src + 2 + 2 * lane);
    const uint4 b = __ldg(src + 3 + 2 * lane);
    const uint32_t lo[4] = {a.x, a.z, b.x, b.z}, hi[4] = {a.y, a.w, b.y, b.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        uint32_t p0, p1;
        pack_snapshot(lo[q], hi[q], p0, p1);
        const int64_t off = ((h.frame * kSnapsPerFrame + 4 * lane + q) * kChannels + h.group * 8) * 2;
        *reinterpret_cast<uint4 *>(beng0 + off) = nibbles_to_int8(p0);
        *reinterpret_cast<uint4 *>(beng1 + off) = nibbles_to_int8(p1);
    }
}

// Mar-2015 SDBE fix (prototyping/cuda/reorder.py:13-43, numpy check :284-293):
// channels with (cid/4) even -- nibbles 0..3 of every group word -- come from
// snapshot (s+2) mod 128; output snapshots >= 69 come from the next B-frame.
__global__ void k_reorder_mar2015(const uint32_t *__restrict__ in, int n_frames, uint32_t *__restrict__ out) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = static_cast<int64_t>(n_frames - 1) * kSnapsPerFrame * kGroups;
    if (idx >= total) return;
    const int g = static_cast<int>(idx % kGroups);
    const int s = static_cast<int>((idx / kGroups) % kSnapsPerFrame);
    const int64_t f = idx / (static_cast<int64_t>(kGroups) * kSnapsPerFrame);
    const int64_t fs = f + (s >= 69 ? 1 : 0);
    const uint32_t shifted = __ldg(in + (fs * kSnapsPerFrame + ((s + 2) & 127)) * kGroups + g);
    const uint32_t plain = __ldg(in + (fs * kSnapsPerFrame + s) * kGroups + g);
    out[idx] = (shifted & 0x0000FFFFu) | (plain & 0xFFFF0000u);
}

// beng_int8_to_cufftComplex (.cu:532-556): (imag, real) int8 -> (real, imag)
// float, row stride 16385 with the Nyquist bin zeroed (.cu:925-926).
__global__ void k_beng_to_complex(const int8_t *__restrict__ beng, int64_t n_spectra, float2 *__restrict__ out) {
    const int64_t idx = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = n_spectra * (kChannels + 1);
    if (idx >= total) return;
    const int64_t sp = idx / (kChannels + 1);
    const int ch = static_cast<int>(idx % (kChannels + 1));
    float2 v = make_float2(0.f, 0.f);
    if (ch < kChannels) {
        const char2 iq = *reinterpret_cast<const char2 *>(beng + (sp * kChannels + ch) * 2);
        v = make_float2(static_cast<float>(iq.y), static_cast<float>(iq.x));
    }
    out[idx] = v;
}

// ---- launchers ---------------------------------------------------------------
void unpack_segs_add(UnpackSegs &S, const UnpackSeg &g) {
    UnpackSeg &d = S.s[S.n++];
    d = g;
    d.blk0 = S.blocks;
    d.fill0 = S.fill_threads;
    S.blocks += (g.n_pkts + kTilePkts - 1) / kTilePkts;
    S.fill_threads += static_cast<int64_t>(g.n_frames) * kPktsPerFrame;
}

cudaError_t launch_unpack_segs(const UnpackSegs &S, cudaStream_t st) {
    if (S.blocks <= 0) return cudaSuccess;
    k_unpack_packed<<<static_cast<unsigned>(S.blocks), 256, 0, st>>>(S);
    return cudaGetLastError();
}

cudaError_t launch_fill_missing_segs(const UnpackSegs &S, cudaStream_t st) {
    if (S.fill_threads <= 0) return cudaSuccess;
    k_fill_missing<<<static_cast<unsigned>((S.fill_threads + 255) / 256), 256, 0, st>>>(S);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const void *pkts, int64_t n_pkts, uint64_t b_zero, int n_frames, int map,
                          uint32_t *spec, int64_t pol_stride, int64_t snap0, uint32_t *bitmap,
                          int32_t *counts, int32_t *rejected, cudaStream_t st, const uint8_t *accept) {
    if (n_pkts <= 0) return cudaSuccess;
    UnpackSegs S{};
    unpack_segs_add(S, UnpackSeg{static_cast<const uint8_t *>(pkts), n_pkts, b_zero, n_frames, map, spec, pol_stride,
                                 snap0, bitmap, counts, rejected, accept, 0, 0});
    return launch_unpack_segs(S, st);
}

cudaError_t launch_fill_missing(const uint32_t *bitmap, int n_frames, int map, uint32_t *spec,
                                int64_t pol_stride, int64_t snap0, cudaStream_t st) {
    if (n_frames <= 0) return cudaSuccess;
    UnpackSegs S{};
    unpack_segs_add(S, UnpackSeg{nullptr, 0, 0, n_frames, map, spec, pol_stride, snap0,
                                 const_cast<uint32_t *>(bitmap), nullptr, nullptr, nullptr, 0, 0});
    return launch_fill_missing_segs(S, st);
}

cudaError_t launch_vdif_to_beng_ref(const void *pkts, int64_t n_pkts, uint64_t b_zero, int n_frames, int map,
                                    int8_t *beng0, int8_t *beng1, cudaStream_t st) {
    if (n_pkts <= 0) return cudaSuccess;
    k_vdif_to_beng_ref<<<static_cast<unsigned>((n_pkts + 7) / 8), 256, 0, st>>>(
        static_cast<const uint8_t *>(pkts), n_pkts, b_zero, n_frames, map, beng0, beng1);
    return cudaGetLastError();
}

cudaError_t launch_reorder_mar2015(const uint32_t *in, int n_frames, uint32_t *out, cudaStream_t st) {
    const int64_t total = static_cast<int64_t>(n_frames - 1) * kSnapsPerFrame * kGroups;
    if (total <= 0) return cudaSuccess;
    k_reorder_mar2015<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(in, n_frames, out);
    return cudaGetLastError();
}

cudaError_t launch_beng_to_complex(const int8_t *beng, int64_t n_spectra, void *out, cudaStream_t st) {
    const int64_t total = n_spectra * (kChannels + 1);
    if (total <= 0) return cudaSuccess;
    k_beng_to_complex<<<static_cast<unsigned>((total + 255) / 256), 256, 0, st>>>(beng, n_spectra,
                                                                                  static_cast<float2 *>(out));
    return cudaGetLastError();
}

}  // namespace sdbe
