// Output VDIF framing (R2DBE format, 8224-B frames).
//
// Header layout: vdif_out_header_t (software/aphids/vdif_out_databuf.h:19-52).
// Constant fields from init_vdif_out (vdif_out_databuf.c:35-64): df_len =
// 8224/8, one channel, version 0, real data, edv5 = 2.  Per-packet fields from
// the output thread (vdif_out_net_thread.c:295-317): secs and data-frame number
// advance per packet with df wrapping at 125000 frames/s, thread 0,
// bps = bit_depth - 1, pol, BDC/receiver sidebands, psn + 1 per packet.
#include "sdbe_internal.cuh"

namespace sdbe {

constexpr uint32_t kFramesPerSecond = 125000;  // VDIF_OUT_FRAMES_PER_SECOND

__global__ void k_vdif_headers(uint8_t *__restrict__ frames, int64_t n_pkts, int64_t pol_stride, uint32_t secs0,
                               uint32_t df0, uint64_t psn0, uint32_t ref_epoch, uint32_t station, uint32_t bdc,
                               uint32_t rx) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_pkts) return;
    const uint32_t pol = blockIdx.y;
    const uint64_t dfs = static_cast<uint64_t>(df0) + static_cast<uint64_t>(i);
    const uint32_t secs = secs0 + static_cast<uint32_t>(dfs / kFramesPerSecond);
    const uint32_t df = static_cast<uint32_t>(dfs % kFramesPerSecond);
    const uint64_t psn = psn0 + static_cast<uint64_t>(i);
    uint4 a, b;
    a.x = secs & 0x3FFFFFFFu;                                    // w0: secs, legacy 0, valid
    a.y = (df & 0xFFFFFFu) | ((ref_epoch & 0x3Fu) << 24);        // w1: df, ref_epoch, UA 0
    a.z = static_cast<uint32_t>(kOutPkt / 8);                    // w2: df_len, 1 channel, ver 0
    a.w = (station & 0xFFFFu) | (1u << 26);                      // w3: station, thread 0, bps 2-1, real
    b.x = (pol & 1u) | ((bdc & 1u) << 1) | ((rx & 1u) << 2) | (2u << 24);  // w4: pol, sidebands, edv5 2
    b.y = 0u;                                                    // w5: PIC status
    b.z = static_cast<uint32_t>(psn & 0xFFFFFFFFull);            // w6-7: psn
    b.w = static_cast<uint32_t>(psn >> 32);
    uint4 *dst = reinterpret_cast<uint4 *>(frames + pol * pol_stride + i * kOutPkt);
    dst[0] = a;
    dst[1] = b;
}

// Time-aligned payloads: output word o of pol p is word o + skip of the
// stream [left (n_left words) | pay]; 4 words per thread, one 16-B store.
// grid (ceil(n_pkts*512/256), 2).
__global__ void k_align_frames(const uint32_t *__restrict__ pay, int64_t pay_pol_stride, const uint32_t *__restrict__ left,
                               int64_t left_pol_stride, int64_t n_left, int64_t skip, int64_t n_pkts,
                               uint8_t *__restrict__ frames, int64_t frame_pol_stride) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n_pkts * (kOutWords / 4)) return;
    const int pol = blockIdx.y;
    const int64_t o = 4 * t;
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int64_t s = o + i + skip;
        w[i] = s < n_left ? left[pol * left_pol_stride + s] : __ldg(pay + pol * pay_pol_stride + (s - n_left));
    }
    const int64_t pkt = o / kOutWords, word = o % kOutWords;
    uint4 *dst = reinterpret_cast<uint4 *>(frames + pol * frame_pol_stride + pkt * kOutPkt + 32 + 4 * word);
    *dst = make_uint4(w[0], w[1], w[2], w[3]);
}

// Words [from, from + count) of the same stream -> the next leftover buffer.
__global__ void k_save_leftover(const uint32_t *__restrict__ pay, int64_t pay_pol_stride,
                                const uint32_t *__restrict__ left, int64_t left_pol_stride, int64_t n_left, int64_t skip,
                                int64_t from, int64_t count, uint32_t *__restrict__ next) {
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const int pol = blockIdx.y;
    const int64_t s = from + i + skip;
    next[pol * left_pol_stride + i] = s < n_left ? left[pol * left_pol_stride + s] : pay[pol * pay_pol_stride + (s - n_left)];
}

cudaError_t launch_align_frames(const uint32_t *pay, int64_t pay_pol_stride, const uint32_t *left, int64_t left_pol_stride,
                                int64_t n_left, int64_t skip, int64_t n_pkts, void *frames, int64_t frame_pol_stride,
                                cudaStream_t st) {
    if (n_pkts <= 0) return cudaSuccess;
    const int64_t threads = n_pkts * (kOutWords / 4);
    dim3 grid(static_cast<unsigned>((threads + 255) / 256), 2);
    k_align_frames<<<grid, 256, 0, st>>>(pay, pay_pol_stride, left, left_pol_stride, n_left, skip, n_pkts,
                                         static_cast<uint8_t *>(frames), frame_pol_stride);
    return cudaGetLastError();
}

cudaError_t launch_save_leftover(const uint32_t *pay, int64_t pay_pol_stride, const uint32_t *left,
                                 int64_t left_pol_stride, int64_t n_left, int64_t skip, int64_t from, int64_t count,
                                 uint32_t *next, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>((count + 255) / 256), 2);
    k_save_leftover<<<grid, 256, 0, st>>>(pay, pay_pol_stride, left, left_pol_stride, n_left, skip, from, count, next);
    return cudaGetLastError();
}

cudaError_t launch_vdif_headers(void *frames, int64_t n_pkts, int64_t pol_stride, uint32_t secs0, uint32_t df0,
                                uint64_t psn0, uint32_t ref_epoch, uint32_t station, uint32_t bdc, uint32_t rx,
                                cudaStream_t st) {
    if (n_pkts <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>((n_pkts + 255) / 256), 2);
    k_vdif_headers<<<grid, 256, 0, st>>>(static_cast<uint8_t *>(frames), n_pkts, pol_stride, secs0, df0, psn0,
                                         ref_epoch, station, bdc, rx);
    return cudaGetLastError();
}

}  // namespace sdbe
