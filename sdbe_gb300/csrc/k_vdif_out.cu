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
