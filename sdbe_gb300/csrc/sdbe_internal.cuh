// Internal definitions shared by the CUDA translation units of libsdbe.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/sdbe.h"

namespace sdbe {

// ---- sizes of the SWARM 11/11 build ------------------------------------
constexpr int kChannels = 16384;                 // BENG_CHANNELS_
constexpr int kGroups = kChannels / 8;           // u32 words per packed spectrum
constexpr int kSnapsPerFrame = 128;              // BENG_SNAPSHOTS
constexpr int kPktsPerFrame = 2048;              // VDIF_PER_BENG
constexpr int kPktBytes = 1056;                  // VDIF_BYTE_SIZE
constexpr int kPktWords = kPktBytes / 4;
constexpr int kPac8Bytes = kPktBytes + 7 * (8 + kPktBytes);  // sizeof(vdif_8pac_packet_t) = 8504
constexpr int kBatchSnaps = 143;                 // RESAMPLE_BATCH_SNAPSHOTS
constexpr int kChunks = 128;                     // FFT_BATCHES_SWARM_R2C
constexpr int kNA = 32768;                       // FFT_SIZE_SWARM_C2R
constexpr int kNB = 36608;                       // FFT_SIZE_SWARM_R2C
constexpr int kNC = 32768;                       // FFT_SIZE_R2DBE_C2R
constexpr int kMA = kNA / 2;                     // 16384-point complex FFT
constexpr int kMB = kNB / 2;                     // 18304-point complex FFT
constexpr int kOutWords = kNC / 16;              // u32 words per output packet
constexpr int kOutPktData = 8192;
constexpr int kOutPkt = 8224;
constexpr int kMaxSkip = kMB - kChannels;        // 1920
constexpr int kDefaultWave = 64;                 // batches per FFT wave when wave_batches = 0 (and the maximum)
constexpr int kTcfBinsLen = kMA + 4;             // fast tensor-core form: R2C bins [skip, skip + 16384] per chunk,
                                                 // padded to a 16-byte multiple

// Packed spectrum nibble: bits 3..2 = real code, bits 1..0 = imag code, value = code - 2.
constexpr uint32_t kMissingWord = 0xAAAAAAAAu;   // codes 2/2 = (0, 0) for all 8 channels

// ---- complex helpers ----------------------------------------------------
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__host__ __device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// ---- twiddle tables (device, built once per handle) -----------------------
struct Twiddles {
    const float2 *w16384;  // exp(-2 pi i k / 16384), k < 16384
    const float2 *w18304;  // exp(-2 pi i k / 18304), k < 18304
    const float2 *w32768;  // exp(-2 pi i k / 32768), k < 16384
    const float2 *w36608;  // exp(-2 pi i k / 36608), k <= 18304
};

// ---- error plumbing -------------------------------------------------------
void set_thread_error(const std::string &msg);
const std::string &thread_error();

}  // namespace sdbe

struct sdbe_resampler;
