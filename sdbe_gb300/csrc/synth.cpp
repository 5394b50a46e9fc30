// Seeded synthetic SWARM B-engine VDIF packets (host code).
//
// Stands in for recorded SDBE scans: per B-frame, snapshot, channel and phased
// sum, a complex Gaussian sample (sigma per component, optional CW tones of
// constant complex amplitude, optional broadband bursts) quantized to 2 bits
// at the fixed levels {-level, 0, +level} as offset-binary codes 0..3.  Codes
// are packed into 1056-B packets exactly as vdif_to_beng reads them
// (software/aphids/vdif_inout_gpu_thread.cu:404-507): per snapshot two u32
// words, bytes 0..3 of the first = channels 3,2,1,0 of the packet and of the
// second = 7,6,5,4; in each byte bits 0-1/2-3 = pol-1 imag/real and
// bits 4-5/6-7 = pol-0 imag/real.  Headers carry b in w4/w5 and (c, f) in w5
// (vdif_in_databuf.h:29-59).  Packets are emitted b-major, then c, then f.
//
// Every B-frame draws from its own generator seeded by (seed, B-counter), so
// output depends neither on the number of threads nor on how a stream is cut
// into calls.
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Xoshiro256 {  // xoshiro256** (Blackman & Vigna)
    uint64_t s[4];
    explicit Xoshiro256(uint64_t seed) {
        for (auto &v : s) v = splitmix64(seed);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    inline double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    inline double gauss() {  // Box-Muller, one value per call
        double u1 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        const double u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

inline double phi(double x) { return 0.5 * std::erfc(-x / std::sqrt(2.0)); }

inline uint32_t quant(double x, double level) {
    return x < -level ? 0u : (x < 0.0 ? 1u : (x < level ? 2u : 3u));
}

}  // namespace

extern "C" {

typedef struct sdbe_synth_cfg {
    double sigma;           // noise sigma per real component
    double level;           // quantizer level (codes split at -level, 0, +level)
    int32_t n_tones;        // up to 8 CW tones
    int32_t tone_channel[8];
    double tone_amp[8];     // complex amplitude magnitude (same units as sigma)
    double tone_phase[8];   // phase of pol 0; pol 1 is offset by 0.7 rad
    double burst_frac;      // fraction of snapshots with sigma * burst_gain
    double burst_gain;
    int32_t channel_map;    // 0: APHIDS 11/11 map, 1: Mar-2015 map
    uint32_t secs0;
    uint32_t ref_epoch;
    uint32_t station;
} sdbe_synth_cfg;

// Writes n_frames*2048 packets (b = b_start .. b_start+n_frames-1) to out.
// Returns the number of packets written, or -1 on a bad argument.
int64_t sdbe_synth_packets(uint8_t *out, int64_t n_frames, uint64_t b_start, uint64_t seed,
                           const sdbe_synth_cfg *cfg, int n_threads) {
    if (!out || !cfg || n_frames < 0 || cfg->n_tones < 0 || cfg->n_tones > 8 || cfg->sigma <= 0.0) return -1;
    const double level = cfg->level;
    // 16-bit uniform thresholds for the plain-noise channels
    auto thresholds = [&](double sig, uint32_t t[3]) {
        const double plo = phi(-level / sig);
        t[0] = static_cast<uint32_t>(std::lround(plo * 65536.0));
        t[1] = 32768u;
        t[2] = static_cast<uint32_t>(std::lround((1.0 - plo) * 65536.0));
    };
    uint32_t t_norm[3], t_burst[3];
    thresholds(cfg->sigma, t_norm);
    thresholds(cfg->sigma * (cfg->burst_gain > 0 ? cfg->burst_gain : 1.0), t_burst);
    std::vector<int> tone_of(16384, -1);
    for (int i = 0; i < cfg->n_tones; ++i)
        if (cfg->tone_channel[i] >= 0 && cfg->tone_channel[i] < 16384) tone_of[cfg->tone_channel[i]] = i;

    auto gen_frame = [&](int64_t fi) {
        const uint64_t b = b_start + static_cast<uint64_t>(fi);
        Xoshiro256 rng(seed * 0x100000001B3ull ^ (b + 1) * 0x9E3779B97F4A7C15ull);
        Xoshiro256 brng(seed ^ 0xB0B5u ^ (b << 20));
        bool burst[128];
        for (int s = 0; s < 128; ++s) burst[s] = cfg->burst_frac > 0.0 && brng.uniform() < cfg->burst_frac;
        uint8_t *frame = out + fi * 2048 * 1056;
        for (uint32_t c = 0; c < 256; ++c) {
            for (uint32_t f = 0; f < 8; ++f) {
                uint8_t *pkt = frame + (c * 8 + f) * 1056;
                uint32_t *w = reinterpret_cast<uint32_t *>(pkt);
                const uint64_t serial = (b * 2048 + c * 8 + f);
                w[0] = cfg->secs0 & 0x3FFFFFFFu;
                w[1] = static_cast<uint32_t>(b % 125000u) | ((cfg->ref_epoch & 0x3Fu) << 24);
                w[2] = 1056u / 8u;
                w[3] = (cfg->station & 0xFFFFu) | (1u << 26) | (1u << 31);
                w[4] = static_cast<uint32_t>(b >> 8);
                w[5] = c | (f << 16) | (static_cast<uint32_t>(b & 0xFFu) << 24);
                w[6] = static_cast<uint32_t>(serial);
                w[7] = static_cast<uint32_t>(serial >> 32);
                const int base = cfg->channel_map == 0 ? static_cast<int>(((c >> 1) * 16 + (c & 1) + 2 * f) * 8)
                                                       : static_cast<int>(8 * (8 * c + f));
                uint8_t *pay = pkt + 32;
                for (int s = 0; s < 128; ++s) {
                    const uint32_t *t = burst[s] ? t_burst : t_norm;
                    const double sig = cfg->sigma * (burst[s] && cfg->burst_gain > 0 ? cfg->burst_gain : 1.0);
                    for (int k = 0; k < 8; ++k) {
                        const int ch = base + k;
                        uint32_t code[4];  // p1 im, p1 re, p0 im, p0 re
                        const int ti = tone_of[ch];
                        if (ti < 0) {
                            const uint64_t r = rng.next();
                            for (int q = 0; q < 4; ++q) {
                                const uint32_t u = static_cast<uint32_t>(r >> (16 * q)) & 0xFFFFu;
                                code[q] = (u >= t[0]) + (u >= t[1]) + (u >= t[2]);
                            }
                        } else {
                            const double a = cfg->tone_amp[ti], ph = cfg->tone_phase[ti];
                            const double re0 = a * std::cos(ph), im0 = a * std::sin(ph);
                            const double re1 = a * std::cos(ph + 0.7), im1 = a * std::sin(ph + 0.7);
                            code[0] = quant(im1 + sig * rng.gauss(), level);
                            code[1] = quant(re1 + sig * rng.gauss(), level);
                            code[2] = quant(im0 + sig * rng.gauss(), level);
                            code[3] = quant(re0 + sig * rng.gauss(), level);
                        }
                        const uint8_t byte =
                            static_cast<uint8_t>(code[0] | (code[1] << 2) | (code[2] << 4) | (code[3] << 6));
                        // channel k lives in word k/4, byte 3 - k%4
                        pay[s * 8 + (k >> 2) * 4 + (3 - (k & 3))] = byte;
                    }
                }
            }
        }
    };
    int nt = n_threads > 0 ? n_threads : static_cast<int>(std::thread::hardware_concurrency());
    nt = std::max(1, std::min<int>(nt, static_cast<int>(std::max<int64_t>(n_frames, 1))));
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t] {
            for (int64_t fi = t; fi < n_frames; fi += nt) gen_frame(fi);
        });
    for (auto &th : pool) th.join();
    return n_frames * 2048;
}

// Drops and displaces packets: each packet is dropped with probability
// drop_frac; each kept packet is, with probability reorder_frac, swapped with
// one up to reorder_max positions later.  Writes the result to out (which
// must not overlap in) and returns the packet count.
int64_t sdbe_synth_impair(const uint8_t *in, int64_t n_pkts, uint8_t *out, uint64_t seed, double drop_frac,
                          double reorder_frac, int32_t reorder_max) {
    if (!in || !out || n_pkts < 0 || reorder_max < 0) return -1;
    Xoshiro256 rng(seed ^ 0xD80Fu);
    std::vector<int64_t> idx;
    idx.reserve(static_cast<size_t>(n_pkts));
    for (int64_t i = 0; i < n_pkts; ++i)
        if (!(rng.uniform() < drop_frac)) idx.push_back(i);
    const int64_t n = static_cast<int64_t>(idx.size());
    if (reorder_max > 0)
        for (int64_t i = 0; i < n; ++i)
            if (rng.uniform() < reorder_frac) {
                const int64_t j = i + 1 + static_cast<int64_t>(rng.next() % static_cast<uint64_t>(reorder_max));
                if (j < n) std::swap(idx[i], idx[j]);
            }
    for (int64_t i = 0; i < n; ++i) std::memcpy(out + i * 1056, in + idx[i] * 1056, 1056);
    return n;
}

}  // extern "C"
