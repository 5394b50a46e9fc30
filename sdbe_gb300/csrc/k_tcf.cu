// The fast tensor-core form (SDBE_PRECISION_TC16_FAST): each transform runs
// as a chain of small DFT GEMMs on the 5th-generation tensor cores, with the
// twiddle multiplications between them on the CUDA cores.
//
// A 16384-point transform (stage A's C2R 32768; stage C) is radices 32 x 32 x
// 16 in decimation in time: with k = 512 n1 + 16 n2 + n3 and
// m = k1 + 32 k2 + 1024 k3,
//   stage 1  rows n' = 16 n2 + n3 (512), DFT-32 over n1, twiddle W_16384^(n' k1)
//   stage 2  rows (k1, n3)       (512), DFT-32 over n2, twiddle W_512^(n3 k2)
//   stage 3  rows (k1, k2)      (1024), DFT-16 over n3, output z[m].
// Every stage is D[row][col] = sum_k X[row][k] G[col][k]: X holds the data as
// FP16 (re, im) pairs along K (the A operand, 128 rows per MMA), G the real
// form of the complex DFT matrix split into FP16 hi and lo halves stacked along
// N ([hi | lo], so the data is read from shared memory once per K-step), and
// D accumulates in FP32 in tensor memory.  The epilogue adds the hi and lo
// halves, applies the twiddles in FP32 and rounds the result to FP16 into the
// next stage's operand (a transposition: each thread's row scatters into the
// next stage's rows).  Operands use the 128-byte (K = 64) and 64-byte (K = 32)
// swizzles, and the row orders of the three stages are chosen so that every
// scatter is one shared-memory wavefront per warp.
//
// One CTA per SM: warp 0 issues the MMAs (one thread), warps 1-16 are four
// epilogue groups of four warps (one per tensor-memory lane quarter); group g
// drains accumulator slot g (128 columns), tiles taking the slots in turn.
// Two operand buffers alternate, so a transform's next stage is written while
// the tensor cores still run the current one, and the next transform's input
// is written while the last stage of the current one runs.  Every mbarrier
// wait is bounded: on time-out the kernel records the failure in `status`,
// stops waiting and completes.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "fft_core.cuh"
#include "handle.cuh"
#include "tcgen05.cuh"

namespace sdbe {
namespace {

using namespace tc5;

constexpr int kEpiWarps = 16;
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kThreadsA = 32 + kEpiThreads;
constexpr uint32_t kTmemCols = 512;

// ---- stage A: shared-memory map (bytes from a 1024-byte aligned base) ------
constexpr uint32_t kOpBytes = 65536;                     // one operand buffer (16384 complex FP16)
constexpr uint32_t kG32Bytes = 128 * 64 * 2;             // DFT-32, [hi | lo] x K 64
constexpr uint32_t kG16Bytes = 64 * 32 * 2;              // DFT-16, [hi | lo] x K 32
constexpr uint32_t kOffX0 = 0, kOffX1 = kOpBytes;
constexpr uint32_t kOffG32 = 2 * kOpBytes;
constexpr uint32_t kOffG16 = kOffG32 + kG32Bytes;
constexpr uint32_t kOffStg = kOffG16 + kG16Bytes;        // packed spectrum of one snapshot (8 KB)
constexpr uint32_t kOffTab = kOffStg + 8192;
// float2 tables: e^{2 pi i n1/64} (n1 <= 16, 32 slots), e^{2 pi i n'/32768} (512),
// e^{2 pi i n'/16384} (512), e^{2 pi i n3/512} (16)
constexpr int kTabA1 = 0, kTabA2 = 32, kTabB = kTabA2 + 512, kTabC = kTabB + 512, kTabLen = kTabC + 16;
constexpr uint32_t kSmemA = kOffTab + kTabLen * 8 + 1024;  // + alignment slack

struct SegTA {
    const uint32_t *spec;     // packed spectra of the stream pair
    void *out;                // time series [pol][snapshot][32768], float or half
    int64_t spec_pol_stride;  // words
    int64_t snap0, n_snaps;   // first snapshot, snapshots per pol
    int64_t out_pol_stride;   // elements
    int64_t item0;
};
struct ArgsTA {
    int64_t n_items;
    int n;
    SegTA s[kMaxSegs];
    const uint8_t *g;         // DFT-32 then DFT-16 matrices (inverse), pre-tiled
    const float2 *tab;        // the kTabLen twiddle values
    int *status;              // set to 1 on a barrier time-out (host-mapped)
};

__device__ __forceinline__ const SegTA &seg_of(const ArgsTA &a, int64_t item) {
    int j = 0;
    while (j + 1 < a.n && item >= a.s[j + 1].item0) ++j;
    return a.s[j];
}

__device__ __forceinline__ void named_sync_epi() { asm volatile("bar.sync 1, %0;" ::"r"(kEpiThreads) : "memory"); }

// Staged packed spectrum: word w at w ^ ((w >> 6) & 1) ^ (((w >> 7) & 1) << 4),
// so that the input stage's 32 lanes (8 values of n2 % 8 x 4 of n1 % 4) read
// 32 distinct banks.
__device__ __forceinline__ uint32_t stg_pos(uint32_t w) { return w ^ ((w >> 6) & 1u) ^ (((w >> 7) & 1u) << 4); }

__device__ __forceinline__ float2 stg_value(const uint32_t *stg, int k) {
    const uint32_t w = stg[stg_pos(static_cast<uint32_t>(k) >> 3)] >> ((k & 7) * 4);
    const float re = __uint_as_float(0x4B400000u | ((w >> 2) & 3u)) - 12582914.0f;
    const float im = __uint_as_float(0x4B400000u | (w & 3u)) - 12582914.0f;
    return make_float2(re, im);
}

// Packed spectrum of an item (segment, pol, snapshot; items are pol-major
// within a segment and a segment holds at most two pols).
__device__ __forceinline__ const uint32_t *item_spec(const ArgsTA &a, int64_t item) {
    const SegTA &s = seg_of(a, item);
    const int64_t local = item - s.item0;
    const int64_t pol = local >= s.n_snaps ? 1 : 0, loc = local - pol * s.n_snaps;
    return s.spec + pol * s.spec_pol_stride + (s.snap0 + loc) * kGroups;
}

template <bool OUT_HALF>
__global__ void __launch_bounds__(kThreadsA, 1) k_tcf_a(const __grid_constant__ ArgsTA a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *sm = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    auto X = [sm](int buf) { return sm + (buf ? kOffX1 : kOffX0); };  // operand buffers
    uint32_t *stg = reinterpret_cast<uint32_t *>(sm + kOffStg);
    float2 *tab = reinterpret_cast<float2 *>(sm + kOffTab);
    __shared__ __align__(8) uint64_t full[4], empty[4], ready[2], done;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int s_err;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        for (int i = 0; i < 4; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 4);
        }
        mbar_init(&ready[0], kEpiWarps);
        mbar_init(&ready[1], kEpiWarps);
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_err = 0;
    }
    // DFT matrices and twiddle tables into shared memory
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.g);
        uint4 *dst = reinterpret_cast<uint4 *>(sm + kOffG32);
        for (int i = tid; i < static_cast<int>((kG32Bytes + kG16Bytes) / 16); i += kThreadsA) dst[i] = __ldg(src + i);
        for (int i = tid; i < kTabLen; i += kThreadsA) tab[i] = __ldg(a.tab + i);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tb = tmem_base;

    if (warp == 0) {
        // ---- MMA issuer ------------------------------------------------------
        if (lane == 0) {
            uint32_t T = 0, uses[2] = {0, 0};
            const uint32_t g32 = smem_u32(sm + kOffG32), g16 = smem_u32(sm + kOffG16);
            auto stage = [&](int buf, int tiles, uint32_t tile_bytes, int ksteps, uint32_t sbo, uint32_t layout,
                             uint32_t g, uint32_t g_sbo, int n) {
                if (!s_err && !mbar_wait(&ready[buf], uses[buf] & 1u)) s_err = 1;
                ++uses[buf];
                fence_after();
                const uint32_t xa = smem_u32(X(buf));
                const uint32_t id = idesc_f16(128, n);
                for (int j = 0; j < tiles; ++j, ++T) {
                    const uint32_t slot = T & 3u;
                    if (T >= 4 && !s_err && !mbar_wait(&empty[slot], ((T >> 2) - 1) & 1u)) s_err = 1;
                    fence_after();
                    if (!s_err) {
                        const uint32_t d = tb + slot * 128;
                        for (int ks = 0; ks < ksteps; ++ks)
                            mma_f16(d, desc(xa + j * tile_bytes + ks * 32, 16, sbo, layout),
                                    desc(g + ks * 256, 128, g_sbo, kNoSwizzle), id, ks > 0);
                    }
                    commit(&full[slot]);
                }
            };
            int p = 0;
            for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x, p ^= 1) {
                stage(p, 4, 16384, 4, 1024, kSwizzle128, g32, 1024, 128);      // DFT-32 over n1
                stage(p ^ 1, 4, 16384, 4, 1024, kSwizzle128, g32, 1024, 128);  // DFT-32 over n2
                stage(p, 8, 8192, 2, 512, kSwizzle64, g16, 512, 64);           // DFT-16 over n3
            }
            commit(&done);  // every MMA retired before tensor memory is freed
            if (!mbar_wait(&done, 0)) s_err = 1;
        }
        __syncwarp();
    } else {
        // ---- epilogue warps -------------------------------------------------------
        const int e = warp - 1, grp = e >> 2, q = warp & 3;
        const int et = e * 32 + lane;  // 0 .. 511
        const uint32_t tl = tb + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(grp) * 128;
        uint32_t T = 0;
        auto wait_tile = [&](uint32_t t) {
            if (!s_err && !mbar_wait(&full[t & 3u], (t >> 2) & 1u)) s_err = 1;
            fence_after();
        };
        auto release_tile = [&](uint32_t t) {
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[t & 3u]);
        };
        auto publish = [&](int buf) {  // this warp's part of an operand is written
            fence_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&ready[buf]);
        };
        // next snapshot's packed spectrum, 16 bytes per thread, held in registers
        uint4 pre = make_uint4(0, 0, 0, 0);
        auto prefetch = [&](int64_t item) {
            if (item < a.n_items) pre = __ldg(reinterpret_cast<const uint4 *>(item_spec(a, item)) + et);
        };
        auto stage_spectrum = [&]() {  // registers -> swizzled staging buffer
            const uint32_t w = 4u * static_cast<uint32_t>(et);
            const uint32_t u0 = (w >> 6) & 1u, u1 = (w >> 7) & 1u;
            uint4 v = pre;
            if (u0) v = make_uint4(pre.y, pre.x, pre.w, pre.z);
            *reinterpret_cast<uint4 *>(stg + (w ^ (u1 << 4))) = v;
        };
        // C2R pairing into the stage-1 operand: Z[k] and Z[16384 - k] for
        // k = 512 n1 + 16 n2 + n3, n3 = this warp, (n2 % 8, n1 % 4) = this lane
        auto input = [&](int buf) {
            uint8_t *op = X(buf);
            const int n3 = e;
#pragma unroll 1
            for (int it = 0; it < 16; ++it) {
                const int n1 = 4 * (it >> 2) + (lane >> 3), n2 = 8 * (it & 3) + (lane & 7);
                const int np = 16 * n2 + n3, k = 512 * n1 + np;
                float2 y = stg_value(stg, k);
                float2 ym = make_float2(0.f, 0.f);
                const int km = kMA - k;
                if (k == 0)
                    y.y = 0.f;  // the DC bin's imaginary part is ignored; X[16384] is zero
                else
                    ym = stg_value(stg, km);
                float2 zk, zm;
                c2r_pair(y, ym, cmul(tab[kTabA1 + n1], tab[kTabA2 + np]), zk, zm);
                *reinterpret_cast<uint32_t *>(op + sw128_off(32 * n3 + n2, n1)) = pack_half2(zk.x, zk.y);
                if (k != 0) {
                    const int n1m = km >> 9, npm = km & 511;
                    *reinterpret_cast<uint32_t *>(op + sw128_off(32 * (npm & 15) + (npm >> 4), n1m)) =
                        pack_half2(zm.x, zm.y);
                }
            }
            if (et == 0) {  // k = 8192, its own mirror
                const float2 y = stg_value(stg, kMA / 2);
                float2 zk, zm;
                c2r_pair(y, y, cmul(tab[kTabA1 + 16], tab[kTabA2]), zk, zm);
                *reinterpret_cast<uint32_t *>(op + sw128_off(0, 16)) = pack_half2(zk.x, zk.y);
            }
        };
        // Stage 1 -> stage-2 operand.  Row n' = 16 lane + n3 (n3 = 4 j + q),
        // column k1; stage-2 row 16 k1 + n3, K index n2 = lane.
        auto epi1 = [&](int j, uint8_t *dst) {
            const int n3 = 4 * j + q, np = 16 * lane + n3;
            const float2 b = tab[kTabB + np];
            float2 w = make_float2(1.f, 0.f);
#pragma unroll
            for (int h = 0; h < 4; ++h) {  // k1 in [8h, 8h + 8)
                uint32_t hi[16], lo[16];
                tmem_ld16(tl + 16 * h, hi);
                tmem_ld16(tl + 64 + 16 * h, lo);
                tmem_wait<16>(hi, lo);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int k1 = 8 * h + i;
                    const float2 v = make_float2(__uint_as_float(hi[2 * i]) + __uint_as_float(lo[2 * i]),
                                                 __uint_as_float(hi[2 * i + 1]) + __uint_as_float(lo[2 * i + 1]));
                    const float2 y = cmul(v, w);
                    w = cmul(w, b);
                    *reinterpret_cast<uint32_t *>(dst + sw128_off(16 * k1 + n3, lane)) = pack_half2(y.x, y.y);
                }
            }
        };
        // Stage 2 -> stage-3 operand.  Row 16 k1 + n3 = 128 j + 32 q + lane,
        // column k2; stage-3 row 32 k2 + k1, K index n3.
        auto epi2 = [&](int j, uint8_t *dst) {
            const int r = 128 * j + 32 * q + lane, k1 = r >> 4, n3 = r & 15;
            const float2 b = tab[kTabC + n3];
            float2 w = make_float2(1.f, 0.f);
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                uint32_t hi[16], lo[16];
                tmem_ld16(tl + 16 * h, hi);
                tmem_ld16(tl + 64 + 16 * h, lo);
                tmem_wait<16>(hi, lo);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int k2 = 8 * h + i;
                    const float2 v = make_float2(__uint_as_float(hi[2 * i]) + __uint_as_float(lo[2 * i]),
                                                 __uint_as_float(hi[2 * i + 1]) + __uint_as_float(lo[2 * i + 1]));
                    const float2 y = cmul(v, w);
                    w = cmul(w, b);
                    *reinterpret_cast<uint32_t *>(dst + sw64_off(32 * k2 + k1, n3)) = pack_half2(y.x, y.y);
                }
            }
        };
        // Stage 3 -> output.  Row 32 k2 + k1 = 128 j + 32 q + lane, column k3:
        // z[k1 + 32 k2 + 1024 k3] = (x[2m], x[2m+1]); a warp stores 32
        // consecutive m.
        auto epi3 = [&](int j, void *out) {
            const int r = 128 * j + 32 * q + lane;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                uint32_t hi[16], lo[16];
                tmem_ld16(tl + 16 * h, hi);
                tmem_ld16(tl + 32 + 16 * h, lo);
                tmem_wait<16>(hi, lo);
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const int m = r + 1024 * (8 * h + i);
                    const float re = __uint_as_float(hi[2 * i]) + __uint_as_float(lo[2 * i]);
                    const float im = __uint_as_float(hi[2 * i + 1]) + __uint_as_float(lo[2 * i + 1]);
                    if constexpr (OUT_HALF) {
                        // a quarter of the unnormalised value: |x| < 32768 * 2 * sqrt(2) / 4 fits FP16
                        __stcs(reinterpret_cast<unsigned int *>(out) + m, pack_half2(0.25f * re, 0.25f * im));
                    } else {
                        __stcs(reinterpret_cast<float2 *>(out) + m, make_float2(re, im));
                    }
                }
            }
        };
        auto out_ptr = [&](int64_t item) -> void * {
            const SegTA &s = seg_of(a, item);
            const int64_t local = item - s.item0;
            const int64_t pol = local >= s.n_snaps ? 1 : 0, loc = local - pol * s.n_snaps;
            const int64_t off = pol * s.out_pol_stride + loc * static_cast<int64_t>(kNA);
            return OUT_HALF ? static_cast<void *>(static_cast<__half *>(s.out) + off)
                            : static_cast<void *>(static_cast<float *>(s.out) + off);
        };

        int p = 0;
        if (blockIdx.x < a.n_items) {
            prefetch(blockIdx.x);
            stage_spectrum();
            named_sync_epi();
            input(0);
            publish(0);
            prefetch(blockIdx.x + gridDim.x);
        }
        for (int64_t item = blockIdx.x; item < a.n_items; item += gridDim.x, p ^= 1) {
            // stage 1 -> operand p ^ 1
            for (int j = 0; j < 4; ++j, ++T)
                if (static_cast<int>(T & 3u) == grp) {
                    wait_tile(T);
                    epi1(j, X(p ^ 1));
                    release_tile(T);
                }
            publish(p ^ 1);
            // stage 2 -> operand p
            for (int j = 0; j < 4; ++j, ++T)
                if (static_cast<int>(T & 3u) == grp) {
                    wait_tile(T);
                    epi2(j, X(p));
                    release_tile(T);
                }
            publish(p);
            // every stage-2 MMA has retired (each group saw its tiles' commits),
            // so operand p ^ 1 takes the next item's input
            named_sync_epi();
            const int64_t next = item + gridDim.x;
            if (next < a.n_items) {
                stage_spectrum();
                named_sync_epi();
                input(p ^ 1);
                publish(p ^ 1);
                prefetch(next + gridDim.x);
            }
            // stage 3 -> output
            void *out = out_ptr(item);
            for (int j = 0; j < 8; ++j, ++T)
                if (static_cast<int>(T & 3u) == grp) {
                    wait_tile(T);
                    epi3(j, out);
                    release_tile(T);
                }
        }
    }
    fence_before();
    __syncthreads();
    if (tid == 0 && s_err) *reinterpret_cast<volatile int *>(a.status) = 1;
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tb), "r"(kTmemCols));
}

// ---- host side ------------------------------------------------------------

// Real form of the complex DFT matrix of size r (sign +1: inverse), split
// into FP16 hi and lo halves stacked along N ([hi | lo]: 4r rows of K = 2r),
// K-major in core-matrix order (8 rows x 16 bytes; 128 bytes between core
// matrices along K, (K / 8) * 128 between row groups).  Row 2 kk + t of a
// half is output component t (re, im) of bin kk; column 2 nn + u is input
// component u of element nn.
std::vector<__half> dft_matrix_hilo(int r, int sign) {
    const int K = 2 * r, N = 4 * r;
    std::vector<__half> out(static_cast<size_t>(N) * K);
    for (int kk = 0; kk < r; ++kk)
        for (int nn = 0; nn < r; ++nn) {
            const long long e = static_cast<long long>(kk) * nn % r;
            const double ang = sign * 2.0 * 3.14159265358979323846 * static_cast<double>(e) / r;
            const double c = std::cos(ang), s = std::sin(ang);
            const double vals[2][2] = {{c, -s}, {s, c}};  // [t][u]
            for (int t = 0; t < 2; ++t)
                for (int u = 0; u < 2; ++u) {
                    const double v = vals[t][u];
                    const __half hv = __float2half_rn(static_cast<float>(v));
                    const __half lv = __float2half_rn(static_cast<float>(v - static_cast<double>(__half2float(hv))));
                    for (int part = 0; part < 2; ++part) {
                        const int n = part * 2 * r + 2 * kk + t, k = 2 * nn + u;
                        const size_t off = static_cast<size_t>((n >> 3) * (K / 8) * 64 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7));
                        out[off] = part ? lv : hv;
                    }
                }
        }
    return out;
}

std::vector<float2> tables_a() {
    std::vector<float2> t(kTabLen, make_float2(0.f, 0.f));
    auto cis = [](double num, double den) {
        const double ang = 2.0 * 3.14159265358979323846 * num / den;
        return make_float2(static_cast<float>(std::cos(ang)), static_cast<float>(std::sin(ang)));
    };
    for (int i = 0; i <= 16; ++i) t[kTabA1 + i] = cis(i, 64);
    for (int i = 0; i < 512; ++i) t[kTabA2 + i] = cis(i, 32768);
    for (int i = 0; i < 512; ++i) t[kTabB + i] = cis(i, 16384);
    for (int i = 0; i < 16; ++i) t[kTabC + i] = cis(i, 512);
    return t;
}

template <bool OUT_HALF>
cudaError_t launch_tcf_a(const ArgsTA &args, cudaStream_t st) {
    if (args.n_items <= 0) return cudaSuccess;
    int dev = 0, sms = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tcf_a<OUT_HALF>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmemA));
    if (e != cudaSuccess) return e;
    const unsigned grid = static_cast<unsigned>(args.n_items < sms ? args.n_items : sms);
    k_tcf_a<OUT_HALF><<<grid, kThreadsA, kSmemA, st>>>(args);
    return cudaGetLastError();
}

}  // namespace

// Tables of the fast tensor-core kernels and the time-out flag, on first use.
int tcf_prepare(sdbe_resampler *h, cudaStream_t st) {
    if (h->tcf_tabs) return SDBE_OK;
    if (!h->tc_status_host) {
        if (cudaHostAlloc(&h->tc_status_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, SDBE_ERR_NOMEM, "cannot allocate the tensor-core status flag");
        }
        *h->tc_status_host = 0;
        SDBE_CK(h, cudaHostGetDevicePointer(reinterpret_cast<void **>(&h->tc_status), h->tc_status_host, 0));
    }
    const std::vector<__half> g32 = dft_matrix_hilo(32, +1), g16 = dft_matrix_hilo(16, +1);
    const std::vector<float2> ta = tables_a();
    std::vector<uint8_t> blob(kG32Bytes + kG16Bytes + ta.size() * sizeof(float2));
    std::memcpy(blob.data(), g32.data(), kG32Bytes);
    std::memcpy(blob.data() + kG32Bytes, g16.data(), kG16Bytes);
    std::memcpy(blob.data() + kG32Bytes + kG16Bytes, ta.data(), ta.size() * sizeof(float2));
    if (cudaMalloc(&h->tcf_tabs, blob.size()) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDBE_ERR_NOMEM, "cannot allocate the tensor-core tables");
    }
    SDBE_CK(h, cudaMemcpyAsync(h->tcf_tabs, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
    SDBE_CK(h, cudaStreamSynchronize(st));  // blob is freed on return
    return SDBE_OK;
}

// Stage A in the fast tensor-core form over several stream pairs in one
// launch: per segment, snapshots [snap0, snap0 + n_snaps) of n_pols pols of
// the packed spectra -> float time series out + pol * out_pol_stride,
// [n_snaps][32768] per pol.
int tcf_stage_a(sdbe_resampler *h, const TcfASeg *segs, int n_segs, int n_pols, cudaStream_t st) {
    if (n_segs < 1 || n_segs > kMaxSegs) return fail(h, SDBE_ERR_ARG, "bad segment count");
    if (int rc = tcf_prepare(h, st)) return rc;
    ArgsTA A{};
    for (int i = 0; i < n_segs; ++i) {
        const TcfASeg &g = segs[i];
        A.s[A.n++] = SegTA{g.spec, g.out, g.spec_pol_stride, g.snap0, g.n_snaps, g.out_pol_stride, A.n_items};
        A.n_items += n_pols * g.n_snaps;
    }
    A.g = static_cast<const uint8_t *>(h->tcf_tabs);
    A.tab = reinterpret_cast<const float2 *>(static_cast<const uint8_t *>(h->tcf_tabs) + kG32Bytes + kG16Bytes);
    A.status = h->tc_status;
    SDBE_CK(h, launch_tcf_a<false>(A, st));
    return SDBE_OK;
}

}  // namespace sdbe
