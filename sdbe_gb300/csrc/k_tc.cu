// Precision form of the resampling stage on the 5th-generation tensor cores:
// every DFT block is a batched FP16 GEMM with FP32 accumulation in tensor
// memory (tcgen05.mma, operands in shared memory), with both the DFT matrix
// and the data split into hi + lo FP16 halves (a compensated product:
// hi*hi + hi*lo + lo*hi).
//
// A complex transform of length 128*N2 (16384 = 128*128 for the inverse
// transforms of stages A and C, 18304 = 128*143 for the forward transform of
// stage B) runs as the four-step factorisation, with n = N2*n1 + n2 and
// k = k1 + 128*k2:
//   step 1  A[k1][n2] = sum_n1 F128[k1][n1] x[N2 n1 + n2]        GEMM, M=128 K=128 N=N2
//   step 2  B[k1][n2] = A[k1][n2] w^(n2 k1)                      twiddles, FP32
//   step 3  X[k1 + 128 k2] = sum_n2 F_N2[k2][n2] B[k1][n2]        GEMM, M=N2 K=N2 N=128
// Complex products are real GEMMs accumulated into two TMEM accumulators
// (Dr = Fr Br - Fi Bi, Di = Fi Br + Fr Bi; the inverse flips the signs of
// the Fi terms through the instruction descriptor's negate-A bit).  Each
// transform's input and step-1 output are scaled by powers of two (exact)
// so that every FP16 half stays below 2^14.  The Hermitian pairings, the
// statistics and the 2-bit packing stay on the CUDA cores.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "fft_core.cuh"
#include "handle.cuh"

namespace sdbe {
namespace {

constexpr int kTcThreads = 256;
constexpr uint32_t kTmemCols = 512;
constexpr int kTile = 4096;  // one [128 rows][16 k] FP16 operand tile, core-matrix order

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of 8
// rows x 16 bytes stored contiguously; LBO = byte step between core matrices
// along K, SBO = byte step along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((saddr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: F32 accumulator, F16 A and B, both K-major.
__device__ __forceinline__ uint32_t instr_desc(int m, int n, bool neg_a) {
    return (1u << 4) | (neg_a ? (1u << 13) : 0u) | (static_cast<uint32_t>(n >> 3) << 17) |
           (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc ? 1u : 0u));
}

// Eight consecutive TMEM columns of this thread's lane (warp-collective).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// Bounded wait for the commit of phase `phase`; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t phase) {
    uint32_t done = 0;
    for (int it = 0; it < (1 << 22) && !done; ++it)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(phase & 1u));
    return done != 0;
}

// Byte offset of element (row, k) in a K-major operand with `kdim` columns.
__device__ __forceinline__ uint32_t op_off(int row, int k, int kdim) {
    return static_cast<uint32_t>((row >> 3) * (kdim / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// v -> four FP16 components (re hi, re lo, im hi, im lo) at `off`.
__device__ __forceinline__ void split_store(uint8_t *comp0, uint32_t comp_bytes, uint32_t off, float2 v) {
    const __half rh = __float2half_rn(v.x), ih = __float2half_rn(v.y);
    const __half rl = __float2half_rn(v.x - __half2float(rh)), il = __float2half_rn(v.y - __half2float(ih));
    *reinterpret_cast<__half *>(comp0 + off) = rh;
    *reinterpret_cast<__half *>(comp0 + comp_bytes + off) = rl;
    *reinterpret_cast<__half *>(comp0 + 2 * comp_bytes + off) = ih;
    *reinterpret_cast<__half *>(comp0 + 3 * comp_bytes + off) = il;
}

// 2^(14 - e) where maxabs < 2^e: the exact scale that brings |values| below 2^14.
__device__ __forceinline__ float pow2_scale(float maxabs) {
    if (!(maxabs > 0.f)) return 1.f;
    const int e = static_cast<int>((__float_as_uint(maxabs) >> 23) & 0xFFu) - 126;
    int s = 14 - e;
    s = s > 100 ? 100 : (s < -100 ? -100 : s);
    return __uint_as_float(static_cast<uint32_t>(127 + s) << 23);
}

__device__ __forceinline__ float block_max(float v, float *red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float m = 0.f;
    for (int w = 0; w < kTcThreads / 32; ++w) m = fmaxf(m, red[w]);
    return m;
}

struct TcFftArgs {
    const float2 *in;
    int64_t in_stride, in_pol_stride;  // complex elements between items / between pols
    float2 *out;
    int64_t out_stride, out_pol_stride;
    int64_t per_pol, n_items;          // items per pol, items in all
    const uint8_t *f1;                 // DFT-128 tiles [8 K-steps][4 comps][4 KB]
    const uint8_t *f2;                 // DFT-N2 tiles [K-steps][M tiles][4 comps][4 KB]
    const float2 *tw;                  // e^{-2 pi i e / (128 N2)}, e < 128 N2
    int *status;                       // set to 1 on a barrier time-out (host-mapped)
};

// One CTA per SM (its shared memory and all 512 TMEM columns), persistent
// over items.
template <int N2, bool INV>
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_fft(const __grid_constant__ TcFftArgs a) {
    constexpr int NP = (N2 + 15) / 16 * 16;  // step-1 N, step-3 K
    constexpr int MT = (N2 + 127) / 128;     // step-3 M tiles
    constexpr int KS3 = NP / 16;
    constexpr int NFFT = 128 * N2;
    constexpr uint32_t COMP = NP * 128 * 2;  // bytes of one B-operand component
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *bop = smem;                     // [4 comps][COMP]
    uint8_t *aop = smem + 4 * COMP;          // [MT][4 comps][4 KB]
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_base;
    __shared__ float red[kTcThreads / 32];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, half = warp >> 2;

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tb = tmem_base;
    const uint32_t lane_base = tb + (static_cast<uint32_t>(quarter * 32) << 16);
    uint32_t phase = 0;
    bool ok = true;

    // One K-step: this step's A tiles copied in, 12 MMAs per M tile (3 split
    // products x 4 real products), committed to the barrier, waited on.
    auto k_step = [&](const uint8_t *atiles, int mtiles, int n, uint32_t b_kdim, int s, uint32_t dstride) -> bool {
        const uint4 *src = reinterpret_cast<const uint4 *>(atiles);
        uint4 *dst = reinterpret_cast<uint4 *>(aop);
        for (int i = tid; i < mtiles * 4 * kTile / 16; i += kTcThreads) dst[i] = __ldg(src + i);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sbo_b = (b_kdim / 8) * 128;
            for (int t = 0; t < mtiles; ++t) {
                const uint32_t dr = tb + t * dstride, di = dr + dstride / 2;
                for (int sp = 0; sp < 3; ++sp) {
                    const int ah = sp == 2 ? 1 : 0, bh = sp == 1 ? 1 : 0;  // (hi,hi) (hi,lo) (lo,hi)
                    auto ad = [&](int comp) { return smem_desc(smem_u32(aop + (t * 4 + comp) * kTile), 128, 256); };
                    auto bd = [&](int comp) { return smem_desc(smem_u32(bop + comp * COMP) + s * 256, 128, sbo_b); };
                    const bool first = s == 0 && sp == 0;
                    // Dr += Fr Br -/+ Fi Bi ; Di += +/-Fi Br + Fr Bi
                    mma_f16(dr, ad(0 + ah), bd(0 + bh), instr_desc(128, n, false), !first);
                    mma_f16(dr, ad(2 + ah), bd(2 + bh), instr_desc(128, n, !INV), true);
                    mma_f16(di, ad(2 + ah), bd(0 + bh), instr_desc(128, n, INV), !first);
                    mma_f16(di, ad(0 + ah), bd(2 + bh), instr_desc(128, n, false), true);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&mbar)));
        }
        const bool done = mbar_wait(&mbar, phase);
        ++phase;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        return __syncthreads_and(done) != 0;  // one verdict for the whole CTA
    };

    for (int64_t item = blockIdx.x; item < a.n_items && ok; item += gridDim.x) {
        const int64_t pol = item / a.per_pol, loc = item % a.per_pol;
        const float2 *x = a.in + pol * a.in_pol_stride + loc * a.in_stride;
        float2 *y = a.out + pol * a.out_pol_stride + loc * a.out_stride;
        // ---- input: scaled below 2^14, split, B[n2][n1] -------------------------
        float m = 0.f;
        for (int n = tid; n < NFFT; n += kTcThreads) {
            const float2 v = __ldg(x + n);
            m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
        const float s1 = pow2_scale(block_max(m, red));
        for (int n = tid; n < NFFT; n += kTcThreads) {
            const float2 v = __ldg(x + n);
            const int n1 = n / N2, n2 = n - n1 * N2;
            split_store(bop, COMP, op_off(n2, n1, 128), make_float2(v.x * s1, v.y * s1));
        }
        for (int i = tid; i < (NP - N2) * 128; i += kTcThreads)  // padded rows n2 >= N2
            split_store(bop, COMP, op_off(N2 + i / 128, i % 128, 128), make_float2(0.f, 0.f));
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        // ---- step 1: D[k1][n2]; Dr at column 0, Di at 256 ------------------------
        for (int s = 0; s < 8 && ok; ++s) ok = k_step(a.f1 + s * 4 * kTile, 1, NP, 128, s, 512);
        if (!ok) break;
        // ---- step 2: twiddles, scale, split into B[k1][n2] -----------------------
        const int k1 = quarter * 32 + lane;
        constexpr int HALF = NP / 2;
        float m2 = 0.f;
        for (int c0 = half * HALF; c0 < (half + 1) * HALF; c0 += 8) {
            float dr[8], di[8];
            tmem_ld8(lane_base + c0, dr);
            tmem_ld8(lane_base + 256 + c0, di);
#pragma unroll
            for (int j = 0; j < 8; ++j) m2 = fmaxf(m2, fmaxf(fabsf(dr[j]), fabsf(di[j])));
        }
        const float s2 = pow2_scale(block_max(m2, red));
        for (int c0 = half * HALF; c0 < (half + 1) * HALF; c0 += 8) {
            float dr[8], di[8];
            tmem_ld8(lane_base + c0, dr);
            tmem_ld8(lane_base + 256 + c0, di);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int n2 = c0 + j;
                float2 v = make_float2(0.f, 0.f);
                if (n2 < N2) {
                    int e = n2 * k1;
                    if (e >= NFFT) e -= NFFT;
                    float2 w = __ldg(a.tw + e);
                    if (INV) w.y = -w.y;
                    v = cmul(make_float2(dr[j], di[j]), w);
                    v.x *= s2;
                    v.y *= s2;
                }
                split_store(bop, COMP, op_off(k1, n2, NP), v);
            }
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        // ---- step 3: D[k2][k1] per M tile; Dr at 256 t, Di at 256 t + 128 ---------
        for (int s = 0; s < KS3 && ok; ++s) ok = k_step(a.f2 + s * MT * 4 * kTile, MT, 128, NP, s, 256);
        if (!ok) break;
        const float inv = (1.f / s1) * (1.f / s2);  // powers of two: exact
        for (int t = 0; t < MT; ++t) {
            const int k2 = t * 128 + quarter * 32 + lane;
            for (int c0 = half * 64; c0 < half * 64 + 64; c0 += 8) {
                float dr[8], di[8];
                tmem_ld8(lane_base + t * 256 + c0, dr);
                tmem_ld8(lane_base + t * 256 + 128 + c0, di);
                if (k2 < N2) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) y[(c0 + j) + 128 * k2] = make_float2(dr[j] * inv, di[j] * inv);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (!ok) {  // a commit never arrived: record it, give the MMAs one more bounded wait, free TMEM
        if (tid == 0) *reinterpret_cast<volatile int *>(a.status) = 1;
        mbar_wait(&mbar, phase - 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tb), "r"(kTmemCols));
}

// ---- CUDA-core steps around the tensor-core transforms ---------------------

// Stage A pairing: packed snapshot -> Z[k], k < 16384 (as k_swarm_c2r).
__global__ void k_tc_prep_a(const uint32_t *__restrict__ spec, int64_t spec_pol_stride, int64_t snap0, int64_t n_snaps,
                            float2 *__restrict__ z, const float2 *__restrict__ w32768) {
    const int64_t item = blockIdx.x;  // pol * n_snaps + s
    const int64_t pol = item / n_snaps, s = item % n_snaps;
    const uint32_t *sp = spec + pol * spec_pol_stride + (snap0 + s) * kGroups;
    float2 *zo = z + item * kMA;
    for (int k = threadIdx.x; k <= kMA / 2; k += blockDim.x) {
        float2 va = nib_value(sp, k);
        float2 vb = make_float2(0.f, 0.f);
        if (k == 0)
            va.y = 0.f;
        else
            vb = nib_value(sp, kMA - k);
        float2 zk, zmk;
        c2r_pair(va, vb, conjf2(__ldg(w32768 + k)), zk, zmk);
        zo[k] = zk;
        if (k != 0 && k != kMA / 2) zo[kMA - k] = zmk;
    }
}

// R2C bin q of a 36608-sample chunk from its half-length transform Z.
__device__ __forceinline__ float2 r2c_at(const float2 *zb, int q, const float2 *w36608) {
    if (q == 0) return make_float2(zb[0].x + zb[0].y, 0.f);
    if (q == kMB) return make_float2(zb[0].x - zb[0].y, 0.f);
    float2 xq, xmq;
    r2c_pair(zb[q], zb[kMB - q], __ldg(w36608 + q), xq, xmq);
    return xq;
}

// Stage B -> C: the R2C pairing of Z (18304 per chunk) and the C2R pairing of
// the bins [skip, skip + 16384] -> Z' (16384 per chunk), as k_resample does.
__global__ void k_tc_pair_bc(const float2 *__restrict__ zb, float2 *__restrict__ zc, int skip,
                             const float2 *__restrict__ w32768, const float2 *__restrict__ w36608) {
    const int64_t item = blockIdx.x;
    const float2 *zi = zb + item * kMB;
    float2 *zo = zc + item * kMA;
    for (int j = threadIdx.x; j <= kMA / 2; j += blockDim.x) {
        float2 yv = r2c_at(zi, skip + j, w36608), ym = r2c_at(zi, skip + kMA - j, w36608);
        if (j == 0) {
            yv.y = 0.f;
            ym.y = 0.f;
        }
        float2 zk, zmk;
        c2r_pair(yv, ym, conjf2(__ldg(w32768 + j)), zk, zmk);
        zo[j] = zk;
        if (j != 0 && j != kMA / 2) zo[kMA - j] = zmk;
    }
}

// Per-chunk (n, mean, M2) of the first batch's floats in FP64 (as k_resample<1>).
__global__ void k_tc_chunk_stats(const float *__restrict__ y, int64_t y_pol_stride, int n_chunks,
                                 double *__restrict__ partials) {
    __shared__ double red[64];
    const int pol = blockIdx.y, c = blockIdx.x;
    const float *src = y + pol * y_pol_stride + static_cast<int64_t>(c) * kNC;
    double s1 = 0.0, s2 = 0.0;
    for (int i = threadIdx.x; i < kNC; i += blockDim.x) {
        const double v = src[i];
        s1 += v;
        s2 += v * v;
    }
    block_sum2(s1, s2, red);
    if (threadIdx.x == 0) {
        const double n = static_cast<double>(kNC), mean = s1 / n;
        double *pp = partials + (static_cast<int64_t>(pol) * n_chunks + c) * 3;
        pp[0] = n;
        pp[1] = mean;
        pp[2] = s2 - s1 * mean;
    }
}

// Pre-tiled DFT matrices for the tensor cores: tile (K-step s, M tile t,
// component c) holds F[128 t + r][16 s + kk] in core-matrix order, F[m][k] =
// e^{-2 pi i m k / nf} (zero outside nf x nf); components re hi, re lo, im
// hi, im lo.  Layout [s][t][c]: one K-step's tiles are contiguous.
std::vector<__half> dft_tiles(int nf, int mtiles, int ksteps) {
    std::vector<__half> out(static_cast<size_t>(mtiles) * ksteps * 4 * (kTile / 2));
    for (int t = 0; t < mtiles; ++t)
        for (int s = 0; s < ksteps; ++s)
            for (int r = 0; r < 128; ++r)
                for (int kk = 0; kk < 16; ++kk) {
                    const int mrow = 128 * t + r, k = 16 * s + kk;
                    double re = 0.0, im = 0.0;
                    if (mrow < nf && k < nf) {
                        const long long e = static_cast<long long>(mrow) * k % nf;
                        const double ang = -2.0 * 3.14159265358979323846 * static_cast<double>(e) / nf;
                        re = std::cos(ang);
                        im = std::sin(ang);
                    }
                    const float rh = __half2float(__float2half_rn(static_cast<float>(re)));
                    const float ih = __half2float(__float2half_rn(static_cast<float>(im)));
                    const __half vals[4] = {__float2half_rn(static_cast<float>(re)),
                                            __float2half_rn(static_cast<float>(re - rh)),
                                            __float2half_rn(static_cast<float>(im)),
                                            __float2half_rn(static_cast<float>(im - ih))};
                    const size_t off = (r >> 3) * 128 + (kk >> 3) * 64 + (r & 7) * 8 + (kk & 7);  // in halves
                    for (int c = 0; c < 4; ++c)
                        out[((static_cast<size_t>(s) * mtiles + t) * 4 + c) * (kTile / 2) + off] = vals[c];
                }
    return out;
}

template <int N2>
constexpr size_t tc_smem() {
    return 4 * static_cast<size_t>((N2 + 15) / 16 * 16) * 128 * 2 + static_cast<size_t>((N2 + 127) / 128) * 4 * kTile;
}

template <int N2, bool INV>
cudaError_t launch_tc_fft(const TcFftArgs &args, cudaStream_t st) {
    if (args.n_items <= 0) return cudaSuccess;
    int dev = 0, sms = 1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)  // cheap; set each time so that every device gets it
        e = cudaFuncSetAttribute(k_tc_fft<N2, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(tc_smem<N2>()));
    if (e != cudaSuccess) return e;
    const unsigned grid = static_cast<unsigned>(args.n_items < sms ? args.n_items : sms);
    k_tc_fft<N2, INV><<<grid, kTcThreads, tc_smem<N2>(), st>>>(args);
    return cudaGetLastError();
}

}  // namespace

// Tables and scratch of the tensor-core path, on first use.
int tc_prepare(sdbe_resampler *h, cudaStream_t st) {
    if (h->tc_f128) return SDBE_OK;
    const std::vector<__half> f128 = dft_tiles(128, 1, 8), f143 = dft_tiles(143, 2, 9);
    const size_t wave_snaps = static_cast<size_t>(h->wave) * kBatchSnaps;
    const size_t wave_chunks = static_cast<size_t>(h->wave) * kChunks;
    if (cudaMalloc(&h->tc_f128, f128.size() * sizeof(__half)) != cudaSuccess ||
        cudaMalloc(&h->tc_f143, f143.size() * sizeof(__half)) != cudaSuccess ||
        cudaMalloc(&h->tc_bufx, 2 * wave_snaps * kMA * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&h->tc_bufy, 2 * wave_chunks * kMB * sizeof(float2)) != cudaSuccess ||
        cudaHostAlloc(&h->tc_status_host, sizeof(int), cudaHostAllocMapped) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SDBE_ERR_NOMEM, "cannot allocate the tensor-core scratch");
    }
    SDBE_CK(h, cudaMemcpyAsync(h->tc_f128, f128.data(), f128.size() * sizeof(__half), cudaMemcpyHostToDevice, st));
    SDBE_CK(h, cudaMemcpyAsync(h->tc_f143, f143.data(), f143.size() * sizeof(__half), cudaMemcpyHostToDevice, st));
    *h->tc_status_host = 0;
    SDBE_CK(h, cudaHostGetDevicePointer(reinterpret_cast<void **>(&h->tc_status), h->tc_status_host, 0));
    SDBE_CK(h, cudaStreamSynchronize(st));  // the host tables are freed on return
    return SDBE_OK;
}

// The FFT chain of sdbe_process in the tensor-core form: per wave, stage A
// (pairing, TC inverse 16384), stage B (TC forward 18304), the pairings, stage
// C (TC inverse 16384) and the 2-bit packing; the first batch of a stream sets
// the thresholds from its FP64 statistics as the FP32 path does.
int tc_chain(sdbe_resampler *h, const uint32_t *spec, int64_t spec_pol_stride, int64_t n_batches,
             const PayloadTarget &tgt, cudaStream_t st) {
    if (n_batches <= 0) return SDBE_OK;
    if (int rc = tc_prepare(h, st)) return rc;
    if (*reinterpret_cast<volatile int *>(h->tc_status_host))  // written by an earlier call's kernels
        return fail(h, SDBE_ERR_CUDA, "a tensor-core transform timed out on its mbarrier wait");
    const Twiddles &tw = h->tw;
    const uint8_t *f128 = static_cast<const uint8_t *>(h->tc_f128);
    const uint8_t *f143 = static_cast<const uint8_t *>(h->tc_f143);
    for (int64_t b = 0; b < n_batches;) {
        const bool first = !h->thresholds_set;
        const int64_t nb = first ? 1 : (n_batches - b < h->wave ? n_batches - b : h->wave);
        const int64_t snaps = nb * kBatchSnaps, chunks = nb * kChunks;
        size_t slot = 0;
        if (!first) SDBE_CK(h, timed_begin(h, 0, 2 * snaps, st, &slot));
        // stage A: Z (bufx) -> time series (ts: complex 16384 per snapshot)
        k_tc_prep_a<<<static_cast<unsigned>(2 * snaps), 256, 0, st>>>(spec, spec_pol_stride, b * kBatchSnaps, snaps,
                                                                      h->tc_bufx, tw.w32768);
        SDBE_CK(h, cudaGetLastError());
        float2 *ts = reinterpret_cast<float2 *>(h->ts);
        const TcFftArgs A{h->tc_bufx, kMA, snaps * kMA, ts, kMA, h->ts_pol_stride / 2,
                          snaps, 2 * snaps, f128, f128, tw.w16384, h->tc_status};
        SDBE_CK(h, (launch_tc_fft<128, true>(A, st)));
        if (!first) {
            SDBE_CK(h, timed_end(h, slot, st));
            SDBE_CK(h, timed_begin(h, 1, 2 * chunks, st, &slot));
        }
        // stage B: chunks of 18304 complex -> Z (bufy)
        const TcFftArgs B{ts, kMB, h->ts_pol_stride / 2, h->tc_bufy, kMB, chunks * kMB,
                          chunks, 2 * chunks, f128, f143, tw.w18304, h->tc_status};
        SDBE_CK(h, (launch_tc_fft<143, false>(B, st)));
        // pairings: bufy -> Z' (bufx)
        k_tc_pair_bc<<<static_cast<unsigned>(2 * chunks), 256, 0, st>>>(h->tc_bufy, h->tc_bufx, h->skip, tw.w32768,
                                                                        tw.w36608);
        SDBE_CK(h, cudaGetLastError());
        // stage C: Z' -> floats (bufy, 32768 per chunk)
        const TcFftArgs C{h->tc_bufx, kMA, chunks * kMA, h->tc_bufy, kMA, chunks * kMA,
                          chunks, 2 * chunks, f128, f128, tw.w16384, h->tc_status};
        SDBE_CK(h, (launch_tc_fft<128, true>(C, st)));
        const float *yf = reinterpret_cast<const float *>(h->tc_bufy);
        if (first) {
            k_tc_chunk_stats<<<dim3(kChunks, 2), 256, 0, st>>>(yf, chunks * kNC, kChunks, h->partials);
            SDBE_CK(h, cudaGetLastError());
            SDBE_CK(h, launch_finalize_thresholds(h->partials, kChunks, h->cfg.pol1_uses_pol0_threshold, h->thr, st));
            h->thresholds_set = true;
        }
        SDBE_CK(h, launch_quantize_chunks(yf, chunks * kNC, chunks, h->thr, tgt.base, tgt.pol_stride, tgt.pkt_stride,
                                          tgt.payload_off, b * kChunks, st));
        if (!first) SDBE_CK(h, timed_end(h, slot, st));
        h->stream_batch = (first ? 0 : h->stream_batch) + nb;
        h->launches += first ? 8 : 6;
        b += nb;
    }
    return SDBE_OK;
}

// Stage entry points in the tensor-core form (sdbe_swarm_c2r and
// sdbe_resample_chunks on a SDBE_PRECISION_TC16 handle), one pol, in pieces
// that fit the handle's scratch.
int tc_swarm_c2r(sdbe_resampler *h, const uint32_t *spec, int64_t n_snaps, float *out, cudaStream_t st) {
    if (n_snaps <= 0) return SDBE_OK;
    if (int rc = tc_prepare(h, st)) return rc;
    const uint8_t *f128 = static_cast<const uint8_t *>(h->tc_f128);
    const int64_t cap = 2 * static_cast<int64_t>(h->wave) * kBatchSnaps;
    for (int64_t s0 = 0; s0 < n_snaps; s0 += cap) {
        const int64_t n = n_snaps - s0 < cap ? n_snaps - s0 : cap;
        k_tc_prep_a<<<static_cast<unsigned>(n), 256, 0, st>>>(spec, 0, s0, n, h->tc_bufx, h->tw.w32768);
        SDBE_CK(h, cudaGetLastError());
        const TcFftArgs A{h->tc_bufx, kMA, 0, reinterpret_cast<float2 *>(out + s0 * kNA), kMA, 0,
                          n, n, f128, f128, h->tw.w16384, h->tc_status};
        SDBE_CK(h, (launch_tc_fft<128, true>(A, st)));
    }
    return SDBE_OK;
}

int tc_resample_chunks(sdbe_resampler *h, const float *in, int64_t n_chunks, float *out, cudaStream_t st) {
    if (n_chunks <= 0) return SDBE_OK;
    if (int rc = tc_prepare(h, st)) return rc;
    const uint8_t *f128 = static_cast<const uint8_t *>(h->tc_f128);
    const uint8_t *f143 = static_cast<const uint8_t *>(h->tc_f143);
    const int64_t cap = 2 * static_cast<int64_t>(h->wave) * kChunks;
    for (int64_t c0 = 0; c0 < n_chunks; c0 += cap) {
        const int64_t n = n_chunks - c0 < cap ? n_chunks - c0 : cap;
        const TcFftArgs B{reinterpret_cast<const float2 *>(in + c0 * kNB), kMB, 0, h->tc_bufy, kMB, 0,
                          n, n, f128, f143, h->tw.w18304, h->tc_status};
        SDBE_CK(h, (launch_tc_fft<143, false>(B, st)));
        k_tc_pair_bc<<<static_cast<unsigned>(n), 256, 0, st>>>(h->tc_bufy, h->tc_bufx, h->skip, h->tw.w32768,
                                                               h->tw.w36608);
        SDBE_CK(h, cudaGetLastError());
        const TcFftArgs C{h->tc_bufx, kMA, 0, reinterpret_cast<float2 *>(out + c0 * kNC), kMA, 0,
                          n, n, f128, f128, h->tw.w16384, h->tc_status};
        SDBE_CK(h, (launch_tc_fft<128, true>(C, st)));
    }
    return SDBE_OK;
}

}  // namespace sdbe
